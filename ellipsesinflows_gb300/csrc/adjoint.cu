// Discrete adjoint of the time step, double-precision form, with the particles
// frozen (their positions and velocities are parameters of the step: no inertia,
// collision, increment or update; the immersed-boundary forcing acts with the
// frozen rigid-body velocities). The step map differentiated is
//
//   for each RK stage k (src/main.c:14-31 without the particle part):
//     A_k  = A(u_k, v_k)                         advection + diffusion (+ forcing)
//     u*   = u_k + dt (a_k A_k + b_k A_{k-1} + g_k G p_k)      update_velocity.c
//     u**  = u* + Avg W (U - I u*)               exchange.c:61-72, update.c:36-59
//     psi  = L^-1 D u** / (g_k dt)               compute_potential.c:48-138
//     u_{k+1} = u** - g_k dt G psi,  p_{k+1} = p_k + psi      correct_velocity.c, update_pressure.c
//
// with dt held fixed (recorded per step): the adjoint is the transpose of the
// linearisation of this map around the recorded stage states, applied backwards:
//
//   projection:  phi = L^-1 (D ubar' + pbar' / (g dt)),  ubar** = ubar' - G phi
//                (on the uniform staggered grid G^T = -D and L = D G is symmetric,
//                so the double-precision Poisson solver of the forward step is reused)
//   forcing:     ubar* = ubar** - I^T W Avg^T ubar**     (W: summed weights per cell)
//   predictor:   ubar_k = ubar* + (dA/du)^T (dt a_k ubar* + Abar_k),
//                pbar += dt g_k G^T ubar*,  Abar_{k-1} = dt b_k ubar*
//
// The transposed stencils are gathers (each input cell sums the contributions of
// the outputs that read it), so the result does not depend on thread order.
#include "eif_internal.cuh"
#include <algorithm>
#include <vector>

namespace eif {

struct Adjoint {
  int max_steps = 0, nrec = 0;
  // recorded stage inputs u_k, v_k (3 per step) and dt per step
  std::vector<double *> tape_u, tape_v;
  std::vector<double> tape_dt;
  // cotangents (double, field layout): velocity, pressure, explicit terms, scratch
  double *ub = nullptr, *vb = nullptr, *pb = nullptr, *abx = nullptr, *aby = nullptr;
  double *tu = nullptr, *tv = nullptr, *rhs = nullptr, *w = nullptr;
};

}  // namespace eif

namespace {

using eifd::ux_idx;
using eifd::uy_idx;
constexpr int AX = 32, AY = 8;

struct AdjGeom {
  const double *rdxf, *rdxc, *cxm, *cxp, *cym, *cyp;
  double rRe, rdy;
  int itot, jtot, ld;
};

__device__ __forceinline__ int wrapj(int j, int jtot) { return j < 1 ? j + jtot : (j > jtot ? j - jtot : j); }

// partial derivatives of the explicit term A_x at face (I, J) (update_velocity.c:30-103)
struct DAx {
  double du0, duw, due, dus, dun, dvsw, dvse, dvnw, dvne;
};
__device__ __forceinline__ DAx dax(const double *u, const double *v, const AdjGeom &g, int I, int J) {
  const int ld = g.ld;
  const int c = ux_idx(I, J, ld), cy = uy_idx(I, J, ld);
  const double u0 = u[c], uw = u[c - 1], ue = u[c + 1], us = u[c - ld], un = u[c + ld];
  const double cxm = g.cxm[I], cxp = g.cxp[I], rdm = g.rdxf[I - 1], rdp = g.rdxf[I], rdc = g.rdxc[I];
  const double vS = cxm * v[cy - 1] + cxp * v[cy], vN = cxm * v[cy - 1 + ld] + cxp * v[cy + ld];
  const double rdy = g.rdy, rRe = g.rRe;
  DAx d;
  d.duw = cxm * rdm * uw + rRe * rdm * rdc;
  d.due = -cxp * rdp * ue + rRe * rdp * rdc;
  d.du0 = -cxm * rdm * u0 + cxp * rdp * u0 - 0.5 * rdy * (vS - vN) + rRe * (-(rdp + rdm) * rdc - 2. * rdy * rdy);
  d.dus = 0.5 * vS * rdy + rRe * rdy * rdy;
  d.dun = -0.5 * vN * rdy + rRe * rdy * rdy;
  d.dvsw = -0.5 * cxm * (u0 - us) * rdy;
  d.dvse = -0.5 * cxp * (u0 - us) * rdy;
  d.dvnw = -0.5 * cxm * (un - u0) * rdy;
  d.dvne = -0.5 * cxp * (un - u0) * rdy;
  return d;
}

// partial derivatives of A_y at cell (I, J) (update_velocity.c:105-173)
struct DAy {
  double dv0, dvw, dve, dvs, dvn, dum, dup;   // dum: u(I, J-1) and u(I, J); dup: u(I+1, J-1) and u(I+1, J)
};
__device__ __forceinline__ DAy day(const double *u, const double *v, const AdjGeom &g, int I, int J) {
  const int ld = g.ld;
  const int c = uy_idx(I, J, ld), cx = ux_idx(I, J, ld);
  const double v0 = v[c], vw = v[c - 1], ve = v[c + 1], vs = v[c - ld], vn = v[c + ld];
  const double rcm = g.rdxc[I], rcp = g.rdxc[I + 1], rf = g.rdxf[I];
  const double cym = g.cym[I], cyp = g.cyp[I];
  const double uxm = 0.5 * u[cx - ld] + 0.5 * u[cx], uxp = 0.5 * u[cx + 1 - ld] + 0.5 * u[cx + 1];
  const double rdy = g.rdy, rRe = g.rRe;
  DAy d;
  d.dvw = cym * uxm * rcm + rRe * rcm * rf;
  d.dve = -cyp * uxp * rcp + rRe * rcp * rf;
  d.dv0 = -cym * uxm * rcm + cyp * uxp * rcp + rRe * (-(rcp + rcm) * rf - 2. * rdy * rdy);
  d.dvs = 0.5 * rdy * vs + rRe * rdy * rdy;
  d.dvn = -0.5 * rdy * vn + rRe * rdy * rdy;
  d.dum = -0.5 * cym * (v0 - vw) * rcm;
  d.dup = -0.5 * cyp * (ve - v0) * rcp;
  return d;
}

struct AdjPredArgs {
  const double *u, *v;          // state u_k, v_k (with halos)
  const double *sbx, *sby;      // cotangents of u*, v*
  double *abx, *aby;            // in: Abar_k (cotangent of A_k); out: dt b_k ubar* (for stage k-1)
  double *ubo, *vbo;            // out: cotangents of u_k, v_k
  double *pb;                   // in/out: pressure cotangent (+= dt g_k G^T ubar*)
  AdjGeom g;
  double adt, bdt, gdt;
};

// weighted cotangent of A at an output: dt a_k ubar* + Abar_k (zero at the wall faces)
__device__ __forceinline__ double gx_at(const AdjPredArgs &a, int I, int J) {
  if (I < 2 || I > a.g.itot) return 0.;
  const int c = ux_idx(I, J, a.g.ld);
  return a.adt * a.sbx[c] + a.abx[c];
}
__device__ __forceinline__ double gy_at(const AdjPredArgs &a, int I, int J) {
  if (I < 1 || I > a.g.itot) return 0.;
  const int c = uy_idx(I, J, a.g.ld);
  return a.adt * a.sby[c] + a.aby[c];
}

// transposed linearised predictor (gather form); first pass: cotangents of the state
__global__ void __launch_bounds__(AX *AY) k_adj_predictor(AdjPredArgs a) {
  const int i = 1 + blockIdx.x * AX + threadIdx.x;
  const int j = 1 + blockIdx.y * AY + threadIdx.y;
  const AdjGeom &g = a.g;
  if (i > g.itot || j > g.jtot) return;
  const int ld = g.ld, jtot = g.jtot, itot = g.itot;
  const int jm = wrapj(j - 1, jtot), jp = wrapj(j + 1, jtot);
  if (i >= 2) {
    // u(i, j): read by A_x at (i, j) [u0], (i+1, j) [uw], (i-1, j) [ue], (i, j+1) [us],
    // (i, j-1) [un] and by A_y at (i, j) and (i, j+1) [u(I, .)], (i-1, j) and (i-1, j+1) [u(I+1, .)]
    const int c = ux_idx(i, j, ld);
    double s = a.sbx[c];
    s += gx_at(a, i, j) * dax(a.u, a.v, g, i, j).du0;
    if (i + 1 <= itot) s += gx_at(a, i + 1, j) * dax(a.u, a.v, g, i + 1, j).duw;
    if (i - 1 >= 2) s += gx_at(a, i - 1, j) * dax(a.u, a.v, g, i - 1, j).due;
    s += gx_at(a, i, jp) * dax(a.u, a.v, g, i, jp).dus;
    s += gx_at(a, i, jm) * dax(a.u, a.v, g, i, jm).dun;
    s += gy_at(a, i, j) * day(a.u, a.v, g, i, j).dum;
    s += gy_at(a, i, jp) * day(a.u, a.v, g, i, jp).dum;
    s += gy_at(a, i - 1, j) * day(a.u, a.v, g, i - 1, j).dup;
    s += gy_at(a, i - 1, jp) * day(a.u, a.v, g, i - 1, jp).dup;
    a.ubo[c] = s;
  }
  {
    // v(i, j): read by A_y at (i, j) [v0], (i+1, j) [vw], (i-1, j) [ve], (i, j+1) [vs],
    // (i, j-1) [vn] and by A_x at (i+1, j) [v(I-1, J)], (i, j) [v(I, J)],
    // (i+1, j-1) [v(I-1, J+1)], (i, j-1) [v(I, J+1)]
    const int c = uy_idx(i, j, ld);
    double s = a.sby[c];
    s += gy_at(a, i, j) * day(a.u, a.v, g, i, j).dv0;
    if (i + 1 <= itot) s += gy_at(a, i + 1, j) * day(a.u, a.v, g, i + 1, j).dvw;
    if (i - 1 >= 1) s += gy_at(a, i - 1, j) * day(a.u, a.v, g, i - 1, j).dve;
    s += gy_at(a, i, jp) * day(a.u, a.v, g, i, jp).dvs;
    s += gy_at(a, i, jm) * day(a.u, a.v, g, i, jm).dvn;
    if (i + 1 <= itot) {
      s += gx_at(a, i + 1, j) * dax(a.u, a.v, g, i + 1, j).dvsw;
      s += gx_at(a, i + 1, jm) * dax(a.u, a.v, g, i + 1, jm).dvnw;
    }
    if (i >= 2) {
      s += gx_at(a, i, j) * dax(a.u, a.v, g, i, j).dvse;
      s += gx_at(a, i, jm) * dax(a.u, a.v, g, i, jm).dvne;
    }
    a.vbo[c] = s;
    // pressure: u* reads p(i, j) through -(p(i) - p(i-1)) rdxc(i) at faces i and i+1,
    // v* through -(p(j) - p(j-1)) rdy at rows j and j+1
    double gp = 0.;
    if (i >= 2) gp -= a.sbx[ux_idx(i, j, ld)] * g.rdxc[i];
    if (i + 1 <= itot) gp += a.sbx[ux_idx(i + 1, j, ld)] * g.rdxc[i + 1];
    gp -= a.sby[c] * g.rdy;
    gp += a.sby[uy_idx(i, jp, ld)] * g.rdy;
    a.pb[c] += a.gdt * gp;
  }
}

// second pass: cotangent of the previous stage's explicit term (srcB)
__global__ void k_adj_srcb(const double *__restrict__ sbx, const double *__restrict__ sby, double *__restrict__ abx,
                           double *__restrict__ aby, double bdt, int itot, int jtot, int ld) {
  const int i = 1 + blockIdx.x * AX + threadIdx.x;
  const int j = 1 + blockIdx.y * AY + threadIdx.y;
  if (i > itot || j > jtot) return;
  const int c = uy_idx(i, j, ld);
  if (i >= 2) abx[ux_idx(i, j, ld)] = bdt * sbx[ux_idx(i, j, ld)];
  aby[c] = bdt * sby[c];
}

// transposed forcing: ubar* = ubar** - I^T W Avg^T ubar**  (cells 1..itot, faces 2..itot)
__global__ void k_adj_forcing(const double *__restrict__ sx, const double *__restrict__ sy, const double *__restrict__ w,
                              double *__restrict__ ox, double *__restrict__ oy, int itot, int jtot, int ld) {
  const int i = 1 + blockIdx.x * AX + threadIdx.x;
  const int j = 1 + blockIdx.y * AY + threadIdx.y;
  if (i > itot || j > jtot) return;
  const int jm = wrapj(j - 1, jtot), jp = wrapj(j + 1, jtot);
  auto ux_b = [&](int I, int J) { return (I >= 2 && I <= itot) ? sx[ux_idx(I, J, ld)] : 0.; };
  // Avg^T: the face values around cell (I, J) in x: faces I and I+1; in y: rows J and J+1
  auto gcx = [&](int I, int J) { return 0.5 * (ux_b(I, J) + ux_b(I + 1, J)); };
  auto gcy = [&](int I, int J) { return 0.5 * (sy[uy_idx(I, J, ld)] + sy[uy_idx(I, wrapj(J + 1, jtot), ld)]); };
  if (i >= 2) {
    const int c = ux_idx(i, j, ld);
    ox[c] = sx[c] - 0.5 * (w[uy_idx(i - 1, j, ld)] * gcx(i - 1, j) + w[uy_idx(i, j, ld)] * gcx(i, j));
  }
  const int c = uy_idx(i, j, ld);
  oy[c] = sy[c] - 0.5 * (w[uy_idx(i, jm, ld)] * gcy(i, jm) + w[c] * gcy(i, j));
  (void)jp;
}

// right-hand side of the transposed projection: D ubar' + pbar' / (g dt)
__global__ void k_adj_rhs(const double *__restrict__ sx, const double *__restrict__ sy, const double *__restrict__ pb,
                          double *__restrict__ rhs, double rdx, double rdy, double inv, int itot, int jtot, int ld) {
  const int i = 1 + blockIdx.x * AX + threadIdx.x;
  const int j = 1 + blockIdx.y * AY + threadIdx.y;
  if (i > itot || j > jtot) return;
  const double ue = (i + 1 <= itot) ? sx[ux_idx(i + 1, j, ld)] : 0.;
  const double uw = (i >= 2) ? sx[ux_idx(i, j, ld)] : 0.;
  const int c = uy_idx(i, j, ld);
  const double vn = sy[uy_idx(i, wrapj(j + 1, jtot), ld)], vs = sy[c];
  rhs[c] = (ue - uw) * rdx + (vn - vs) * rdy + pb[c] * inv;
}

// ubar** = ubar' - G phi
__global__ void k_adj_grad(const double *__restrict__ phi, const double *__restrict__ rdxc, double *__restrict__ sx,
                           double *__restrict__ sy, double rdy, int itot, int jtot, int ld) {
  const int i = 1 + blockIdx.x * AX + threadIdx.x;
  const int j = 1 + blockIdx.y * AY + threadIdx.y;
  if (i > itot || j > jtot) return;
  const int c = uy_idx(i, j, ld);
  if (i >= 2) sx[ux_idx(i, j, ld)] -= (phi[c] - phi[c - 1]) * rdxc[i];
  sy[c] -= (phi[c] - phi[uy_idx(i, wrapj(j - 1, jtot), ld)]) * rdy;
}

dim3 agrid(const eif_ctx *c) { return dim3((c->itot + AX - 1) / AX, (c->jtot + AY - 1) / AY); }

}  // namespace

using namespace eif;

namespace {

void adj_free(eif_ctx *c) {
  Adjoint *a = c->adj;
  if (!a) return;
  for (double *p : a->tape_u) cudaFree(p);
  for (double *p : a->tape_v) cudaFree(p);
  for (double *p : {a->ub, a->vb, a->pb, a->abx, a->aby, a->tu, a->tv, a->rhs, a->w})
    if (p) cudaFree(p);
  delete a;
  c->adj = nullptr;
}

int adj_check(eif_ctx *c) {
  if (!c) return EIF_ERR_ARG;
  if (!c->adj) return fail(c, EIF_ERR_STATE, "call eif_adjoint_begin first");
  return EIF_OK;
}

}  // namespace

extern "C" {

int eif_adjoint_begin(eif_ctx *c, int max_steps) {
  if (!c || max_steps <= 0) return EIF_ERR_ARG;
  if (c->cfg.precision != EIF_PREC_FP64) return fail(c, EIF_ERR_ARG, "the adjoint is built on the double-precision form");
  if (!c->fluid_pushed) return fail(c, EIF_ERR_STATE, "push the fluid state before eif_adjoint_begin");
  adj_free(c);
  Adjoint *a = new Adjoint;
  c->adj = a;
  a->max_steps = max_steps;
  const size_t bytes = sizeof(double) * c->nfield;
  for (int k = 0; k < 3 * max_steps; k++) {
    double *u = nullptr, *v = nullptr;
    EIF_CK(c, cudaMalloc((void **)&u, bytes));
    a->tape_u.push_back(u);
    EIF_CK(c, cudaMalloc((void **)&v, bytes));
    a->tape_v.push_back(v);
  }
  for (double **p : {&a->ub, &a->vb, &a->pb, &a->abx, &a->aby, &a->tu, &a->tv, &a->rhs, &a->w}) {
    EIF_CK(c, cudaMalloc((void **)p, bytes));
    EIF_CK(c, cudaMemsetAsync(*p, 0, bytes, c->stream));
  }
  // summed indicator weights of the frozen particles: the exchange with the weights
  // as the cell contributions (double-precision kernels) gathers them into dux
  if (c->np > 0) {
    c->ibm_weights_only = true;
    c->boxes_x_valid = false;
    c->weights_x_valid = false;
    const int rc = launch_exchange(c);
    c->ibm_weights_only = false;
    c->weights_x_valid = false;
    if (rc) return rc;
    EIF_CK(c, cudaMemcpyAsync(a->w, c->dux, bytes, cudaMemcpyDeviceToDevice, c->stream));
  }
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return check_records(c);
}

int eif_adjoint_end(eif_ctx *c) {
  if (!c) return EIF_ERR_ARG;
  cudaStreamSynchronize(c->stream);
  adj_free(c);
  return EIF_OK;
}

// one forward step with the particles frozen and the current dt; with record != 0
// the stage inputs are recorded for eif_adjoint_backward. The step counter and time
// advance as in eif_advance.
int eif_adjoint_forward(eif_ctx *c, int record) {
  int rc = adj_check(c);
  if (rc) return rc;
  Adjoint *a = c->adj;
  if (record && a->nrec >= a->max_steps) return fail(c, EIF_ERR_ARG, "the adjoint tape holds %d steps", a->max_steps);
  const size_t bytes = sizeof(double) * c->nfield;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  a->tape_dt.resize(a->max_steps);
  if (record) a->tape_dt[a->nrec] = c->dt_host;
  const bool ibm = c->np > 0;
  for (int rk = 0; rk < 3; rk++) {
    if (record) {
      EIF_CK(c, cudaMemcpyAsync(a->tape_u[3 * a->nrec + rk], c->ux[c->cur], bytes, cudaMemcpyDeviceToDevice,
                                c->stream));
      EIF_CK(c, cudaMemcpyAsync(a->tape_v[3 * a->nrec + rk], c->uy[c->cur], bytes, cudaMemcpyDeviceToDevice,
                                c->stream));
    }
    if ((rc = launch_predictor(c, rk))) return rc;
    if (ibm && (rc = launch_exchange(c))) return rc;
    if ((rc = launch_potential(c, rk, ibm))) return rc;
    if ((rc = launch_correct(c, rk, ibm, true))) return rc;
  }
  if (record) a->nrec++;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  c->step += 1;
  c->time += c->dt_host;
  return check_records(c);
}

// Cotangents of the state after the last recorded step, from host arrays in the
// eif_push_fluid layouts. The halo rows of the state are copies of rows jtot and 1
// and the pressure's wall columns copies of columns 1 and itot, so their cotangents
// are added to those entries; the velocity wall columns are constants (no
// cotangent). The pressure is determined up to a constant, so the mean of its
// cotangent over the cells is removed. p_bar may be NULL for zero.
int eif_adjoint_seed(eif_ctx *c, const double *ux_bar, const double *uy_bar, const double *p_bar) {
  int rc = adj_check(c);
  if (rc) return rc;
  if (!ux_bar || !uy_bar) return EIF_ERR_ARG;
  Adjoint *a = c->adj;
  const int it = c->itot, jt = c->jtot, rows = jt + 2;
  const int wx = it + 1, wy = it + 2;
  std::vector<double> hx(ux_bar, ux_bar + (size_t)wx * rows), hy(uy_bar, uy_bar + (size_t)wy * rows);
  std::vector<double> hp(p_bar ? p_bar : hy.data(), (p_bar ? p_bar : hy.data()) + (size_t)wy * rows);
  if (!p_bar) std::fill(hp.begin(), hp.end(), 0.);
  auto fold_rows = [&](std::vector<double> &h, int w) {
    for (int i = 0; i < w; i++) {
      h[(size_t)jt * w + i] += h[i];
      h[(size_t)1 * w + i] += h[(size_t)(jt + 1) * w + i];
      h[i] = 0.;
      h[(size_t)(jt + 1) * w + i] = 0.;
    }
  };
  fold_rows(hx, wx);
  fold_rows(hy, wy);
  fold_rows(hp, wy);
  double mean = 0.;
  for (int j = 1; j <= jt; j++) {
    double *r = hp.data() + (size_t)j * wy;
    r[1] += r[0];
    r[it] += r[it + 1];
    r[0] = r[it + 1] = 0.;
    hx[(size_t)j * wx + 0] = hx[(size_t)j * wx + it] = 0.;   // wall faces 1 and itot+1
    hy[(size_t)j * wy + 0] = hy[(size_t)j * wy + it + 1] = 0.;
    for (int i = 1; i <= it; i++) mean += r[i];
  }
  mean /= (double)it * jt;
  for (int j = 1; j <= jt; j++)
    for (int i = 1; i <= it; i++) hp[(size_t)j * wy + i] -= mean;
  const size_t dp = sizeof(double) * c->ld;
  EIF_CK(c, cudaMemcpy2DAsync(a->ub, dp, hx.data(), sizeof(double) * wx, sizeof(double) * wx, rows,
                              cudaMemcpyHostToDevice, c->stream));
  EIF_CK(c, cudaMemcpy2DAsync(a->vb, dp, hy.data(), sizeof(double) * wy, sizeof(double) * wy, rows,
                              cudaMemcpyHostToDevice, c->stream));
  EIF_CK(c, cudaMemcpy2DAsync(a->pb, dp, hp.data(), sizeof(double) * wy, sizeof(double) * wy, rows,
                              cudaMemcpyHostToDevice, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return EIF_OK;
}

// the transposed step of the last recorded forward step: the cotangents of its output
// become those of its input (the step is removed from the tape)
int eif_adjoint_backward(eif_ctx *c) {
  int rc = adj_check(c);
  if (rc) return rc;
  Adjoint *a = c->adj;
  if (a->nrec == 0) return fail(c, EIF_ERR_STATE, "no recorded step to go back through");
  const int s = a->nrec - 1;
  const double dt = a->tape_dt[s];
  const size_t bytes = sizeof(double) * c->nfield;
  AdjGeom g;
  g.rdxf = c->rdxf; g.rdxc = c->rdxc; g.cxm = c->cxm; g.cxp = c->cxp; g.cym = c->cym; g.cyp = c->cyp;
  g.rRe = 1. / c->cfg.Re; g.rdy = 1. / c->dy;
  g.itot = c->itot; g.jtot = c->jtot; g.ld = c->ld;
  EIF_CK(c, cudaMemsetAsync(a->abx, 0, bytes, c->stream));
  EIF_CK(c, cudaMemsetAsync(a->aby, 0, bytes, c->stream));
  for (int rk = 2; rk >= 0; rk--) {
    const RK k = rk_coef(rk);
    // projection: phi = L^-1 (D ubar' + pbar' / (g dt)), ubar** = ubar' - G phi
    k_adj_rhs<<<agrid(c), dim3(AX, AY), 0, c->stream>>>(a->ub, a->vb, a->pb, a->rhs, 1. / c->dx, 1. / c->dy,
                                                         1. / (k.gamma * dt), c->itot, c->jtot, c->ld);
    EIF_LAUNCH_CK(c);
    c->adj_rhs = a->rhs;
    rc = launch_potential(c, rk, false);
    c->adj_rhs = nullptr;
    if (rc) return rc;
    k_adj_grad<<<agrid(c), dim3(AX, AY), 0, c->stream>>>(c->psi, c->rdxc, a->ub, a->vb, 1. / c->dy, c->itot, c->jtot,
                                                          c->ld);
    EIF_LAUNCH_CK(c);
    // forcing of the frozen particles
    const double *sx = a->ub, *sy = a->vb;
    if (c->np > 0) {
      k_adj_forcing<<<agrid(c), dim3(AX, AY), 0, c->stream>>>(a->ub, a->vb, a->w, a->tu, a->tv, c->itot, c->jtot,
                                                               c->ld);
      EIF_LAUNCH_CK(c);
      sx = a->tu;
      sy = a->tv;
    }
    // predictor around the recorded stage input
    AdjPredArgs p;
    p.u = a->tape_u[3 * s + rk];
    p.v = a->tape_v[3 * s + rk];
    p.sbx = sx; p.sby = sy;
    p.abx = a->abx; p.aby = a->aby;
    double *ox = c->np > 0 ? a->ub : a->tu, *oy = c->np > 0 ? a->vb : a->tv;
    p.ubo = ox; p.vbo = oy;
    p.pb = a->pb;
    p.g = g;
    p.adt = k.alpha * dt; p.bdt = k.beta * dt; p.gdt = k.gamma * dt;
    k_adj_predictor<<<agrid(c), dim3(AX, AY), 0, c->stream>>>(p);
    EIF_LAUNCH_CK(c);
    k_adj_srcb<<<agrid(c), dim3(AX, AY), 0, c->stream>>>(sx, sy, a->abx, a->aby, k.beta * dt, c->itot, c->jtot, c->ld);
    EIF_LAUNCH_CK(c);
    if (c->np == 0) {
      std::swap(a->ub, a->tu);
      std::swap(a->vb, a->tv);
    }
  }
  a->nrec--;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return check_records(c);
}

int eif_adjoint_pull(eif_ctx *c, double *ux_bar, double *uy_bar, double *p_bar) {
  int rc = adj_check(c);
  if (rc) return rc;
  Adjoint *a = c->adj;
  const size_t dp = sizeof(double) * c->ld;
  const int rows = c->jtot + 2;
  const size_t wx = sizeof(double) * (c->itot + 1), wy = sizeof(double) * (c->itot + 2);
  if (ux_bar) EIF_CK(c, cudaMemcpy2DAsync(ux_bar, wx, a->ub, dp, wx, rows, cudaMemcpyDeviceToHost, c->stream));
  if (uy_bar) EIF_CK(c, cudaMemcpy2DAsync(uy_bar, wy, a->vb, dp, wy, rows, cudaMemcpyDeviceToHost, c->stream));
  if (p_bar) EIF_CK(c, cudaMemcpy2DAsync(p_bar, wy, a->pb, dp, wy, rows, cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return EIF_OK;
}

int eif_adjoint_recorded(eif_ctx *c) { return (c && c->adj) ? c->adj->nrec : 0; }

}  // extern "C"
