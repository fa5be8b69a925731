// Discrete adjoint of the time step in the double-precision form.
//
// The step map (src/main.c:14-52) with dt held at its recorded value is, per RK
// stage k, with the particle state Pi = (X, Y, az, U, V, Omega):
//   I0   = Inert(u_k; X)                       inertia.c:9-70 (cnstep 0)
//   u*   = u_k + dt (a_k A(u_k) + b_k A_{k-1} - g_k G p_k)      update_velocity.c
//   F, dux = Exch(u*; X, U)                    exchange.c:13-88
//   u**  = u* + Avg dux                        update.c:36-59
//   psi  = L^-1 D u** / (g_k dt), u_{k+1} = u** - g_k dt G psi, p_{k+1} = p_k + psi
//   dX_0 = 0; for m < K: I1_m = Inert(u_{k+1}; X + dX_m),
//        dU_{m+1} = dt F + I1_m - I0 + c,  dX_{m+1} = g_k dt (U + dU_{m+1} / 2)
//   U' = U + dU_K, X' = X + dX_K                increment.c, update.c:8-34
// (main.c:32-49; K is the recorded sub-iteration count). Collision forces enter as
// constants: the adjoint is that of contact-free motion ("collision away from
// contact"), and a recorded step with a non-zero collision force is reported.
// The adjoint applies the transposed linearisation around the recorded states in
// reverse: the sub-iterations from m = K-1 down to 0 (each a transposed inertia
// evaluation at X + dX_m), the projection, the exchange, the predictor and the
// inertia at X. The transposed box evaluations are in ibm.cu (launch_adj_pass).
//
//   projection:  phi = L^-1 (D ubar' + pbar' / (g dt)),  ubar** = ubar' - G phi
//                (on the uniform staggered grid G^T = -D and L = D G is symmetric,
//                so the double-precision Poisson solver of the forward step is reused)
//   predictor:   ubar_k = ubar* + (dA/du)^T (dt a_k ubar* + Abar_k),
//                pbar += dt g_k G^T ubar*,  Abar_{k-1} = dt b_k ubar*
//
// A second mode freezes the particles (their records are parameters; no inertia,
// collision, increment or update runs; the forcing acts with their rigid-body
// velocities). The transposed stencils are gathers (each input sums the
// contributions of the outputs that read it), so results do not depend on thread
// order and a recomputed segment reproduces the same bits.
#include "eif_internal.cuh"
#include <algorithm>
#include <cstring>
#include <vector>

namespace eif {

struct Adjoint {
  int mode = EIF_ADJOINT_COUPLED;
  int max_steps = 0, nrec = 0, np = 0;
  // per step: dt, contact seen; per stage (3 per step): inputs u_k, v_k, predictor
  // outputs u*, v* (coupled), particle state (6 x np), sub-iteration count and
  // increments dX_m (m = 1..K, 3 x np each); per step the final velocity (coupled)
  std::vector<double *> tape_u, tape_v, tape_us, tape_vs, tape_out_u, tape_out_v, tape_p, tape_dx;
  std::vector<double> tape_dt;
  std::vector<int> tape_k;
  std::vector<char> tape_contact;
  // fluid cotangents (field layout): velocity, pressure, explicit terms, scratch
  double *ub = nullptr, *vb = nullptr, *pb = nullptr, *abx = nullptr, *aby = nullptr;
  double *tu = nullptr, *tv = nullptr, *rhs = nullptr, *w = nullptr, *fcx = nullptr, *fcy = nullptr;
  double *gcx = nullptr, *gcy = nullptr;   // cell cotangents of the field response (cell layout)
  // particle cotangents (3 x np each): position, velocity, carried increment, force,
  // inertia at X, inertia of one sub-iteration; box-pass output (6 x np) and scratch
  double *xb = nullptr, *vpb = nullptr, *dub = nullptr, *fb = nullptr, *i0b = nullptr, *i1b = nullptr;
  double *pout = nullptr, *part = nullptr;
  int part_cap = 0;
  // indicator geometry of the box cells at X, shared by the three transposed evaluations
  // at X of a stage (last sub-iteration, exchange, inertia at the stage start)
  double *geom = nullptr;
  size_t geom_cap = 0;
  // wall-velocity cotangent: per row (2 x jtot) and accumulated (2)
  double *wall_rows = nullptr, *wall = nullptr;
  double *pbackup = nullptr;   // particle records during backward
  int *d_contact = nullptr;
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
  double *wall;                 // 2 x jtot: per row, cotangents of the wall values of uy
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
    // the wall values uy(0, j) and uy(itot+1, j) are read by A_y at cells 1 and itot
    if (i == 1) a.wall[j - 1] = gy_at(a, 1, j) * day(a.u, a.v, g, 1, j).dvw;
    if (i == itot) a.wall[jtot + j - 1] = gy_at(a, itot, j) * day(a.u, a.v, g, itot, j).dve;
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


__global__ void k_adj_wall_sum(const double *__restrict__ rows, double *__restrict__ wall, int jtot) {
  // one block: fixed-order tree sums of the two rows of per-row wall cotangents
  __shared__ double s[2][256];
  for (int side = 0; side < 2; side++) {
    double v = 0.;
    for (int j = threadIdx.x; j < jtot; j += blockDim.x) v += rows[side * jtot + j];
    s[side][threadIdx.x] = v;
  }
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      s[0][threadIdx.x] += s[0][threadIdx.x + o];
      s[1][threadIdx.x] += s[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    wall[0] += s[0][0];
    wall[1] += s[1][0];
  }
}

// cell cotangents of the field response from the face cotangents of u**:
// u**(face i) = u*(face i) + (dux(i-1) + dux(i)) / 2  (update.c:36-59)
__global__ void k_adj_cellavg(const double *__restrict__ sx, const double *__restrict__ sy, double *__restrict__ gx,
                              double *__restrict__ gy, int itot, int jtot, int ld) {
  const int i = 1 + blockIdx.x * AX + threadIdx.x;
  const int j = 1 + blockIdx.y * AY + threadIdx.y;
  if (i > itot || j > jtot) return;
  const double uw = i >= 2 ? sx[ux_idx(i, j, ld)] : 0., ue = i + 1 <= itot ? sx[ux_idx(i + 1, j, ld)] : 0.;
  const int c = uy_idx(i, j, ld);
  gx[c] = 0.5 * (uw + ue);
  gy[c] = 0.5 * (sy[c] + sy[uy_idx(i, wrapj(j + 1, jtot), ld)]);
}

// face cotangents from cell cotangents of face-averaged velocities
// (u_c = (u(face i) + u(face i+1)) / 2, v_c = (v(j) + v(j+1)) / 2): added
__global__ void k_adj_avgT_add(const double *__restrict__ gx, const double *__restrict__ gy, double *__restrict__ sx,
                               double *__restrict__ sy, int itot, int jtot, int ld) {
  const int i = 1 + blockIdx.x * AX + threadIdx.x;
  const int j = 1 + blockIdx.y * AY + threadIdx.y;
  if (i > itot || j > jtot) return;
  const int c = uy_idx(i, j, ld);
  if (i >= 2) sx[ux_idx(i, j, ld)] += 0.5 * (gx[c - 1] + gx[c]);
  sy[c] += 0.5 * (gy[uy_idx(i, wrapj(j - 1, jtot), ld)] + gy[c]);
}

// ---- particle state and cotangents (one thread per particle) ----
__device__ __forceinline__ int pstate_field(int k) {
  return k < 3 ? EIF_P_X + k : EIF_P_UX + (k - 3);   // x, y, az, ux, uy, vz
}

__global__ void k_adj_psave(const double *__restrict__ P, int pcap, int np, double *__restrict__ dst) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= np) return;
#pragma unroll
  for (int k = 0; k < 6; k++) dst[k * np + n] = P[pstate_field(k) * pcap + n];
}
// the particle state of a stage start, increments zero
__global__ void k_adj_pload(double *__restrict__ P, int pcap, int np, const double *__restrict__ src) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= np) return;
#pragma unroll
  for (int k = 0; k < 6; k++) P[pstate_field(k) * pcap + n] = src[k * np + n];
  P[EIF_P_DX * pcap + n] = 0.;
  P[EIF_P_DY * pcap + n] = 0.;
  P[EIF_P_DAZ * pcap + n] = 0.;
}
__global__ void k_adj_dxsave(const double *__restrict__ P, int pcap, int np, double *__restrict__ dst) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= np) return;
  dst[n] = P[EIF_P_DX * pcap + n];
  dst[np + n] = P[EIF_P_DY * pcap + n];
  dst[2 * np + n] = P[EIF_P_DAZ * pcap + n];
}
__global__ void k_adj_dxload(double *__restrict__ P, int pcap, int np, const double *__restrict__ src) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= np) return;
  P[EIF_P_DX * pcap + n] = src[n];
  P[EIF_P_DY * pcap + n] = src[np + n];
  P[EIF_P_DAZ * pcap + n] = src[2 * np + n];
}
// any non-zero collision force or torque of this stage (increment.c:24-36)
__global__ void k_adj_contact(const double *__restrict__ P, int pcap, int np, int *__restrict__ flag) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= np) return;
  bool any = false;
  for (int f = EIF_P_CFX0; f <= EIF_P_CTZ1; f++) any |= P[f * pcap + n] != 0.;
  if (any) *flag = 1;
}
// reverse of U' = U + dU_K, X' = X + dX_K, dX_K = g dt (U + dU_K / 2):
// dUbar = Ubar' + (g dt / 2) Xbar', Ubar = Ubar' + g dt Xbar', Xbar = Xbar'
__global__ void k_adj_stage_init(int np, double gdt, const double *__restrict__ xb, double *__restrict__ vpb,
                                 double *__restrict__ dub, double *__restrict__ fb, double *__restrict__ i0b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * np) return;
  dub[t] = vpb[t] + 0.5 * gdt * xb[t];
  vpb[t] += gdt * xb[t];
  fb[t] = 0.;
  i0b[t] = 0.;
}
// reverse of dU_{m+1} = dt F + I1_m - I0
__global__ void k_adj_iter_pre(int np, double dt, const double *__restrict__ dub, double *__restrict__ fb,
                               double *__restrict__ i0b, double *__restrict__ i1b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * np) return;
  fb[t] += dt * dub[t];
  i0b[t] -= dub[t];
  i1b[t] = dub[t];
}
// reverse of I1_m = Inert(X + dX_m) in the particle state: the position cotangent z
// goes to X, and for m >= 1 through dX_m = g dt (U + dU_m / 2) to U and dU_m
__global__ void k_adj_iter_post(int np, double gdt, const double *__restrict__ pout, double *__restrict__ xb,
                                double *__restrict__ vpb, double *__restrict__ dub, int more) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * np) return;
  const double z = pout[t];
  xb[t] += z;
  if (more) {
    vpb[t] += gdt * z;
    dub[t] = 0.5 * gdt * z;
  }
}
__global__ void k_adj_part_add(int np, const double *__restrict__ pout, double *__restrict__ xb,
                               double *__restrict__ vpb, int with_velocity) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * np) return;
  xb[t] += pout[t];
  if (with_velocity) vpb[t] += pout[3 * np + t];
}

dim3 agrid(const eif_ctx *c) { return dim3((c->itot + AX - 1) / AX, (c->jtot + AY - 1) / AY); }
int pblocks(int n) { return (n + 127) / 128; }

}  // namespace

using namespace eif;

namespace {

void adj_free(eif_ctx *c) {
  Adjoint *a = c->adj;
  if (!a) return;
  for (auto *v : {&a->tape_u, &a->tape_v, &a->tape_us, &a->tape_vs, &a->tape_out_u, &a->tape_out_v, &a->tape_p,
                  &a->tape_dx})
    for (double *p : *v)
      if (p) cudaFree(p);
  for (double *p : {a->ub, a->vb, a->pb, a->abx, a->aby, a->tu, a->tv, a->rhs, a->w, a->fcx, a->fcy, a->gcx, a->gcy, a->xb, a->vpb,
                    a->dub, a->fb, a->i0b, a->i1b, a->pout, a->part, a->wall_rows, a->wall, a->pbackup, a->geom})
    if (p) cudaFree(p);
  if (a->d_contact) cudaFree(a->d_contact);
  delete a;
  c->adj = nullptr;
}

int adj_check(eif_ctx *c) {
  if (!c) return EIF_ERR_ARG;
  if (!c->adj) return fail(c, EIF_ERR_STATE, "call eif_adjoint_begin first");
  return EIF_OK;
}

int read_scalars(eif_ctx *c) {
  EIF_CK(c, cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(double) * 4, cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaMemcpyAsync(c->h_flags, c->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  int rc = check_records(c);
  if (rc) return rc;
  return check_flags(c);
}

int set_device_dt(eif_ctx *c, double dt) {
  c->h_scal[0] = dt;
  EIF_CK(c, cudaMemcpyAsync(c->d_scal, c->h_scal, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return EIF_OK;
}

// one RK stage of the frozen-particle forward (fluid only)
int frozen_stage(eif_ctx *c, int rk) {
  int rc;
  const bool ibm = c->np > 0;
  if ((rc = launch_predictor(c, rk))) return rc;
  if (ibm && (rc = launch_exchange(c))) return rc;
  if ((rc = launch_potential(c, rk, ibm))) return rc;
  return launch_correct(c, rk, ibm, true);
}

// one RK stage of the full step (src/main.c:14-52), recording for the adjoint when
// slot >= 0: u_k, u*, the particle state and every sub-iteration's increments
int coupled_stage(eif_ctx *c, int rk, int slot) {
  Adjoint *a = c->adj;
  const size_t bytes = sizeof(double) * c->nfield;
  const int np = c->np;
  int rc;
  if (slot >= 0 && np > 0) {
    k_adj_psave<<<pblocks(np), 128, 0, c->stream>>>(c->P, c->pcap, np, a->tape_p[slot]);
    EIF_LAUNCH_CK(c);
  }
  if ((rc = launch_reset_increments(c))) return rc;
  if ((rc = launch_inertia(c, 0))) return rc;
  if (slot >= 0) {
    EIF_CK(c, cudaMemcpyAsync(a->tape_u[slot], c->ux[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
    EIF_CK(c, cudaMemcpyAsync(a->tape_v[slot], c->uy[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
  }
  if ((rc = launch_predictor(c, rk))) return rc;
  if (slot >= 0) {
    EIF_CK(c, cudaMemcpyAsync(a->tape_us[slot], c->ux[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
    EIF_CK(c, cudaMemcpyAsync(a->tape_vs[slot], c->uy[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
  }
  const bool ibm = np > 0;
  if (ibm && (rc = launch_exchange(c))) return rc;
  if ((rc = launch_potential(c, rk, ibm))) return rc;
  if ((rc = launch_correct(c, rk, ibm, true))) return rc;
  if (np == 0) {
    if (slot >= 0) a->tape_k[slot] = 0;
    return EIF_OK;
  }
  if ((rc = launch_collision(c, 0))) return rc;
  int m = 0;
  for (;; m++) {
    if ((rc = launch_inertia(c, 1))) return rc;
    if ((rc = launch_collision(c, 1))) return rc;
    if ((rc = launch_increment(c, rk))) return rc;
    if (slot >= 0) {
      // dX_{m+1}: the positions of the next sub-iteration's inertia
      k_adj_dxsave<<<pblocks(np), 128, 0, c->stream>>>(c->P, c->pcap, np,
                                                        a->tape_dx[slot] + (size_t)3 * np * (m + 1));
      EIF_LAUNCH_CK(c);
      k_adj_contact<<<pblocks(np), 128, 0, c->stream>>>(c->P, c->pcap, np, a->d_contact);
      EIF_LAUNCH_CK(c);
    }
    if ((rc = read_scalars(c))) return rc;
    if (c->h_scal[1] < 1.e-8) break;   // main.c:40-48
    if (m > 100) break;
  }
  if (slot >= 0) a->tape_k[slot] = m + 1;
  return launch_update_particles(c);
}

}  // namespace

extern "C" {

int eif_adjoint_begin(eif_ctx *c, int max_steps, int mode) {
  if (!c || max_steps <= 0 || (mode != EIF_ADJOINT_COUPLED && mode != EIF_ADJOINT_FROZEN)) return EIF_ERR_ARG;
  if (c->cfg.precision != EIF_PREC_FP64) return fail(c, EIF_ERR_ARG, "the adjoint is built on the double-precision form");
  if (!c->fluid_pushed) return fail(c, EIF_ERR_STATE, "push the fluid state before eif_adjoint_begin");
  adj_free(c);
  Adjoint *a = new Adjoint;
  c->adj = a;
  a->mode = mode;
  a->max_steps = max_steps;
  a->np = c->np;
  const bool coupled = mode == EIF_ADJOINT_COUPLED;
  const size_t bytes = sizeof(double) * c->nfield;
  const int np = c->np;
  auto field = [&](std::vector<double *> &v, int n) -> int {
    for (int k = 0; k < n; k++) {
      double *p = nullptr;
      EIF_CK(c, cudaMalloc((void **)&p, bytes));
      v.push_back(p);
    }
    return EIF_OK;
  };
  int rc;
  if ((rc = field(a->tape_u, 3 * max_steps)) || (rc = field(a->tape_v, 3 * max_steps))) return rc;
  if (coupled) {
    if ((rc = field(a->tape_us, 3 * max_steps)) || (rc = field(a->tape_vs, 3 * max_steps))) return rc;
    if ((rc = field(a->tape_out_u, max_steps)) || (rc = field(a->tape_out_v, max_steps))) return rc;
    for (int k = 0; np > 0 && k < 3 * max_steps; k++) {
      double *p = nullptr, *q = nullptr;
      EIF_CK(c, cudaMalloc((void **)&p, sizeof(double) * 6 * np));
      a->tape_p.push_back(p);
      // increments of up to 102 sub-iterations (main.c:46) plus dX_0
      EIF_CK(c, cudaMalloc((void **)&q, sizeof(double) * 3 * np * 104));
      EIF_CK(c, cudaMemsetAsync(q, 0, sizeof(double) * 3 * np, c->stream));
      a->tape_dx.push_back(q);
    }
  }
  a->tape_dt.assign(max_steps, 0.);
  a->tape_k.assign(3 * max_steps, 0);
  a->tape_contact.assign(max_steps, 0);
  for (double **p : {&a->ub, &a->vb, &a->pb, &a->abx, &a->aby, &a->tu, &a->tv, &a->rhs, &a->w, &a->fcx, &a->fcy,
                     &a->gcx, &a->gcy}) {
    EIF_CK(c, cudaMalloc((void **)p, bytes));
    EIF_CK(c, cudaMemsetAsync(*p, 0, bytes, c->stream));
  }
  const int n3 = std::max(1, 3 * np);
  for (double **p : {&a->xb, &a->vpb, &a->dub, &a->fb, &a->i0b, &a->i1b}) {
    EIF_CK(c, cudaMalloc((void **)p, sizeof(double) * n3));
    EIF_CK(c, cudaMemsetAsync(*p, 0, sizeof(double) * n3, c->stream));
  }
  EIF_CK(c, cudaMalloc((void **)&a->pout, sizeof(double) * 2 * n3));
  EIF_CK(c, cudaMalloc((void **)&a->wall_rows, sizeof(double) * 2 * c->jtot));
  EIF_CK(c, cudaMemsetAsync(a->wall_rows, 0, sizeof(double) * 2 * c->jtot, c->stream));
  EIF_CK(c, cudaMalloc((void **)&a->wall, sizeof(double) * 2));
  EIF_CK(c, cudaMemsetAsync(a->wall, 0, sizeof(double) * 2, c->stream));
  EIF_CK(c, cudaMalloc((void **)&a->pbackup, sizeof(double) * EIF_NFIELDS * std::max(1, c->pcap)));
  EIF_CK(c, cudaMalloc((void **)&a->d_contact, sizeof(int)));
  EIF_CK(c, cudaMemsetAsync(a->d_contact, 0, sizeof(int), c->stream));
  if (np > 0) {
    a->part_cap = adj_chunk_cap(c);
    EIF_CK(c, cudaMalloc((void **)&a->part, sizeof(double) * 6 * std::max(1, a->part_cap)));
  }
  // frozen mode: summed indicator weights of the particles, from the exchange with the
  // weights as the cell contributions (double-precision kernels) gathered into dux
  if (!coupled && np > 0) {
    c->ibm_weights_only = true;
    c->boxes_x_valid = false;
    c->weights_x_valid = false;
    rc = launch_exchange(c);
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

// One forward step with the current dt (the particles moving, or frozen); with
// record != 0 the step is recorded for eif_adjoint_backward. The step counter and
// time advance as in eif_advance.
int eif_adjoint_forward(eif_ctx *c, int record) {
  int rc = adj_check(c);
  if (rc) return rc;
  Adjoint *a = c->adj;
  if (c->np != a->np) return fail(c, EIF_ERR_STATE, "the particle count changed since eif_adjoint_begin");
  if (record && a->nrec >= a->max_steps) return fail(c, EIF_ERR_ARG, "the adjoint tape holds %d steps", a->max_steps);
  const size_t bytes = sizeof(double) * c->nfield;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  const int s = a->nrec;
  if (record) a->tape_dt[s] = c->dt_host;
  if (a->mode == EIF_ADJOINT_FROZEN) {
    for (int rk = 0; rk < 3; rk++) {
      if (record) {
        EIF_CK(c, cudaMemcpyAsync(a->tape_u[3 * s + rk], c->ux[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
        EIF_CK(c, cudaMemcpyAsync(a->tape_v[3 * s + rk], c->uy[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
      }
      if ((rc = frozen_stage(c, rk))) return rc;
    }
  } else {
    if (record) EIF_CK(c, cudaMemsetAsync(a->d_contact, 0, sizeof(int), c->stream));
    for (int rk = 0; rk < 3; rk++)
      if ((rc = coupled_stage(c, rk, record ? 3 * s + rk : -1))) return rc;
    if (record) {
      EIF_CK(c, cudaMemcpyAsync(a->tape_out_u[s], c->ux[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
      EIF_CK(c, cudaMemcpyAsync(a->tape_out_v[s], c->uy[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
      int contact = 0;
      EIF_CK(c, cudaMemcpyAsync(&contact, a->d_contact, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      EIF_CK(c, cudaStreamSynchronize(c->stream));
      a->tape_contact[s] = contact ? 1 : 0;
    }
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
// cotangent of the state; theirs starts the wall-velocity gradient). The pressure
// is determined up to a constant, so the mean of its cotangent over the cells is
// removed. p_bar may be NULL for zero. The particle cotangents are reset to zero.
int eif_adjoint_seed(eif_ctx *c, const double *ux_bar, const double *uy_bar, const double *p_bar) {
  int rc = adj_check(c);
  if (rc) return rc;
  if (!ux_bar || !uy_bar) return EIF_ERR_ARG;
  Adjoint *a = c->adj;
  const int it = c->itot, jt = c->jtot, rows = jt + 2;
  const int wx = it + 1, wy = it + 2;
  std::vector<double> hx(ux_bar, ux_bar + (size_t)wx * rows), hy(uy_bar, uy_bar + (size_t)wy * rows);
  std::vector<double> hp((size_t)wy * rows, 0.);
  // the uy wall columns of the state (all rows) hold the wall velocities: their
  // cotangents start the wall-velocity gradient
  double hw[2] = {0., 0.};
  for (int j = 0; j < rows; j++) {
    hw[0] += hy[(size_t)j * wy];
    hw[1] += hy[(size_t)j * wy + it + 1];
  }
  if (p_bar) std::memcpy(hp.data(), p_bar, sizeof(double) * hp.size());
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
  const size_t n3 = sizeof(double) * std::max(1, 3 * a->np);
  EIF_CK(c, cudaMemsetAsync(a->xb, 0, n3, c->stream));
  EIF_CK(c, cudaMemsetAsync(a->vpb, 0, n3, c->stream));
  EIF_CK(c, cudaMemcpyAsync(a->wall, hw, sizeof(double) * 2, cudaMemcpyHostToDevice, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return EIF_OK;
}

// particle cotangents after the last recorded step: n records of EIF_NFIELDS
// doubles, of which x, y, az, ux, uy, vz are read (coupled mode)
int eif_adjoint_seed_particles(eif_ctx *c, int n, const double *rec_bar) {
  int rc = adj_check(c);
  if (rc) return rc;
  Adjoint *a = c->adj;
  if (n != a->np || (n > 0 && !rec_bar)) return fail(c, EIF_ERR_ARG, "expected %d particle records", a->np);
  if (n == 0) return EIF_OK;
  std::vector<double> h(6 * (size_t)n);
  static const int f[6] = {EIF_P_X, EIF_P_Y, EIF_P_AZ, EIF_P_UX, EIF_P_UY, EIF_P_VZ};
  for (int k = 0; k < 6; k++)
    for (int q = 0; q < n; q++) h[(size_t)k * n + q] = rec_bar[(size_t)q * EIF_NFIELDS + f[k]];
  EIF_CK(c, cudaMemcpyAsync(a->xb, h.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
  EIF_CK(c, cudaMemcpyAsync(a->vpb, h.data() + 3 * n, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
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
  const bool coupled = a->mode == EIF_ADJOINT_COUPLED;
  if (coupled && a->tape_contact[s])
    return fail(c, EIF_ERR_STATE, "a collision force acted in the recorded step: the adjoint covers contact-free motion");
  const double dt = a->tape_dt[s];
  const size_t bytes = sizeof(double) * c->nfield;
  const int np = a->np;
  const dim3 G = agrid(c), B(AX, AY);
  AdjGeom g;
  g.rdxf = c->rdxf; g.rdxc = c->rdxc; g.cxm = c->cxm; g.cxp = c->cxp; g.cym = c->cym; g.cyp = c->cyp;
  g.rRe = 1. / c->cfg.Re; g.rdy = 1. / c->dy;
  g.itot = c->itot; g.jtot = c->jtot; g.ld = c->ld;
  // the particle records and dt of the forward stay as they were
  const double dt_keep = c->dt_host;
  if ((rc = set_device_dt(c, dt))) return rc;
  if (coupled && np > 0) {
    if (adj_chunk_cap(c) > a->part_cap) {
      cudaFree(a->part);
      a->part = nullptr;
      a->part_cap = adj_chunk_cap(c);
      EIF_CK(c, cudaMalloc((void **)&a->part, sizeof(double) * 6 * a->part_cap));
    }
    if (adj_slot_cap(c) > a->geom_cap) {
      if (a->geom) cudaFree(a->geom);
      a->geom = nullptr;
      a->geom_cap = adj_slot_cap(c);
      EIF_CK(c, cudaMalloc((void **)&a->geom, sizeof(double) * 3 * a->geom_cap));
    }
    EIF_CK(c, cudaMemcpyAsync(a->pbackup, c->P, sizeof(double) * EIF_NFIELDS * c->pcap, cudaMemcpyDeviceToDevice,
                              c->stream));
  }
  EIF_CK(c, cudaMemsetAsync(a->abx, 0, bytes, c->stream));
  EIF_CK(c, cudaMemsetAsync(a->aby, 0, bytes, c->stream));
  AdjPass pass;
  pass.part = a->part;
  pass.out = a->pout;
  pass.fx = a->fcx;
  pass.fy = a->fcy;
  for (int rk = 2; rk >= 0; rk--) {
    const RK k = rk_coef(rk);
    const int slot = 3 * s + rk;
    const double gdt = k.gamma * dt;
    if (coupled && np > 0) {
      // sub-iterations in reverse (the particle state of the stage start in P)
      k_adj_pload<<<pblocks(np), 128, 0, c->stream>>>(c->P, c->pcap, np, a->tape_p[slot]);
      EIF_LAUNCH_CK(c);
      c->boxes_x_valid = false;
      c->weights_x_valid = false;
      c->bands_x_valid = false;
      k_adj_stage_init<<<pblocks(3 * np), 128, 0, c->stream>>>(np, gdt, a->xb, a->vpb, a->dub, a->fb, a->i0b);
      EIF_LAUNCH_CK(c);
      pass.mode = 0;
      pass.ux = rk < 2 ? a->tape_u[slot + 1] : a->tape_out_u[s];
      pass.uy = rk < 2 ? a->tape_v[slot + 1] : a->tape_out_v[s];
      pass.bar = a->i1b;
      for (int m = a->tape_k[slot] - 1; m >= 0; m--) {
        k_adj_iter_pre<<<pblocks(3 * np), 128, 0, c->stream>>>(np, dt, a->dub, a->fb, a->i0b, a->i1b);
        EIF_LAUNCH_CK(c);
        k_adj_dxload<<<pblocks(np), 128, 0, c->stream>>>(c->P, c->pcap, np, a->tape_dx[slot] + (size_t)3 * np * m);
        EIF_LAUNCH_CK(c);
        pass.use_increment = m > 0;
        pass.geo = m == 0 ? 1 : 0;   // the pass at X keeps the geometry for the two below
        pass.geom = a->geom;
        if ((rc = launch_adj_pass(c, pass))) return rc;
        k_adj_avgT_add<<<G, B, 0, c->stream>>>(a->fcx, a->fcy, a->ub, a->vb, c->itot, c->jtot, c->ld);
        EIF_LAUNCH_CK(c);
        k_adj_iter_post<<<pblocks(3 * np), 128, 0, c->stream>>>(np, gdt, a->pout, a->xb, a->vpb, a->dub, m > 0);
        EIF_LAUNCH_CK(c);
      }
      k_adj_dxload<<<pblocks(np), 128, 0, c->stream>>>(c->P, c->pcap, np, a->tape_dx[slot]);   // dX_0 = 0
      EIF_LAUNCH_CK(c);
      // the boxes of the last pass (m = 0) are those at X, kept for the passes below
    }
    // projection: phi = L^-1 (D ubar' + pbar' / (g dt)), ubar** = ubar' - G phi
    k_adj_rhs<<<G, B, 0, c->stream>>>(a->ub, a->vb, a->pb, a->rhs, 1. / c->dx, 1. / c->dy, 1. / gdt, c->itot, c->jtot,
                                      c->ld);
    EIF_LAUNCH_CK(c);
    c->adj_rhs = a->rhs;
    rc = launch_potential(c, rk, false);
    c->adj_rhs = nullptr;
    if (rc) return rc;
    k_adj_grad<<<G, B, 0, c->stream>>>(c->psi, c->rdxc, a->ub, a->vb, 1. / c->dy, c->itot, c->jtot, c->ld);
    EIF_LAUNCH_CK(c);
    // exchange: u** = u* + Avg dux(u*, X, U), F = F(u*, X, U)
    if (np > 0 && coupled) {
      k_adj_cellavg<<<G, B, 0, c->stream>>>(a->ub, a->vb, a->gcx, a->gcy, c->itot, c->jtot, c->ld);
      EIF_LAUNCH_CK(c);
      pass.mode = 1;
      pass.use_increment = false;
      pass.geo = a->tape_k[slot] > 0 ? 2 : 0;
      pass.ux = a->tape_us[slot];
      pass.uy = a->tape_vs[slot];
      pass.bar = a->fb;
      pass.gx = a->gcx;
      pass.gy = a->gcy;
      if ((rc = launch_adj_pass(c, pass))) return rc;
      k_adj_avgT_add<<<G, B, 0, c->stream>>>(a->fcx, a->fcy, a->ub, a->vb, c->itot, c->jtot, c->ld);
      EIF_LAUNCH_CK(c);
      k_adj_part_add<<<pblocks(3 * np), 128, 0, c->stream>>>(np, a->pout, a->xb, a->vpb, 1);
      EIF_LAUNCH_CK(c);
    } else if (np > 0) {
      k_adj_forcing<<<G, B, 0, c->stream>>>(a->ub, a->vb, a->w, a->tu, a->tv, c->itot, c->jtot, c->ld);
      EIF_LAUNCH_CK(c);
      std::swap(a->ub, a->tu);
      std::swap(a->vb, a->tv);
    }
    // predictor around the recorded stage input
    AdjPredArgs p;
    p.u = a->tape_u[slot];
    p.v = a->tape_v[slot];
    p.sbx = a->ub; p.sby = a->vb;
    p.abx = a->abx; p.aby = a->aby;
    p.ubo = a->tu; p.vbo = a->tv;
    p.pb = a->pb;
    p.wall = a->wall_rows;
    p.g = g;
    p.adt = k.alpha * dt; p.bdt = k.beta * dt; p.gdt = gdt;
    k_adj_predictor<<<G, B, 0, c->stream>>>(p);
    EIF_LAUNCH_CK(c);
    k_adj_srcb<<<G, B, 0, c->stream>>>(a->ub, a->vb, a->abx, a->aby, k.beta * dt, c->itot, c->jtot, c->ld);
    EIF_LAUNCH_CK(c);
    k_adj_wall_sum<<<1, 256, 0, c->stream>>>(a->wall_rows, a->wall, c->jtot);
    EIF_LAUNCH_CK(c);
    std::swap(a->ub, a->tu);
    std::swap(a->vb, a->tv);
    // inertia at the stage start: I0 = Inert(u_k; X)
    if (coupled && np > 0) {
      pass.mode = 0;
      pass.use_increment = false;
      pass.geo = a->tape_k[slot] > 0 ? 2 : 0;
      pass.ux = a->tape_u[slot];
      pass.uy = a->tape_v[slot];
      pass.bar = a->i0b;
      if ((rc = launch_adj_pass(c, pass))) return rc;
      k_adj_avgT_add<<<G, B, 0, c->stream>>>(a->fcx, a->fcy, a->ub, a->vb, c->itot, c->jtot, c->ld);
      EIF_LAUNCH_CK(c);
      k_adj_part_add<<<pblocks(3 * np), 128, 0, c->stream>>>(np, a->pout, a->xb, a->vpb, 0);
      EIF_LAUNCH_CK(c);
    }
  }
  if (coupled && np > 0) {
    EIF_CK(c, cudaMemcpyAsync(c->P, a->pbackup, sizeof(double) * EIF_NFIELDS * c->pcap, cudaMemcpyDeviceToDevice,
                              c->stream));
    c->boxes_x_valid = false;
    c->weights_x_valid = false;
    c->bands_x_valid = false;
  }
  a->nrec--;
  if ((rc = set_device_dt(c, dt_keep))) return rc;
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

int eif_adjoint_pull_particles(eif_ctx *c, int n, double *rec_bar) {
  int rc = adj_check(c);
  if (rc) return rc;
  Adjoint *a = c->adj;
  if (n != a->np || (n > 0 && !rec_bar)) return fail(c, EIF_ERR_ARG, "expected %d particle records", a->np);
  if (n == 0) return EIF_OK;
  std::vector<double> h(6 * (size_t)n);
  EIF_CK(c, cudaMemcpyAsync(h.data(), a->xb, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaMemcpyAsync(h.data() + 3 * n, a->vpb, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  static const int f[6] = {EIF_P_X, EIF_P_Y, EIF_P_AZ, EIF_P_UX, EIF_P_UY, EIF_P_VZ};
  std::memset(rec_bar, 0, sizeof(double) * EIF_NFIELDS * (size_t)n);
  for (int k = 0; k < 6; k++)
    for (int q = 0; q < n; q++) rec_bar[(size_t)q * EIF_NFIELDS + f[k]] = h[(size_t)k * n + q];
  return EIF_OK;
}

int eif_adjoint_wall_gradient(eif_ctx *c, double *d_uy_wall) {
  int rc = adj_check(c);
  if (rc) return rc;
  if (!d_uy_wall) return EIF_ERR_ARG;
  EIF_CK(c, cudaMemcpyAsync(d_uy_wall, c->adj->wall, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return EIF_OK;
}

int eif_adjoint_recorded(eif_ctx *c) { return (c && c->adj) ? c->adj->nrec : 0; }

int eif_adjoint_substeps(eif_ctx *c, int step, int *substeps) {
  int rc = adj_check(c);
  if (rc) return rc;
  if (step < 0 || step >= c->adj->nrec || !substeps) return EIF_ERR_ARG;
  for (int rk = 0; rk < 3; rk++) substeps[rk] = c->adj->tape_k[3 * step + rk];
  return EIF_OK;
}

}  // extern "C"
