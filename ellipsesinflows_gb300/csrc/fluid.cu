// Fluid kernels: boundary values, RK predictor, projection, pressure update,
// time-step size and divergence diagnostics.
//
// Reference functions restated here (NaokiHori/EllipsesInFlows):
//   fluid_update_boundaries_{ux,uy,p}   src/fluid/boundary_conditions.c:7-62
//   compute_src_ux / compute_src_uy     src/fluid/update_velocity.c:9-173
//   update_ux / update_uy               src/fluid/update_velocity.c:175-227
//   suspensions_update_momentum_fleid   src/suspensions/update.c:36-59
//   fluid_correct_velocity              src/fluid/correct_velocity.c:6-42
//   fluid_update_pressure               src/fluid/update_pressure.c:7-24
//   param_decide_dt                     src/param/decide_dt.c:11-81
//   check_divergence                    src/logging.c:40-80
#include "eif_internal.cuh"
#include "eif_df.cuh"
#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <cstdlib>
#include <cuda.h>
#include <cudaTypedefs.h>

namespace {

using eifd::ux_idx;
using eifd::uy_idx;

constexpr int TX = 32;
// tile heights of the stencil kernels the tuner chooses from (results do not depend on it)
constexpr int TY_DEFAULT = 8;

// ---------------------------------------------------------------------------
// boundary and halo values of one field kind
// kind 0: ux-like (halo i=2..itot, walls i=1,itot+1 set to 0)
// kind 1: uy-like (halo i=1..itot, walls i=0,itot+1 set to the wall velocity)
// kind 2: p-like  (halo i=1..itot, Neumann copies at i=0,itot+1 incl. halo rows)
// s (velocities of the mixed form, else null): the field rounded to float, kept with it
__global__ void k_bc(double *__restrict__ a, float *__restrict__ s, int kind, int itot, int jtot, int ld, double w0,
                     double w1) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  auto put = [&](int idx, double v) {
    a[idx] = v;
    if (s) s[idx] = eifd::d2f(v);
  };
  // halo rows
  const int ilo = kind == 0 ? 2 : 1;
  const int ihi = itot;
  const int col = kind == 0 ? -1 : 0;  // ux stores UX(i) at i-1
  if (t >= ilo && t <= ihi) {
    put(0 * ld + t + col, a[jtot * ld + t + col]);
    put((jtot + 1) * ld + t + col, a[1 * ld + t + col]);
  }
  // wall columns, rows 0..jtot+1
  if (t <= jtot + 1) {
    const int j = t;
    if (kind == 0) {
      put(ux_idx(1, j, ld), 0.);
      put(ux_idx(itot + 1, j, ld), 0.);
    } else if (kind == 1) {
      put(uy_idx(0, j, ld), w0);
      put(uy_idx(itot + 1, j, ld), w1);
    } else {
      // source row of the (already periodic) value: halo rows mirror rows jtot and 1
      const int js = j == 0 ? jtot : (j == jtot + 1 ? 1 : j);
      a[uy_idx(0, j, ld)] = a[uy_idx(1, js, ld)];
      a[uy_idx(itot + 1, j, ld)] = a[uy_idx(itot, js, ld)];
    }
  }
}

// ---------------------------------------------------------------------------
// RK predictor: explicit/implicit source terms and the velocity update fused,
// reading (ux, uy, p) and writing the other velocity buffer
// (src/fluid/update_velocity.c:9-237). Also writes the halo rows of the new
// velocities; wall columns of both buffers are constant and set at creation.
struct PredArgs {
  const double *ux, *uy, *p;
  const double *sxb, *syb;     // previous explicit terms (srcB)
  double *sxa, *sya;           // new explicit terms (srcA)
  double *uxn, *uyn;           // new velocities
  const double *rdxf, *rdxc, *cxm, *cxp, *cym, *cyp;
  const double *dt;
  double alpha, beta, gamma, rRe, rdy, ext;
  int itot, jtot, ld;
};

template <int TY>
__global__ void __launch_bounds__(TX *TY) k_predictor(PredArgs a) {
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  if (i > a.itot || j > a.jtot) return;
  const int ld = a.ld;
  const double dt = __ldg(a.dt);
  const double adt = a.alpha * dt, bdt = a.beta * dt, gdt = a.gamma * dt;
  const double rdy = a.rdy;
  // ---- ux at face i (2..itot) ----
  if (i >= 2) {
    const int c = ux_idx(i, j, ld);
    const double u0 = __ldg(a.ux + c);
    const double uw = __ldg(a.ux + c - 1), ue = __ldg(a.ux + c + 1);
    const double us = __ldg(a.ux + c - ld), un = __ldg(a.ux + c + ld);
    const double rdxf_m = __ldg(a.rdxf + i - 1), rdxf_p = __ldg(a.rdxf + i);
    const double cxm = __ldg(a.cxm + i), cxp = __ldg(a.cxp + i);
    const double duxdx_xm = (u0 - uw) * rdxf_m;
    const double duxdx_xp = (ue - u0) * rdxf_p;
    const double duxdy_ym = (u0 - us) * rdy;
    const double duxdy_yp = (un - u0) * rdy;
    const double ux_xm = 0.5 * uw + 0.5 * u0;
    const double ux_xp = 0.5 * u0 + 0.5 * ue;
    const double adv1 = -cxm * ux_xm * duxdx_xm - cxp * ux_xp * duxdx_xp;
    const int cy = uy_idx(i, j, ld);
    const double uy_ym = cxm * __ldg(a.uy + cy - 1) + cxp * __ldg(a.uy + cy);
    const double uy_yp = cxm * __ldg(a.uy + cy - 1 + ld) + cxp * __ldg(a.uy + cy + ld);
    const double adv2 = -0.5 * uy_ym * duxdy_ym - 0.5 * uy_yp * duxdy_yp;
    const double rdxc = __ldg(a.rdxc + i);
    const double dif1 = a.rRe * (duxdx_xp - duxdx_xm) * rdxc;
    const double dif2 = a.rRe * (duxdy_yp - duxdy_ym) * rdy;
    const double pre = -(__ldg(a.p + cy) - __ldg(a.p + cy - 1)) * rdxc;
    const double A = (adv1 + adv2) + (dif1 + dif2);
    const double B = __ldg(a.sxb + c);
    a.sxa[c] = A;
    const double un_ = u0 + (adt * A + bdt * B + gdt * pre);
    a.uxn[c] = un_;
    if (j == 1) a.uxn[c + a.jtot * ld] = un_;
    if (j == a.jtot) a.uxn[c - a.jtot * ld] = un_;
  }
  // ---- uy at cell i (1..itot) ----
  {
    const int c = uy_idx(i, j, ld);
    const double v0 = __ldg(a.uy + c);
    const double vw = __ldg(a.uy + c - 1), ve = __ldg(a.uy + c + 1);
    const double vs = __ldg(a.uy + c - ld), vn = __ldg(a.uy + c + ld);
    const double rdxc_m = __ldg(a.rdxc + i), rdxc_p = __ldg(a.rdxc + i + 1);
    const double duydx_xm = (v0 - vw) * rdxc_m;
    const double duydx_xp = (ve - v0) * rdxc_p;
    const double duydy_ym = (v0 - vs) * rdy;
    const double duydy_yp = (vn - v0) * rdy;
    const double cym = __ldg(a.cym + i), cyp = __ldg(a.cyp + i);
    const int cx = ux_idx(i, j, ld);
    const double ux_xm = 0.5 * __ldg(a.ux + cx - ld) + 0.5 * __ldg(a.ux + cx);
    const double ux_xp = 0.5 * __ldg(a.ux + cx + 1 - ld) + 0.5 * __ldg(a.ux + cx + 1);
    const double adv1 = -cym * ux_xm * duydx_xm - cyp * ux_xp * duydx_xp;
    const double uy_ym = 0.5 * vs + 0.5 * v0;
    const double uy_yp = 0.5 * v0 + 0.5 * vn;
    const double adv2 = -0.5 * uy_ym * duydy_ym - 0.5 * uy_yp * duydy_yp;
    const double dif1 = a.rRe * (duydx_xp - duydx_xm) * __ldg(a.rdxf + i);
    const double dif2 = a.rRe * (duydy_yp - duydy_ym) * rdy;
    const double pre = -(__ldg(a.p + c) - __ldg(a.p + c - ld)) * rdy;
    const double A = (adv1 + adv2) + (dif1 + dif2) + a.ext;
    const double B = __ldg(a.syb + c);
    a.sya[c] = A;
    const double vn_ = v0 + (adt * A + bdt * B + gdt * pre);
    a.uyn[c] = vn_;
    if (j == 1) a.uyn[c + a.jtot * ld] = vn_;
    if (j == a.jtot) a.uyn[c - a.jtot * ld] = vn_;
  }
}

// ---------------------------------------------------------------------------
// Mixed-precision predictor: the same update with the source terms computed in
// single precision. Each block stages a (TX+2) x (TY+2) tile of ux, uy and p in
// shared memory as unevaluated float pairs hi + lo, so that differences of
// neighbouring values keep their relative precision although the values
// themselves are O(1); one double subtraction per staged value, instead of one
// per stencil difference. The explicit terms are stored in float; the velocity
// update u + (alpha A + beta B + gamma G) dt is added in double precision.
struct PredArgsF {
  const double *ux, *uy, *p;
  const float *sxb, *syb;
  float *sxa, *sya;
  double *uxn, *uyn;
  float *uxfn, *uyfn;  // the new velocities rounded to float (eifd::d2f)
  const float *rdxf, *rdxc, *cxm, *cxp, *cym, *cyp;
  const float *coef;   // alpha dt, beta dt, gamma dt of this stage
  float rRe, rdy, ext;
  // uniform x metrics (kernels with UNI set): rdxf, rdxc, cxm = cxp, cym = cyp away
  // from the wall cells, bitwise the values of the arrays
  float u_rdxf, u_rdxc, u_cx, u_cy;
  int itot, jtot, ld;
};

__device__ __forceinline__ float dif(float2 a, float2 b) { return (a.x - b.x) + (a.y - b.y); }
__device__ __forceinline__ float val(float2 a) { return a.x + a.y; }

// the update of cell (i, j) of the mixed predictor from the staged float-pair tiles (the
// cell at tile position (x, y)); u_own, v_own are the cell's old velocities in double,
// Bx, By its old explicit terms. UNI: the x metrics are the uniform arguments except at
// the wall cells i = 1 (rdxc(1), cym(1)) and i = itot (rdxc(itot + 1), cyp(itot)), which
// are loaded; the values, and so the results, are those of the arrays.
template <int PY, int PX, bool UNI = false>
__device__ __forceinline__ void pred_mixed_cell(const PredArgsF &a, const float2 (&tux)[PY][PX],
                                                const float2 (&tuy)[PY][PX], const float2 (&tp)[PY][PX], int i, int j,
                                                int x, int y, double u_own, double v_own, float Bx, float By) {
  const int ld = a.ld, jtot = a.jtot;
  const float adt = __ldg(a.coef), bdt = __ldg(a.coef + 1), gdt = __ldg(a.coef + 2);
  const float rdy = a.rdy;
  if (i >= 2) {
    const float2 u0 = tux[y][x], uw = tux[y][x - 1], ue = tux[y][x + 1], us = tux[y - 1][x], un = tux[y + 1][x];
    const float cxm = UNI ? a.u_cx : __ldg(a.cxm + i), cxp = UNI ? a.u_cx : __ldg(a.cxp + i);
    const float rdxf_m = UNI ? a.u_rdxf : __ldg(a.rdxf + i - 1), rdxf_p = UNI ? a.u_rdxf : __ldg(a.rdxf + i);
    const float duxdx_xm = dif(u0, uw) * rdxf_m;
    const float duxdx_xp = dif(ue, u0) * rdxf_p;
    const float duxdy_ym = dif(u0, us) * rdy;
    const float duxdy_yp = dif(un, u0) * rdy;
    const float ux_xm = 0.5f * (val(uw) + val(u0));
    const float ux_xp = 0.5f * (val(u0) + val(ue));
    const float adv1 = -cxm * ux_xm * duxdx_xm - cxp * ux_xp * duxdx_xp;
    const float uy_ym = cxm * val(tuy[y][x - 1]) + cxp * val(tuy[y][x]);
    const float uy_yp = cxm * val(tuy[y + 1][x - 1]) + cxp * val(tuy[y + 1][x]);
    const float adv2 = -0.5f * uy_ym * duxdy_ym - 0.5f * uy_yp * duxdy_yp;
    const float rdxc = UNI ? a.u_rdxc : __ldg(a.rdxc + i);
    const float dif_ = a.rRe * ((dif(ue, u0) * rdxf_p - dif(u0, uw) * rdxf_m) * rdxc +
                                (dif(un, u0) - dif(u0, us)) * rdy * rdy);
    const float pre = -dif(tp[y][x], tp[y][x - 1]) * rdxc;
    const float A = (adv1 + adv2) + dif_;
    const int c = j * ld + (i - 1);
    a.sxa[c] = A;
    const double un_ = u_own + eifd::f2d(adt * A + bdt * Bx + gdt * pre);
    const float unf = eifd::d2f(un_);
    a.uxn[c] = un_;
    a.uxfn[c] = unf;
    if (j == 1) { a.uxn[c + jtot * ld] = un_; a.uxfn[c + jtot * ld] = unf; }
    if (j == jtot) { a.uxn[c - jtot * ld] = un_; a.uxfn[c - jtot * ld] = unf; }
  }
  {
    const float2 v0 = tuy[y][x], vw = tuy[y][x - 1], ve = tuy[y][x + 1], vs = tuy[y - 1][x], vn = tuy[y + 1][x];
    const bool wall_w = !UNI || i == 1, wall_e = !UNI || i == a.itot;
    const float rdxc_m = wall_w ? __ldg(a.rdxc + i) : a.u_rdxc;
    const float rdxc_p = wall_e ? __ldg(a.rdxc + i + 1) : a.u_rdxc;
    const float duydx_xm = dif(v0, vw) * rdxc_m;
    const float duydx_xp = dif(ve, v0) * rdxc_p;
    const float duydy_ym = dif(v0, vs) * rdy;
    const float duydy_yp = dif(vn, v0) * rdy;
    const float cym = wall_w ? __ldg(a.cym + i) : a.u_cy, cyp = wall_e ? __ldg(a.cyp + i) : a.u_cy;
    const float ux_xm = 0.5f * (val(tux[y - 1][x]) + val(tux[y][x]));
    const float ux_xp = 0.5f * (val(tux[y - 1][x + 1]) + val(tux[y][x + 1]));
    const float adv1 = -cym * ux_xm * duydx_xm - cyp * ux_xp * duydx_xp;
    const float uy_ym = 0.5f * (val(vs) + val(v0));
    const float uy_yp = 0.5f * (val(v0) + val(vn));
    const float adv2 = -0.5f * uy_ym * duydy_ym - 0.5f * uy_yp * duydy_yp;
    const float dif_ = a.rRe * ((duydx_xp - duydx_xm) * (UNI ? a.u_rdxf : __ldg(a.rdxf + i)) +
                                (duydy_yp - duydy_ym) * rdy);
    const float pre = -dif(tp[y][x], tp[y - 1][x]) * rdy;
    const float A = (adv1 + adv2) + dif_ + a.ext;
    const int c = j * ld + i;
    a.sya[c] = A;
    const double vn_ = v_own + eifd::f2d(adt * A + bdt * By + gdt * pre);
    const float vnf = eifd::d2f(vn_);
    a.uyn[c] = vn_;
    a.uyfn[c] = vnf;
    if (j == 1) { a.uyn[c + jtot * ld] = vn_; a.uyfn[c + jtot * ld] = vnf; }
    if (j == jtot) { a.uyn[c - jtot * ld] = vn_; a.uyfn[c - jtot * ld] = vnf; }
  }
}

template <int TY, bool UNI>
__global__ void __launch_bounds__(TX *TY) k_predictor_mixed(PredArgsF a) {
  constexpr int PX = TX + 2, PY = TY + 2;
  __shared__ float2 tux[PY][PX], tuy[PY][PX], tp[PY][PX];
  const int ld = a.ld, itot = a.itot, jtot = a.jtot;
  const int ib = 1 + blockIdx.x * TX, jb = 1 + blockIdx.y * TY;
  // stage the tile: tile (tx, ty) holds index (ib - 1 + tx, jb - 1 + ty). Every thread
  // stages its own cell (and keeps its two doubles for the update), the first threads
  // the ring of 2 (TX + 2) + 2 TY halo cells.
  auto stage = [&](int tx, int ty, double *u_keep, double *v_keep) {
    const int i = ib - 1 + tx, j = jb - 1 + ty;
    float2 vux = make_float2(0.f, 0.f), vuy = vux, vp = vux;
    if (j <= jtot + 1) {
      if (i >= 1 && i <= itot + 1) {
        const double u = __ldg(a.ux + j * ld + (i - 1));
        if (u_keep) *u_keep = u;
        vux = eifd::split(u);
      }
      if (i <= itot + 1) {
        const double v = __ldg(a.uy + j * ld + i);
        if (v_keep) *v_keep = v;
        vuy = eifd::split(v);
        vp = eifd::split(__ldg(a.p + j * ld + i));
      }
    }
    tux[ty][tx] = vux;
    tuy[ty][tx] = vuy;
    tp[ty][tx] = vp;
  };
  // the old explicit terms are streamed once and used after the barrier: their loads
  // are issued first, so that they are in flight together with the staging loads
  const int i = ib + threadIdx.x, j = jb + threadIdx.y;
  const bool live = i <= itot && j <= jtot;
  float Bx = 0.f, By = 0.f;
  if (live) {
    if (i >= 2) Bx = __ldg(a.sxb + j * ld + (i - 1));
    By = __ldg(a.syb + j * ld + i);
  }
  double u_own = 0., v_own = 0.;
  stage(threadIdx.x + 1, threadIdx.y + 1, &u_own, &v_own);
  {
    constexpr int RING = 2 * PX + 2 * TY;
    const int t = threadIdx.y * TX + threadIdx.x;
    if (t < RING) {
      int tx, ty;
      if (t < PX) { tx = t; ty = 0; }                              // bottom halo row
      else if (t < 2 * PX) { tx = t - PX; ty = PY - 1; }          // top halo row
      else if (t < 2 * PX + TY) { tx = 0; ty = 1 + (t - 2 * PX); } // left column
      else { tx = PX - 1; ty = 1 + (t - 2 * PX - TY); }            // right column
      stage(tx, ty, nullptr, nullptr);
    }
  }
  __syncthreads();
  if (!live) return;
  pred_mixed_cell<PY, PX, UNI>(a, tux, tuy, tp, i, j, threadIdx.x + 1, threadIdx.y + 1, u_own, v_own, Bx, By);
}

// ---------------------------------------------------------------------------
// The mixed predictor with its tiles staged by the tensor memory accelerator. A
// persistent grid walks the (32 x TY)-cell tiles; for each tile one thread issues three
// 2-D bulk tensor copies (ux, uy, p as doubles, with their one-cell halo) into one of two
// shared-memory stages, so that the copies of the next tile are in flight while a tile
// is computed; an mbarrier per stage counts the bytes in. The staged doubles are then
// split into the float-pair tiles of k_predictor_mixed and the cell update is that
// kernel's (pred_mixed_cell): the results are identical. Tensor coordinates: the ux box
// starts at column 32 bx - 2 (UX(32 bx - 1) sits at column 32 bx - 2; an even column
// keeps the copy on a 16-byte boundary), the uy and p boxes at column 32 bx; rows from
// TY by (the halo row below the tile). Cells outside the tensor are filled with zeros,
// as k_predictor_mixed stages them; the padding columns of the fields are zero.
constexpr int TMA_BWX = 36, TMA_BWY = 34;   // box columns (doubles): ux, and uy / p
__host__ __device__ constexpr int round128(int v) { return (v + 127) & ~127; }
template <int TY> struct TmaLayout {
  static constexpr int PY = TY + 2;
  static constexpr int UX = 0;
  static constexpr int UY = round128(TMA_BWX * PY * 8);
  static constexpr int P = UY + round128(TMA_BWY * PY * 8);
  static constexpr int STAGE = P + round128(TMA_BWY * PY * 8);
  static constexpr unsigned BYTES = (TMA_BWX + 2 * TMA_BWY) * PY * 8;   // expected per stage
  static constexpr int SMEM = 2 * STAGE + 128;                          // + alignment slack
};

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// bounded wait for the phase of the given parity: false when it did not complete
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
  const unsigned addr = smem_u32(bar);
  for (int it = 0; it < (1 << 22); it++) {
    unsigned done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done) : "r"(addr), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
               ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
               : "memory");
}

template <int TY>
__global__ void __launch_bounds__(TX *TY) k_predictor_tma(const __grid_constant__ CUtensorMap mux,
                                                          const __grid_constant__ CUtensorMap muy,
                                                          const __grid_constant__ CUtensorMap mp, PredArgsF a, int nbx,
                                                          int ntiles, unsigned *flags) {
  using L = TmaLayout<TY>;
  constexpr int PX = TX + 2, PY = TY + 2;
  extern __shared__ unsigned char smem_dyn[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_dyn) + 127) & ~uintptr_t(127));
  __shared__ float2 tux[PY][PX], tuy[PY][PX], tp[PY][PX];
  __shared__ uint64_t bar[2];
  const int tid = threadIdx.y * TX + threadIdx.x;
  const int ld = a.ld;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int tile, int s) {
    const int bx = tile % nbx, by = tile / nbx;
    unsigned char *st = base + s * L::STAGE;
    mbar_expect_tx(&bar[s], L::BYTES);
    tma_load_2d(st + L::UX, &mux, TX * bx - 2, TY * by, &bar[s]);
    tma_load_2d(st + L::UY, &muy, TX * bx, TY * by, &bar[s]);
    tma_load_2d(st + L::P, &mp, TX * bx, TY * by, &bar[s]);
  };
  const int g = gridDim.x;
  if (tid == 0) {
    if ((int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
    if ((int)blockIdx.x + g < ntiles) issue(blockIdx.x + g, 1);
  }
  int n = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += g, n++) {
    const int s = n & 1;
    const int bx = tile % nbx, by = tile / nbx;
    const int i = 1 + TX * bx + threadIdx.x, j = 1 + TY * by + threadIdx.y;
    const bool live = i <= a.itot && j <= a.jtot;
    // the old explicit terms are streamed once: their loads go first
    float Bx = 0.f, By = 0.f;
    if (live) {
      if (i >= 2) Bx = __ldg(a.sxb + j * ld + (i - 1));
      By = __ldg(a.syb + j * ld + i);
    }
    const bool ok = mbar_wait(&bar[s], (n >> 1) & 1);
    if (__syncthreads_or(!ok)) {
      // a copy did not arrive: report it, wait (bounded) for the copies still in flight
      // into this block's shared memory, and stop
      if (tid == 0) {
        atomicOr(flags, EIF_FLAG_TIMEOUT);
        mbar_wait(&bar[s], (n >> 1) & 1);
        if (tile + g < ntiles) mbar_wait(&bar[s ^ 1], ((n + 1) >> 1) & 1);
      }
      return;
    }
    const unsigned char *st = base + s * L::STAGE;
    const double *rux = reinterpret_cast<const double *>(st + L::UX);
    const double *ruy = reinterpret_cast<const double *>(st + L::UY);
    const double *rp = reinterpret_cast<const double *>(st + L::P);
    // tile (tx, ty) holds index (ib - 1 + tx, jb - 1 + ty): ux column tx + 1, uy and p column tx
    for (int q = tid; q < PY * PX; q += TX * TY) {
      const int ty = q / PX, tx = q - ty * PX;
      tux[ty][tx] = eifd::split(rux[ty * TMA_BWX + tx + 1]);
      tuy[ty][tx] = eifd::split(ruy[ty * TMA_BWY + tx]);
      tp[ty][tx] = eifd::split(rp[ty * TMA_BWY + tx]);
    }
    const double u_own = rux[(threadIdx.y + 1) * TMA_BWX + threadIdx.x + 2];
    const double v_own = ruy[(threadIdx.y + 1) * TMA_BWY + threadIdx.x + 1];
    __syncthreads();
    // the stage is consumed: the copies of the tile after next go into it
    if (tid == 0 && tile + 2 * g < ntiles) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(tile + 2 * g, s);
    }
    if (live) pred_mixed_cell(a, tux, tuy, tp, i, j, threadIdx.x + 1, threadIdx.y + 1, u_own, v_own, Bx, By);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Projection (src/fluid/correct_velocity.c:6-42), optionally preceded by the
// IBM field response (src/suspensions/update.c:36-59) and followed by the
// pressure update (src/fluid/update_pressure.c:7-24), in one pass. The IBM
// response and the projection are applied as two separately rounded updates,
// as the reference applies them in two functions.
struct CorrArgs {
  double *ux, *uy, *p;
  const double *psi, *dux, *duy, *rdxc, *dt;
  double gamma, rdy;
  int itot, jtot, ld, with_ibm, with_proj, with_pressure;
};

template <int TY>
__global__ void __launch_bounds__(TX *TY) k_correct(CorrArgs a) {
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  if (i > a.itot || j > a.jtot) return;
  const int ld = a.ld, jtot = a.jtot, itot = a.itot;
  const double gdt = a.with_proj ? a.gamma * __ldg(a.dt) : 0.;
  const int cy = uy_idx(i, j, ld);
  const double psi0 = (a.with_proj || a.with_pressure) ? __ldg(a.psi + cy) : 0.;
  const bool vel = a.with_ibm || a.with_proj;
  if (vel && i >= 2) {
    const int c = ux_idx(i, j, ld);
    double u = a.ux[c];
    if (a.with_ibm) u = u + 0.5 * (__ldg(a.dux + cy - 1) + __ldg(a.dux + cy));
    if (a.with_proj) u = u - gdt * (psi0 - __ldg(a.psi + cy - 1)) * __ldg(a.rdxc + i);
    a.ux[c] = u;
    if (j == 1) a.ux[c + jtot * ld] = u;
    if (j == jtot) a.ux[c - jtot * ld] = u;
  }
  if (vel) {
    double v = a.uy[cy];
    if (a.with_ibm) v = v + 0.5 * (__ldg(a.duy + cy - ld) + __ldg(a.duy + cy));
    if (a.with_proj) v = v - gdt * (psi0 - __ldg(a.psi + cy - ld)) * a.rdy;
    a.uy[cy] = v;
    if (j == 1) a.uy[cy + jtot * ld] = v;
    if (j == jtot) a.uy[cy - jtot * ld] = v;
  }
  if (a.with_pressure) {
    const double pv = a.p[cy] + psi0;
    a.p[cy] = pv;
    // periodic halo rows and Neumann wall copies (boundary_conditions.c:45-62)
    if (j == 1) a.p[cy + jtot * ld] = pv;
    if (j == jtot) a.p[cy - jtot * ld] = pv;
    if (i == 1) {
      a.p[cy - 1] = pv;
      if (j == 1) a.p[cy - 1 + jtot * ld] = pv;
      if (j == jtot) a.p[cy - 1 - jtot * ld] = pv;
    }
    if (i == itot) {
      a.p[cy + 1] = pv;
      if (j == 1) a.p[cy + 1 + jtot * ld] = pv;
      if (j == jtot) a.p[cy + 1 - jtot * ld] = pv;
    }
  }
}

// Mixed-precision projection. The FP64 pipe is used only where the result must
// keep double precision: the differences of psi (exact for neighbouring values),
// the rounding of the double-float increment to a double, and the final sums.
// The products gamma dt (psi_i - psi_{i-1}) / dxc and the IBM response (single-
// precision field values, summed exactly) are formed in double-float arithmetic.
struct CorrArgsDF {
  double *ux, *uy, *p;
  float *uxf, *uyf;         // the velocities rounded to float (eifd::d2f), kept with ux, uy
  const double *psi;
  // psi as the float pair psi1 + psi2 of the refined solve (psi1 at psi, psi2 at
  // psi1 + psi2_off floats), or null: psi in double
  const float *psi1;
  size_t psi2_off;
  const float *dux, *duy;   // IBM field response in single precision
  const float2 *rdxc;       // 1/dxc as (hi, lo)
  const float *coef;        // [20 + 2 rk], [21 + 2 rk]: gamma dt
  eifdf::DF rdy;
  int rk, itot, jtot, ld, with_ibm, with_proj, with_pressure;
};

// capped for 12 resident CTAs of 32 x 4 threads per SM (39 registers, no spills):
// measured 9 % faster than the uncapped 52 registers (9 CTAs)
template <int TY>
__global__ void __launch_bounds__(TX *TY, 48 / TY) k_correct_df(CorrArgsDF a) {
  using namespace eifdf;
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  if (i > a.itot || j > a.jtot) return;
  const int ld = a.ld, jtot = a.jtot, itot = a.itot;
  const int cy = uy_idx(i, j, ld), c = ux_idx(i, j, ld);
  const bool vel = a.with_ibm || a.with_proj;
  const bool xface = vel && i >= 2;
  // Every load is issued before the first store: a thread reads only its own cells
  // and the read-only psi and responses, and writes only its own cells and halo copies
  // that no thread of this launch reads, so the order does not change a result, but
  // the three old values then come from memory together instead of one after another.
  const double u_old = xface ? a.ux[c] : 0.;
  const double v_old = vel ? a.uy[cy] : 0.;
  const double p_old = a.with_pressure ? a.p[cy] : 0.;
  // psi at the cell and its west and south neighbours: doubles, or float pairs
  double psi0 = 0., psi_w = 0., psi_s = 0.;
  DF q0{0.f, 0.f}, qw{0.f, 0.f}, qs{0.f, 0.f};
  const bool need0 = a.with_proj || a.with_pressure, needw = a.with_proj && xface, needs = a.with_proj && vel;
  if (a.psi1) {
    const float *p2 = a.psi1 + a.psi2_off;
    if (need0) q0 = DF{__ldg(a.psi1 + cy), __ldg(p2 + cy)};
    if (needw) qw = DF{__ldg(a.psi1 + cy - 1), __ldg(p2 + cy - 1)};
    if (needs) qs = DF{__ldg(a.psi1 + cy - ld), __ldg(p2 + cy - ld)};
  } else {
    if (need0) psi0 = __ldg(a.psi + cy);
    if (needw) psi_w = __ldg(a.psi + cy - 1);
    if (needs) psi_s = __ldg(a.psi + cy - ld);
  }
  // psi_0 - psi_nb as a double-float: exact double differences, or the difference of
  // two float pairs (an exact difference of the leading parts)
  auto dpsi = [&](double pnb, DF qnb) -> DF {
    if (a.psi1) {
      const DF s = two_sum(q0.hi, -qnb.hi);
      return fast_sum(s.hi, s.lo + (q0.lo - qnb.lo));
    }
    return df_of(psi0 - pnb);
  };
  float dw = 0.f, de = 0.f, ds = 0.f, dn = 0.f;
  if (a.with_ibm) {
    if (xface) { dw = __ldg(a.dux + cy - 1); de = __ldg(a.dux + cy); }
    ds = __ldg(a.duy + cy - ld);
    dn = __ldg(a.duy + cy);
  }
  const float2 r = xface ? __ldg(a.rdxc + i) : make_float2(0.f, 0.f);
  const DF gdt = a.with_proj ? DF{__ldg(a.coef + 20 + 2 * a.rk), __ldg(a.coef + 21 + 2 * a.rk)} : DF{0.f, 0.f};
  if (xface) {
    DF inc{0.f, 0.f};
    if (a.with_ibm) inc = two_sum(dw, de);
    inc = df_scale(inc, 0.5f);
    if (a.with_proj) {
      const DF g = df_mul(df_mul(gdt, dpsi(psi_w, qw)), DF{r.x, r.y});
      inc = df_add_nw(inc, df_neg(g));
    }
    const double u = u_old + df_to_double(inc);
    const float uf = eifd::d2f(u);
    a.ux[c] = u;
    a.uxf[c] = uf;
    if (j == 1) { a.ux[c + jtot * ld] = u; a.uxf[c + jtot * ld] = uf; }
    if (j == jtot) { a.ux[c - jtot * ld] = u; a.uxf[c - jtot * ld] = uf; }
  }
  if (vel) {
    DF inc{0.f, 0.f};
    if (a.with_ibm) inc = two_sum(ds, dn);
    inc = df_scale(inc, 0.5f);
    if (a.with_proj) {
      const DF g = df_mul(df_mul(gdt, dpsi(psi_s, qs)), a.rdy);
      inc = df_add_nw(inc, df_neg(g));
    }
    const double v = v_old + df_to_double(inc);
    const float vf = eifd::d2f(v);
    a.uy[cy] = v;
    a.uyf[cy] = vf;
    if (j == 1) { a.uy[cy + jtot * ld] = v; a.uyf[cy + jtot * ld] = vf; }
    if (j == jtot) { a.uy[cy - jtot * ld] = v; a.uyf[cy - jtot * ld] = vf; }
  }
  if (a.with_pressure) {
    // psi1 + psi2 as a double without the FP64 pipe (bit-identical to the FP64 addition;
    // the pipe is the kernel's bound)
    const double pv = p_old + (a.psi1 ? eifd::pair_to_double(q0.hi, q0.lo) : psi0);
    a.p[cy] = pv;
    if (j == 1) a.p[cy + jtot * ld] = pv;
    if (j == jtot) a.p[cy - jtot * ld] = pv;
    if (i == 1) {
      a.p[cy - 1] = pv;
      if (j == 1) a.p[cy - 1 + jtot * ld] = pv;
      if (j == jtot) a.p[cy - 1 - jtot * ld] = pv;
    }
    if (i == itot) {
      a.p[cy + 1] = pv;
      if (j == 1) a.p[cy + 1 + jtot * ld] = pv;
      if (j == jtot) a.p[cy + 1 - jtot * ld] = pv;
    }
  }
}

// ---------------------------------------------------------------------------
// dt: column maxima of |ux| and the global maximum of |uy| as order-preserving
// integer maxima of the IEEE bit patterns (non-negative doubles order like
// their bits), so the result is independent of the reduction order.
constexpr int CM_THREADS = 256;   // column pairs per block: 8 KB of a row per block and row
__global__ void __launch_bounds__(CM_THREADS) k_dt_colmax(const double *__restrict__ ux, const double *__restrict__ uy,
                                                          int itot, int jtot, int ld,
                                                          unsigned long long *__restrict__ colmax,
                                                          unsigned long long *__restrict__ uymax,
                                                          unsigned *__restrict__ flags) {
  // each thread owns the pair of row entries 2p, 2p + 1 (16-byte loads; rows start on
  // 256-byte boundaries) over the rows blockIdx.y + 1, + gridDim.y, ...: ux entry k is
  // UX(k + 1), counted for 2 <= k + 1 <= itot; uy entry k is UY(k), for 1 <= k <= itot
  const int p = blockIdx.x * CM_THREADS + threadIdx.x;
  const int k0 = 2 * p;
  unsigned long long mx0 = 0ull, mx1 = 0ull, my = 0ull;
  bool bad = false;
  if (k0 <= itot) {
    const bool x0 = k0 >= 1 && k0 <= itot - 1, x1 = k0 + 1 <= itot - 1;
    const bool y0 = k0 >= 1, y1 = k0 + 1 <= itot;
#pragma unroll 4
    for (int j = 1 + blockIdx.y; j <= jtot; j += gridDim.y) {
      const double2 u = __ldg(reinterpret_cast<const double2 *>(ux + (size_t)j * ld) + p);
      const double2 v = __ldg(reinterpret_cast<const double2 *>(uy + (size_t)j * ld) + p);
      const unsigned long long bu0 = __double_as_longlong(u.x) & 0x7fffffffffffffffull;
      const unsigned long long bu1 = __double_as_longlong(u.y) & 0x7fffffffffffffffull;
      const unsigned long long bv0 = y0 ? __double_as_longlong(v.x) & 0x7fffffffffffffffull : 0ull;
      const unsigned long long bv1 = y1 ? __double_as_longlong(v.y) & 0x7fffffffffffffffull : 0ull;
      if (x0) mx0 = bu0 > mx0 ? bu0 : mx0;
      if (x1) mx1 = bu1 > mx1 ? bu1 : mx1;
      const unsigned long long bv = bv0 > bv1 ? bv0 : bv1;
      my = bv > my ? bv : my;
      bad |= (x0 && bu0 >= 0x7ff0000000000000ull) || (x1 && bu1 >= 0x7ff0000000000000ull) ||
             bv >= 0x7ff0000000000000ull;
    }
  }
  // maximum of uy over the block: warp reduce then one atomic per warp
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, my, o);
    my = other > my ? other : my;
  }
  if ((threadIdx.x & 31) == 0 && my) atomicMax(uymax, my);
  if (bad) atomicOr(flags, EIF_FLAG_NONFINITE);
  if (mx0) atomicMax(colmax + k0 + 1, mx0);
  if (mx1) atomicMax(colmax + k0 + 2, mx1);
}

// single-precision products of dt used by the mixed-precision kernels, formed
// once per time step instead of once per thread
__device__ __forceinline__ void write_coef(double dt, float *coef) {
  const double al[3] = {32. / 60., 25. / 60., 45. / 60.};
  const double be[3] = {0. / 60., -17. / 60., -25. / 60.};
  for (int rk = 0; rk < 3; rk++) {
    coef[3 * rk + 0] = (float)(al[rk] * dt);
    coef[3 * rk + 1] = (float)(be[rk] * dt);
    coef[3 * rk + 2] = (float)((al[rk] + be[rk]) * dt);
  }
  coef[9] = (float)(1. / dt);
  for (int rk = 0; rk < 3; rk++) {
    const double gdt = (al[rk] + be[rk]) * dt;
    const float hi = (float)gdt;
    coef[20 + 2 * rk] = hi;
    coef[21 + 2 * rk] = (float)(gdt - (double)hi);
  }
  for (int rk = 0; rk < 3; rk++) {
    const double inv = 1. / ((al[rk] + be[rk]) * dt);
    const float hi = (float)inv;
    coef[12 + 2 * rk] = hi;
    coef[13 + 2 * rk] = (float)(inv - (double)hi);
  }
}

// dt from the maxima (decide_dt.c:25-80): one block.
// dt limits of one slice of columns and particles (partial minima, one triple per
// block), then the final combination: the divisions are spread over DT_BLOCKS SMs
constexpr int DT_BLOCKS = 32;

__global__ void k_dt_partial(const unsigned long long *__restrict__ colmax, const unsigned long long *__restrict__ uymax,
                             const double *__restrict__ dxc, int itot, double dy, double lx, double dx_uniform,
                             const double *__restrict__ P, int pcap, int np, double *__restrict__ part) {
  const double small = 1.e-8;
  double dta = 5.e-2, dxmin = lx, dtp = DBL_MAX;
  const int stride = gridDim.x * blockDim.x;
  for (int i = 2 + blockIdx.x * blockDim.x + threadIdx.x; i <= itot; i += stride) {
    const double vel = fmax(__longlong_as_double((long long)colmax[i]), small);
    dta = fmin(dta, dxc[i] / vel);
    dxmin = fmin(dxmin, dxc[i]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double vel = fmax(__longlong_as_double((long long)uymax[0]), small);
    dta = fmin(dta, dy / vel);
  }
  const double delta = fmin(dx_uniform, dy);
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < np; n += stride) {
    const double a = P[EIF_P_A * pcap + n], b = P[EIF_P_B * pcap + n];
    const double r = fmax(a, b);
    const double vz = P[EIF_P_VZ * pcap + n];
    const double pux = fmax(fabs(P[EIF_P_UX * pcap + n]) + fabs(r * vz), small);
    const double puy = fmax(fabs(P[EIF_P_UY * pcap + n]) + fabs(r * vz), small);
    dtp = fmin(dtp, delta / fmax(pux, puy));
  }
  __shared__ double s[3][32];
  for (int o = 16; o > 0; o >>= 1) {
    dta = fmin(dta, __shfl_xor_sync(0xffffffffu, dta, o));
    dxmin = fmin(dxmin, __shfl_xor_sync(0xffffffffu, dxmin, o));
    dtp = fmin(dtp, __shfl_xor_sync(0xffffffffu, dtp, o));
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { s[0][w] = dta; s[1][w] = dxmin; s[2][w] = dtp; }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int k = 1; k < nw; k++) { dta = fmin(dta, s[0][k]); dxmin = fmin(dxmin, s[1][k]); dtp = fmin(dtp, s[2][k]); }
    part[3 * blockIdx.x + 0] = dta;
    part[3 * blockIdx.x + 1] = dxmin;
    part[3 * blockIdx.x + 2] = dtp;
  }
}

// param_decide_dt (decide_dt.c:11-81): minima of the partial limits, the safety
// factors, dt and the single-precision dt products
// one warp: every lane loads one block's partial limits (nparts <= 32), a shuffle
// reduction forms the minima (exact, so independent of the order)
__global__ void k_dt_final(const double *__restrict__ part, int nparts, double dy, double Re, double sf_adv,
                           double sf_dif, double sf_par, double *__restrict__ dt_out, float *__restrict__ coef) {
  const int l = threadIdx.x;
  const int q = l < nparts ? l : 0;
  double dta = part[3 * q], dxmin = part[3 * q + 1], dtp = part[3 * q + 2];
  for (int o = 16; o > 0; o >>= 1) {
    dta = fmin(dta, __shfl_xor_sync(0xffffffffu, dta, o));
    dxmin = fmin(dxmin, __shfl_xor_sync(0xffffffffu, dxmin, o));
    dtp = fmin(dtp, __shfl_xor_sync(0xffffffffu, dtp, o));
  }
  if (l != 0) return;
  dta *= sf_adv;
  double difx = 0.25 * Re * (dxmin * dxmin);
  double dify = 0.25 * Re * (dy * dy);
  difx *= sf_dif;
  dify *= sf_dif;
  dtp *= sf_par;
  const double dt = fmin(fmin(dta, fmin(difx, dify)), dtp);
  *dt_out = dt;
  write_coef(dt, coef);
}

__global__ void k_coef(const double *__restrict__ dt, float *__restrict__ coef) { write_coef(*dt, coef); }

// ---------------------------------------------------------------------------
// check_divergence (logging.c:52-65): (UX(i+1) - UX(i)) / DXF(i) + (UY(j+1) - UY(j)) / dy
__global__ void k_divergence(const double *__restrict__ ux, const double *__restrict__ uy, const double *__restrict__ dxf,
                             double dy, int itot, int jtot, int ld, double *__restrict__ out /* per block: max, sum */) {
  double mx = 0., sm = 0.;
  const int n = itot * jtot;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int i = 1 + t % itot, j = 1 + t / itot;
    const double d = (ux[ux_idx(i + 1, j, ld)] - ux[ux_idx(i, j, ld)]) / dxf[i] +
                     (uy[uy_idx(i, j + 1, ld)] - uy[uy_idx(i, j, ld)]) / dy;
    mx = fmax(mx, fabs(d));
    sm += d;
  }
  mx = eifd::warp_max(mx);
  sm = eifd::warp_sum(sm);
  __shared__ double s[2][32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { s[0][w] = mx; s[1][w] = sm; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); k++) { mx = fmax(mx, s[0][k]); sm += s[1][k]; }
    out[2 * blockIdx.x] = mx;
    out[2 * blockIdx.x + 1] = sm;
  }
}

// Sums of the logging diagnostics (logging.c:87-172) over the interior rows: x momentum
// and energy over the faces i = 1..itot+1 with the cell size DXC(i) dy, y momentum and
// energy over the cells i = 1..itot with DXF(i) dy. One partial sum of each per block,
// in a fixed grid-stride order; the host adds the partials in block order.
constexpr int FS_BLOCKS = 296, FS_THREADS = 256;
__global__ void __launch_bounds__(FS_THREADS) k_field_sums(const double *__restrict__ ux,
                                                          const double *__restrict__ uy,
                                                          const double *__restrict__ dxc,
                                                          const double *__restrict__ dxf, double dy, int itot,
                                                          int jtot, int ld, double *__restrict__ out) {
  double s[4] = {0., 0., 0., 0.};
  const long long nx = (long long)(itot + 1) * jtot, ny = (long long)itot * jtot;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nx; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % (itot + 1)), j = 1 + (int)(t / (itot + 1));
    const double u = ux[ux_idx(i, j, ld)];
    const double cs = dxc[i] * dy;
    s[0] += u * cs;
    s[2] += 0.5 * (u * u) * cs;
  }
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ny; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % itot), j = 1 + (int)(t / itot);
    const double v = uy[uy_idx(i, j, ld)];
    const double cs = dxf[i] * dy;
    s[1] += v * cs;
    s[3] += 0.5 * (v * v) * cs;
  }
  __shared__ double sh[4][FS_THREADS / 32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const double v = eifd::warp_sum(s[k]);
    if (l == 0) sh[k][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double v = 0.;
    for (int q = 0; q < FS_THREADS / 32; q++) v += sh[threadIdx.x][q];
    out[4 * blockIdx.x + threadIdx.x] = v;
  }
}

}  // namespace

namespace eif {

int launch_field_sums(eif_ctx *c, double *q) {
  double *part = c->qhat;  // scratch: 4 per block
  EIF_PROF(c, "field_sums", 1);
  k_field_sums<<<FS_BLOCKS, FS_THREADS, 0, c->stream>>>(c->ux[c->cur], c->uy[c->cur], c->dxc, c->dxf, c->dy, c->itot,
                                                        c->jtot, c->ld, part);
  EIF_LAUNCH_CK(c);
  double h[4 * FS_BLOCKS];
  EIF_CK(c, cudaMemcpyAsync(h, part, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 4; k++) {
    double v = 0.;
    for (int b = 0; b < FS_BLOCKS; b++) v += h[4 * b + k];
    q[k] = v;
  }
  return EIF_OK;
}

RK rk_coef(int rk) {
  // src/param/init.c:177-189
  static const double al[3] = {32. / 60., 25. / 60., 45. / 60.};
  static const double be[3] = {0. / 60., -17. / 60., -25. / 60.};
  return RK{al[rk], be[rk], al[rk] + be[rk]};
}

static dim3 cell_grid(const eif_ctx *c, int ty) {
  return dim3((c->itot + TX - 1) / TX, (c->jtot + ty - 1) / ty);
}

// launch of a stencil kernel with the tile height chosen by the tuner (4, 8 or 16 rows)
template <typename Args>
static void launch_tiled(void (*k4)(Args), void (*k8)(Args), void (*k16)(Args), int ty, eif_ctx *c, const Args &a) {
  if (ty == 4) {
    k4<<<cell_grid(c, 4), dim3(TX, 4), 0, c->stream>>>(a);
  } else if (ty == 16) {
    k16<<<cell_grid(c, 16), dim3(TX, 16), 0, c->stream>>>(a);
  } else {
    k8<<<cell_grid(c, 8), dim3(TX, 8), 0, c->stream>>>(a);
  }
}

// out[t] = eifd::d2f(in[t]): the rounding the single-precision kernels apply to the doubles
__global__ void k_round_to_float(const double *__restrict__ in, float *__restrict__ out, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    out[t] = eifd::d2f(in[t]);
}
int launch_round_to_float(eif_ctx *c, const double *in, float *out, size_t n) {
  k_round_to_float<<<c->sms * 4, 256, 0, c->stream>>>(in, out, n);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

int launch_bc_p_like(eif_ctx *c, double *a) {
  EIF_PROF(c, "boundaries", 1);
  const int n = (c->itot > c->jtot ? c->itot : c->jtot) + 2;
  k_bc<<<(n + 255) / 256, 256, 0, c->stream>>>(a, nullptr, 2, c->itot, c->jtot, c->ld, 0., 0.);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

int launch_boundaries(eif_ctx *c) {
  EIF_PROF(c, "boundaries", 5);
  const int n = (c->itot > c->jtot ? c->itot : c->jtot) + 2;
  for (int b = 0; b < 2; b++) {
    k_bc<<<(n + 255) / 256, 256, 0, c->stream>>>(c->ux[b], c->uxf[b], 0, c->itot, c->jtot, c->ld, 0., 0.);
    k_bc<<<(n + 255) / 256, 256, 0, c->stream>>>(c->uy[b], c->uyf[b], 1, c->itot, c->jtot, c->ld,
                                                 c->cfg.uy_wall[0], c->cfg.uy_wall[1]);
  }
  k_bc<<<(n + 255) / 256, 256, 0, c->stream>>>(c->p, nullptr, 2, c->itot, c->jtot, c->ld, 0., 0.);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to the driver library)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
  }
  return fn;
}

// 2-D map of a double field (ld columns, jtot + 2 rows) with boxes of w x h values
static bool field_map(CUtensorMap *m, const double *field, const eif_ctx *c, int w, int h) {
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)c->ld, (cuuint64_t)(c->jtot + 2)};
  const cuuint64_t strides[1] = {(cuuint64_t)c->ld * sizeof(double)};
  const cuuint32_t box[2] = {(cuuint32_t)w, (cuuint32_t)h};
  const cuuint32_t es[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double *>(field), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// launches the tensor-copy predictor of tile height TY; false when it cannot run
template <int TY>
static bool launch_predictor_tma(eif_ctx *c, const PredArgsF &a, int per_sm) {
  using L = TmaLayout<TY>;
  alignas(64) CUtensorMap mux, muy, mp;
  if (!field_map(&mux, a.ux, c, TMA_BWX, TY + 2) || !field_map(&muy, a.uy, c, TMA_BWY, TY + 2) ||
      !field_map(&mp, a.p, c, TMA_BWY, TY + 2))
    return false;
  const int nbx = (c->itot + TX - 1) / TX, nby = (c->jtot + TY - 1) / TY;
  const int ntiles = nbx * nby;
  const int grid = std::min(ntiles, c->sms * per_sm);
  k_predictor_tma<TY><<<grid, dim3(TX, TY), L::SMEM, c->stream>>>(mux, muy, mp, a, nbx, ntiles, c->d_flags);
  return true;
}

int predictor_prepare(eif_ctx *c) {
  if (c->cfg.precision != EIF_PREC_MIXED || getenv("EIF_NO_TMA") || !tensor_map_encoder()) return EIF_OK;
  int v = 0;
  EIF_CK(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_predictor_tma<4>, TX * 4, TmaLayout<4>::SMEM));
  c->pred_tma_ctas[0] = v;
  EIF_CK(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_predictor_tma<8>, TX * 8, TmaLayout<8>::SMEM));
  c->pred_tma_ctas[1] = v;
  EIF_CK(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_predictor_tma<16>, TX * 16, TmaLayout<16>::SMEM));
  c->pred_tma_ctas[2] = v;
  return EIF_OK;
}

static int launch_predictor_mixed(eif_ctx *c, int rk) {
  const RK k = rk_coef(rk);
  PredArgsF a;
  a.ux = c->ux[c->cur];
  a.uy = c->uy[c->cur];
  a.p = c->p;
  a.sxb = c->sxf[1 - c->scur];
  a.syb = c->syf[1 - c->scur];
  a.sxa = c->sxf[c->scur];
  a.sya = c->syf[c->scur];
  a.uxn = c->ux[1 - c->cur];
  a.uyn = c->uy[1 - c->cur];
  a.uxfn = c->uxf[1 - c->cur];
  a.uyfn = c->uyf[1 - c->cur];
  a.rdxf = c->rdxf_f; a.rdxc = c->rdxc_f;
  a.cxm = c->cxm_f; a.cxp = c->cxp_f; a.cym = c->cym_f; a.cyp = c->cyp_f;
  (void)k;
  a.coef = c->d_coef + 3 * rk;
  a.rRe = (float)(1. / c->cfg.Re);
  a.rdy = (float)(1. / c->dy);
  a.ext = (float)c->cfg.extfrcy;
  a.u_rdxf = c->uni_x.rdxf; a.u_rdxc = c->uni_x.rdxc; a.u_cx = c->uni_x.cx; a.u_cy = c->uni_x.cy;
  a.itot = c->itot; a.jtot = c->jtot; a.ld = c->ld;
  EIF_PROF(c, "predictor", 1);
  const int ty = c->tiles.pred;
  const int slot = ty == 4 ? 0 : (ty == 16 ? 2 : 1);
  bool done = false;
  if (c->tiles.pred_copy && c->pred_tma_ctas[slot] > 0) {
    if (ty == 4) done = launch_predictor_tma<4>(c, a, c->pred_tma_ctas[0]);
    else if (ty == 16) done = launch_predictor_tma<16>(c, a, c->pred_tma_ctas[2]);
    else done = launch_predictor_tma<8>(c, a, c->pred_tma_ctas[1]);
  }
  if (!done && c->uni_x.on)
    launch_tiled(k_predictor_mixed<4, true>, k_predictor_mixed<8, true>, k_predictor_mixed<16, true>, ty, c, a);
  else if (!done)
    launch_tiled(k_predictor_mixed<4, false>, k_predictor_mixed<8, false>, k_predictor_mixed<16, false>, ty, c, a);
  EIF_LAUNCH_CK(c);
  c->cur = 1 - c->cur;
  return EIF_OK;
}

int launch_predictor(eif_ctx *c, int rk) {
  const RK k = rk_coef(rk);
  // the explicit term of the previous stage becomes srcB (update_velocity.c:26,110)
  c->scur = 1 - c->scur;
  if (c->cfg.precision == EIF_PREC_MIXED) return launch_predictor_mixed(c, rk);
  PredArgs a;
  a.ux = c->ux[c->cur];
  a.uy = c->uy[c->cur];
  a.p = c->p;
  a.sxb = c->sxa[1 - c->scur];
  a.syb = c->sya[1 - c->scur];
  a.sxa = c->sxa[c->scur];
  a.sya = c->sya[c->scur];
  a.uxn = c->ux[1 - c->cur];
  a.uyn = c->uy[1 - c->cur];
  a.rdxf = c->rdxf; a.rdxc = c->rdxc;
  a.cxm = c->cxm; a.cxp = c->cxp; a.cym = c->cym; a.cyp = c->cyp;
  a.dt = c->d_scal;
  a.alpha = k.alpha; a.beta = k.beta; a.gamma = k.gamma;
  a.rRe = 1. / c->cfg.Re;
  a.rdy = 1. / c->dy;
  a.ext = c->cfg.extfrcy;
  a.itot = c->itot; a.jtot = c->jtot; a.ld = c->ld;
  EIF_PROF(c, "predictor", 1);
  launch_tiled(k_predictor<4>, k_predictor<8>, k_predictor<16>, c->tiles.pred, c, a);
  EIF_LAUNCH_CK(c);
  c->cur = 1 - c->cur;
  return EIF_OK;
}

static int launch_corr(eif_ctx *c, int rk, int with_ibm, int with_proj, int with_pressure) {
  if (c->cfg.precision == EIF_PREC_MIXED) {
    CorrArgsDF a;
    a.ux = c->ux[c->cur];
    a.uy = c->uy[c->cur];
    a.uxf = c->uxf[c->cur];
    a.uyf = c->uyf[c->cur];
    a.p = c->p;
    a.psi = c->psi;
    a.psi1 = c->psi_pair ? reinterpret_cast<const float *>(c->psi) : nullptr;
    a.psi2_off = c->nfield;
    a.dux = reinterpret_cast<const float *>(c->dux);
    a.duy = reinterpret_cast<const float *>(c->duy);
    a.rdxc = c->rdxc_df;
    a.coef = c->d_coef;
    const double rdy = 1. / c->dy;
    const float hi = (float)rdy;
    a.rdy = eifdf::DF{hi, (float)(rdy - (double)hi)};
    a.rk = rk >= 0 ? rk : 0;
    a.itot = c->itot; a.jtot = c->jtot; a.ld = c->ld;
    a.with_ibm = with_ibm; a.with_proj = with_proj; a.with_pressure = with_pressure;
    EIF_PROF(c, "correct", 1);
    launch_tiled(k_correct_df<4>, k_correct_df<8>, k_correct_df<16>, c->tiles.corr, c, a);
    EIF_LAUNCH_CK(c);
    return EIF_OK;
  }
  CorrArgs a;
  a.ux = c->ux[c->cur];
  a.uy = c->uy[c->cur];
  a.p = c->p;
  a.psi = c->psi;
  a.dux = c->dux;
  a.duy = c->duy;
  a.rdxc = c->rdxc;
  a.dt = c->d_scal;
  a.gamma = rk >= 0 ? rk_coef(rk).gamma : 0.;
  a.rdy = 1. / c->dy;
  a.itot = c->itot; a.jtot = c->jtot; a.ld = c->ld;
  a.with_ibm = with_ibm; a.with_proj = with_proj; a.with_pressure = with_pressure;
  EIF_PROF(c, "correct", 1);
  launch_tiled(k_correct<4>, k_correct<8>, k_correct<16>, c->tiles.corr, c, a);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

int launch_update_momentum_field(eif_ctx *c) { return launch_corr(c, -1, 1, 0, 0); }
int launch_correct(eif_ctx *c, int rk, bool with_ibm, bool with_pressure) {
  return launch_corr(c, rk, with_ibm ? 1 : 0, 1, with_pressure ? 1 : 0);
}
int launch_update_pressure(eif_ctx *c) { return launch_corr(c, -1, 0, 0, 1); }

int launch_decide_dt(eif_ctx *c) {
  unsigned long long *colmax = reinterpret_cast<unsigned long long *>(c->qhat);  // scratch: itot+2 words
  unsigned long long *uymax = colmax + c->itot + 2;
  EIF_PROF(c, "decide_dt", 3);
  EIF_CK(c, cudaMemsetAsync(colmax, 0, sizeof(unsigned long long) * (c->itot + 3), c->stream));
  const int gx = (c->itot / 2 + 1 + CM_THREADS - 1) / CM_THREADS;   // column pairs 0 .. itot/2
  const int gy = std::max(1, std::min(c->jtot, (c->sms * 8 + gx - 1) / gx));
  k_dt_colmax<<<dim3(gx, gy), CM_THREADS, 0, c->stream>>>(c->ux[c->cur], c->uy[c->cur], c->itot, c->jtot, c->ld,
                                                            colmax, uymax, c->d_flags);
  EIF_LAUNCH_CK(c);
  double *part = reinterpret_cast<double *>(uymax + 1);   // scratch: 3 * DT_BLOCKS words
  k_dt_partial<<<DT_BLOCKS, 64, 0, c->stream>>>(colmax, uymax, c->dxc, c->itot, c->dy, c->lx, c->dx, c->P, c->pcap,
                                                c->np, part);
  EIF_LAUNCH_CK(c);
  static_assert(DT_BLOCKS <= 32, "one warp combines the dt partials");
  k_dt_final<<<1, 32, 0, c->stream>>>(part, DT_BLOCKS, c->dy, c->cfg.Re, c->cfg.safefactors[0], c->cfg.safefactors[1],
                                     c->cfg.safefactors[2], c->d_scal, c->d_coef);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

int launch_divergence(eif_ctx *c, double *divmax, double *divsum) {
  const int blocks = c->sms * 2;
  double *part = c->qhat;  // scratch
  EIF_PROF(c, "divergence", 1);
  k_divergence<<<blocks, 256, 0, c->stream>>>(c->ux[c->cur], c->uy[c->cur], c->dxf, c->dy, c->itot, c->jtot, c->ld,
                                               part);
  EIF_LAUNCH_CK(c);
  double *h = new double[2 * blocks];
  cudaError_t e = cudaMemcpyAsync(h, part, sizeof(double) * 2 * blocks, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    delete[] h;
    return check_cuda(c, e, "divergence readback");
  }
  double mx = 0., sm = 0.;
  for (int b = 0; b < blocks; b++) { mx = fmax(mx, h[2 * b]); sm += h[2 * b + 1]; }
  delete[] h;
  *divmax = mx;
  *divsum = sm;
  return EIF_OK;
}

}  // namespace eif

// ---------------------------------------------------------------------------
// self-test of eifd::d2f / eifd::f2d against the hardware conversions
namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__global__ void k_selftest_cvt(int n, unsigned long long *counts) {
  unsigned long long bad_d2f = 0, bad_f2d = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    // doubles whose exponents cover the float normal range and beyond
    const unsigned long long r = mix64((unsigned long long)t);
    const unsigned long long e = 850ull + (r >> 53) % 350ull;
    const unsigned long long bits = (r & 0x800fffffffffffffull) | (e << 52);
    double x = __longlong_as_double((long long)bits);
    if (t == 0) x = 0.;
    if (t == 1) x = -0.;
    if (t == 2) x = 1.;
    if (t == 3) x = 3.4028234663852886e38;  // FLT_MAX
    if (t == 4) x = 1.1754943508222875e-38; // FLT_MIN
    const float hw = __double2float_rn(x);
    const float me = eifd::d2f(x);
    const bool normal = fabs(x) >= 1.1754943508222875e-38 && fabs(x) <= 3.4028234663852886e38;
    if (normal) {
      const int diff = abs((int)__float_as_uint(hw) - (int)__float_as_uint(me));
      if (diff > 1) bad_d2f++;
      if (diff == 1) {
        // allowed only on an exact tie (the discarded bits are exactly one half)
        const unsigned lo = (unsigned)__double2loint(x);
        if ((lo & 0x1fffffffu) != 0x10000000u) bad_d2f++;
      }
    }
    // float -> double on the normal floats
    const float xf = __uint_as_float((unsigned)(r & 0xffffffffu));
    const unsigned mag = __float_as_uint(xf) & 0x7fffffffu;
    if (mag >= 0x00800000u && mag < 0x7f800000u) {
      if (__double_as_longlong(eifd::f2d(xf)) != __double_as_longlong((double)xf)) bad_f2d++;
    }
    // float pairs -> double (eifd::pair_to_double against the FP64 addition it stands
    // for): lo of every size below hi, of either sign, and zero
    const unsigned long long r2 = mix64(r);
    const float lo = (r2 & 0xffull) == 0ull ? 0.f
                   : xf * __uint_as_float((unsigned)(127 - (int)((r2 >> 8) % 48ull)) << 23) *
                         ((float)((r2 >> 16) & 0xffffffull) * (1.f / 16777216.f)) * ((r2 >> 63) ? -1.f : 1.f);
    const double want = eifd::f2d(xf) + eifd::f2d(lo);
    const double got = eifd::pair_to_double(xf, lo);
    if (__double_as_longlong(want) != __double_as_longlong(got) && !(want != want && got != got)) bad_f2d++;
  }
  atomicAdd(counts, bad_d2f);
  atomicAdd(counts + 1, bad_f2d);
}

}  // namespace

extern "C" int eif_selftest_conversions(int device, int n, long long *d2f_mismatch, long long *f2d_mismatch) {
  if (n <= 0 || !d2f_mismatch || !f2d_mismatch) return EIF_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return EIF_ERR_CUDA;
  unsigned long long *d = nullptr;
  if (cudaMalloc((void **)&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return EIF_ERR_NOMEM;
  unsigned long long h[2] = {0, 0};
  cudaError_t e = cudaMemset(d, 0, sizeof(h));
  if (e == cudaSuccess) {
    k_selftest_cvt<<<256, 256>>>(n, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return EIF_ERR_CUDA;
  *d2f_mismatch = (long long)h[0];
  *f2d_mismatch = (long long)h[1];
  return EIF_OK;
}

// ---------------------------------------------------------------------------
// element-wise precision conversion of whole arrays (state transfer in the mixed form)
namespace {
__global__ void k_f2d_copy(const float *__restrict__ in, double *__restrict__ out, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    out[t] = (double)in[t];
}
__global__ void k_d2f_copy(const double *__restrict__ in, float *__restrict__ out, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    out[t] = __double2float_rn(in[t]);
}
}  // namespace

namespace eif {
int launch_f2d_copy(eif_ctx *c, const float *in, double *out, size_t n) {
  k_f2d_copy<<<c->sms * 4, 256, 0, c->stream>>>(in, out, n);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}
int launch_d2f_copy(eif_ctx *c, const double *in, float *out, size_t n) {
  k_d2f_copy<<<c->sms * 4, 256, 0, c->stream>>>(in, out, n);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}
}  // namespace eif

namespace eif {
int launch_coef(eif_ctx *c) {
  k_coef<<<1, 1, 0, c->stream>>>(c->d_scal, c->d_coef);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}
}  // namespace eif
