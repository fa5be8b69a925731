// Pressure Poisson solve for the scalar potential psi
// (src/fluid/compute_potential.c:48-138, src/tdm.c:37-131).
//
// The reference computes the right-hand side q = div(u)/(gamma dt), applies a
// DCT-II (FFTW REDFT10) along x to each row, transposes, solves one periodic
// tridiagonal system along y per x-wavenumber (tdm.c, Thomas on the leading
// n-1 rows plus a correction vector and the last row), transposes back,
// applies a DCT-III (REDFT01) and scales by 1/(2 itot).
//
// On the GPU no transpose is needed: rows stay x-contiguous, so a warp of
// threads over consecutive wavenumbers walks a column with coalesced loads.
//   1. k_dct2: one CTA per row. The right-hand side is formed in the load
//      (including the IBM field response u** = u* + avg(dux), which is
//      therefore never stored), then the DCT-II is computed as a length-n/2
//      complex FFT (Makhoul's reordering + real-to-complex split) in shared
//      memory with a mixed radix-4/2/3 Stockham autosort FFT.
//   2. k_tdm_local: the column of each wavenumber is cut into blocks of
//      EIF_TDM_M rows: EIF_TDM_M-1 interior rows and one interface row. Each
//      thread solves the interior rows of one block in registers with
//      pre-factored Thomas coefficients (the matrix is constant along y).
//   3. k_tdm_reduced: one thread per wavenumber solves the cyclic system of
//      the interface values, which again has constant coefficients and is
//      solved with the reference's cyclic algorithm (tdm.c:64-108), on
//      right-hand sides and factors staged in shared memory.
//   4. k_dct3: one CTA per row; the interior values are reconstructed from
//      the block solution and the two neighbouring interface values in the
//      load, then DCT-III, scaling and the Neumann/halo values of psi
//      (compute_potential.c:130-137).
// The kx = 0 system is singular; the reference leaves its additive constant
// to rounding noise (tdm.c:100-102, the guard does not fire). Here that
// constant is fixed by pinning the last interface value of kx = 0 to zero.
// The constant shifts psi (and p) uniformly and does not change velocities.
#include "eif_internal.cuh"
#include "eif_df.cuh"
#include <cmath>
#include <vector>
#include <algorithm>

namespace {

using eifd::ux_idx;
using eifd::uy_idx;

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 conjd(double2 a) { return make_double2(a.x, -a.y); }
// multiply by +i or -i
__device__ __forceinline__ double2 mul_i(double2 a, int sign) {
  return sign > 0 ? make_double2(-a.y, a.x) : make_double2(a.y, -a.x);
}

struct FftDesc {
  int m, nfac;
  int fac[16];
};

// Stockham autosort FFT of length d.m on shared memory buffers x and y;
// returns the buffer holding the result. sign = -1 forward, +1 inverse
// (unnormalised). tw[k] = exp(-2 pi i k / m).
__device__ double2 *fft_smem(double2 *x, double2 *y, const FftDesc &d, const double2 *__restrict__ tw, int sign) {
  const int m = d.m;
  int L = 1;
  for (int s = 0; s < d.nfac; s++) {
    const int R = d.fac[s];
    const int Ls = L * R;
    const int nb = m / R;
    const int tws = m / Ls;
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
      const int k = j % L;
      const int blk = j / L;
      double2 a[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        if (r < R) {
          double2 v = x[j + r * nb];
          if (r > 0 && k > 0) {
            double2 w = __ldg(tw + r * k * tws);
            if (sign > 0) w.y = -w.y;
            v = cmul(v, w);
          }
          a[r] = v;
        }
      }
      const int o = blk * Ls + k;
      if (R == 4) {
        const double2 s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
        const double2 s13 = cadd(a[1], a[3]), d13 = mul_i(csub(a[1], a[3]), sign);
        y[o] = cadd(s02, s13);
        y[o + L] = cadd(d02, d13);
        y[o + 2 * L] = csub(s02, s13);
        y[o + 3 * L] = csub(d02, d13);
      } else if (R == 2) {
        y[o] = cadd(a[0], a[1]);
        y[o + L] = csub(a[0], a[1]);
      } else {  // R == 3
        const double c1 = -0.5;
        const double s1 = sign * 0.86602540378443864676;  // sin(2 pi / 3)
        const double2 t = cadd(a[1], a[2]);
        const double2 u = csub(a[1], a[2]);
        const double2 base = make_double2(a[0].x + c1 * t.x, a[0].y + c1 * t.y);
        const double2 rot = make_double2(-s1 * u.y, s1 * u.x);
        y[o] = cadd(a[0], t);
        y[o + L] = cadd(base, rot);
        y[o + 2 * L] = csub(base, rot);
      }
    }
    __syncthreads();
    double2 *t = x;
    x = y;
    y = t;
    L = Ls;
  }
  return x;
}

struct Dct2Args {
  const double *ux, *uy, *dux, *duy, *dt;
  const double *rhs;   // when set: the right-hand side itself (uy layout), used as given
  double *qhat;
  const double2 *tw, *rot, *wn;
  FftDesc fd;
  double gamma, rdx, rdy;
  int itot, jtot, ld, with_ibm;
};

// RHS + DCT-II of one row (compute_potential.c:70-92)
__global__ void __launch_bounds__(256) k_dct2(Dct2Args a) {
  extern __shared__ double2 sm[];
  const int n = a.itot, m = n / 2, ld = a.ld;
  double *q = reinterpret_cast<double *>(sm + 2 * m);
  const int j = 1 + blockIdx.x;
  const double inv = 1. / (a.gamma * __ldg(a.dt));
  for (int i = 1 + threadIdx.x; i <= n; i += blockDim.x) {
    if (a.rhs) {
      q[i - 1] = __ldg(a.rhs + uy_idx(i, j, ld));
      continue;
    }
    // velocities after the IBM response, evaluated as the reference stores them
    double uxm = __ldg(a.ux + ux_idx(i, j, ld)), uxp = __ldg(a.ux + ux_idx(i + 1, j, ld));
    double uym = __ldg(a.uy + uy_idx(i, j, ld)), uyp = __ldg(a.uy + uy_idx(i, j + 1, ld));
    if (a.with_ibm) {
      const int c = uy_idx(i, j, ld);
      const double dw = __ldg(a.dux + c - 1), d0 = __ldg(a.dux + c), de = __ldg(a.dux + c + 1);
      if (i >= 2) uxm = uxm + 0.5 * (dw + d0);
      if (i + 1 <= n) uxp = uxp + 0.5 * (d0 + de);
      const double ds = __ldg(a.duy + c - ld), e0 = __ldg(a.duy + c), en = __ldg(a.duy + c + ld);
      uym = uym + 0.5 * (ds + e0);
      uyp = uyp + 0.5 * (e0 + en);
    }
    q[i - 1] = inv * ((uxp - uxm) * a.rdx + (uyp - uym) * a.rdy);
  }
  __syncthreads();
  // Makhoul reordering v[t] = q[2t], v[n-1-t] = q[2t+1]; z[s] = v[2s] + i v[2s+1]
  double2 *x = sm, *y = sm + m;
  for (int s = threadIdx.x; s < m; s += blockDim.x) {
    const int t0 = 2 * s, t1 = 2 * s + 1;
    const double v0 = t0 < m ? q[2 * t0] : q[2 * (n - 1 - t0) + 1];
    const double v1 = t1 < m ? q[2 * t1] : q[2 * (n - 1 - t1) + 1];
    x[s] = make_double2(v0, v1);
  }
  __syncthreads();
  const double2 *Z = fft_smem(x, y, a.fd, a.tw, -1);
  double *out = a.qhat + (size_t)(j - 1) * ld;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int kk = k <= m ? k : n - k;
    const double2 zk = Z[kk % m];
    const double2 zm = conjd(Z[(m - kk) % m]);
    const double2 e = make_double2(0.5 * (zk.x + zm.x), 0.5 * (zk.y + zm.y));
    const double2 df = csub(zk, zm);
    const double2 o = make_double2(0.5 * df.y, -0.5 * df.x);  // (zk - zm) / 2i
    double2 v = cadd(e, cmul(__ldg(a.wn + kk), o));
    if (k > m) v.y = -v.y;
    const double2 r = __ldg(a.rot + k);
    out[k] = 2. * (r.x * v.x - r.y * v.y);
  }
}

// interior Thomas solve of one block in registers
template <int M>
__global__ void __launch_bounds__(256) k_tdm_local(double *__restrict__ qhat, const double *__restrict__ inv,
                                                  const double *__restrict__ up, double *__restrict__ iface_a,
                                                  double *__restrict__ first, double l, int itot, int nblk, int ld) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (k >= itot) return;
  double v[M - 1];
  const size_t base = (size_t)b * M * ld + k;
#pragma unroll
  for (int r = 0; r < M - 1; r++) v[r] = qhat[base + (size_t)r * ld];
  const double rif = qhat[base + (size_t)(M - 1) * ld];
  v[0] = v[0] * __ldg(inv + k);
#pragma unroll
  for (int r = 1; r < M - 1; r++) v[r] = (v[r] - l * v[r - 1]) * __ldg(inv + r * itot + k);
#pragma unroll
  for (int r = M - 3; r >= 0; r--) v[r] = v[r] - __ldg(up + r * itot + k) * v[r + 1];
#pragma unroll
  for (int r = 0; r < M - 1; r++) qhat[base + (size_t)r * ld] = v[r];
  // interface equation: r_iface - l y[M-2] (this block) - l y[0] (next block)
  iface_a[(size_t)b * itot + k] = rif - l * v[M - 2];
  first[(size_t)b * itot + k] = v[0];
}

// cyclic system of the interface values of one wavenumber. One thread per
// wavenumber runs the serial sweeps; the block's other threads first stage the
// right-hand sides and the elimination factors of its `cols` wavenumbers in
// shared memory (many loads in flight), so that the sweeps run at shared-memory
// latency, and afterwards write the results back. With iface_f set, the solved values
// are also stored rounded to float (eifd::d2f), the input of the single-precision DCT-III,
// which then converts each of them once instead of once per row of its block.
constexpr int RED_THREADS = 256;

__global__ void __launch_bounds__(RED_THREADS) k_tdm_reduced(double *__restrict__ iface, const double *__restrict__ first,
                                                             const double *__restrict__ rinv, const double *__restrict__ rup,
                                                             const double *__restrict__ rq1, const double *__restrict__ rcoef,
                                                             double l, int itot, int nblk, int cols,
                                                             float *__restrict__ iface_f) {
  extern __shared__ double zs[];  // [nblk][cols] right-hand sides, then [nblk][cols] rinv, rup; [cols] last
  const int P = nblk;
  double *fi = zs + (size_t)P * cols, *fu = fi + (size_t)P * cols, *lastv = fu + (size_t)P * cols;
  const int k0 = blockIdx.x * cols;
  // right-hand side R_b = (r_iface - l y_b[M-2]) - l y_{b+1}[0]; factors
  for (int idx = threadIdx.x; idx < P * cols; idx += blockDim.x) {
    const int b = idx / cols, t = idx - b * cols;
    const int kk = min(k0 + t, itot - 1);
    zs[idx] = iface[(size_t)b * itot + kk] - l * first[(size_t)((b + 1) % P) * itot + kk];
    fi[idx] = rinv[(size_t)b * itot + kk];
    fu[idx] = rup[(size_t)b * itot + kk];
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t < cols) {
    const int kk = min(k0 + t, itot - 1);
    const double A = rcoef[4 * kk + 0];
    const double den = rcoef[4 * kk + 2];
    const bool pin = rcoef[4 * kk + 3] != 0.;
    const double rP = zs[(P - 1) * cols + t];
    // Thomas on the leading P-1 rows
    double zprev = zs[t] * fi[t];
    zs[t] = zprev;
#pragma unroll 8
    for (int b = 1; b < P - 1; b++) {
      zprev = (zs[b * cols + t] - A * zprev) * fi[b * cols + t];
      zs[b * cols + t] = zprev;
    }
#pragma unroll 8
    for (int b = P - 3; b >= 0; b--) {
      zprev = zs[b * cols + t] - fu[b * cols + t] * zprev;
      zs[b * cols + t] = zprev;
    }
    const double z0 = zs[t], zl = zs[(P - 2) * cols + t];
    const double num = rP - A * z0 - A * zl;
    lastv[t] = pin ? 0. : num / den;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < P * cols; idx += blockDim.x) {
    const int b = idx / cols, tt = idx - b * cols;
    const int k = k0 + tt;
    if (k >= itot) continue;
    const double last = lastv[tt];
    const double v = b == P - 1 ? last : zs[idx] + last * rq1[(size_t)b * itot + k];
    iface[(size_t)b * itot + k] = v;
    if (iface_f) iface_f[(size_t)b * itot + k] = eifd::d2f(v);
  }
}

// The same partition one level down. The reduced system of a wavenumber (P
// interface values, constant coefficients A, B) is cut into Q groups of G: G-1
// interior values and one second-level interface value t_g per group. Every
// thread solves one group's interior with zero interfaces (factors inv2/up2 for
// the off-diagonal A and diagonal B) and its interface equation's right-hand
// side; one thread per wavenumber solves the cyclic system of the Q values t_g
// (A2 = A phi[G-2], B2 = B + 2 A phi[0], the reference's cyclic algorithm as at the
// first level, kx = 0 pinned with its last value 0); every thread then adds
// t_{g-1} phi[i] + t_g phi[G-2-i] to its interior. Block: RED2_K wavenumbers x Q
// groups (8 wavenumbers per block spread the FP64 work over 256 blocks at 2048 x 4096);
// the factors of the Q-value solve are staged in shared memory by the whole block
// before its serial sweep. iface_f (optional): the solved values rounded to float, as in
// k_tdm_reduced.
constexpr int RED2_K = 8;
constexpr size_t red2_smem_bytes(int Q) { return sizeof(double) * 6 * RED2_K * (size_t)Q; }
template <int G>
__global__ void __launch_bounds__(1024) k_tdm_reduced2(double *__restrict__ iface, const double *__restrict__ first,
                                                       const double *__restrict__ rcoef, const double *__restrict__ inv2,
                                                       const double *__restrict__ up2, const double *__restrict__ phi2,
                                                       const double *__restrict__ ri2, const double *__restrict__ ru2,
                                                       const double *__restrict__ rq2, const double *__restrict__ rc2,
                                                       double l, int itot, int P, int Q, float *__restrict__ iface_f) {
  // [Q][RED2_K] first interior values, right-hand sides, interface values, and the
  // second-level factors ri2, ru2, rq2
  extern __shared__ double sm2[];
  constexpr int K = RED2_K;
  double *y0s = sm2, *rhs = sm2 + (size_t)Q * K, *ts = sm2 + (size_t)2 * Q * K;
  double *s_ri = sm2 + (size_t)3 * Q * K, *s_ru = sm2 + (size_t)4 * Q * K, *s_rq = sm2 + (size_t)5 * Q * K;
  const int kk = threadIdx.x % K, g = threadIdx.x / K;
  const int k = blockIdx.x * K + kk;
  const bool on = k < itot;
  const int kc = on ? k : itot - 1;
  const double A = rcoef[4 * kc + 0];
  // the factors of the second-level sweep (q < Q - 1; the tables hold max(G, Q) rows)
  if (g < Q - 1) {
    s_ri[g * K + kk] = ri2[(size_t)g * itot + kc];
    s_ru[g * K + kk] = ru2[(size_t)g * itot + kc];
    s_rq[g * K + kk] = rq2[(size_t)g * itot + kc];
  }
  double y[G];
  // level-one reduced right-hand sides R_b = (r_iface - l y_b[M-2]) - l y_{b+1}[0]
#pragma unroll
  for (int i = 0; i < G; i++) {
    const int b = g * G + i;
    y[i] = iface[(size_t)b * itot + kc] - l * first[(size_t)((b + 1) % P) * itot + kc];
  }
  const double rlast = y[G - 1];
  y[0] = y[0] * inv2[kc];
#pragma unroll
  for (int i = 1; i < G - 1; i++) y[i] = (y[i] - A * y[i - 1]) * inv2[(size_t)i * itot + kc];
#pragma unroll
  for (int i = G - 3; i >= 0; i--) y[i] = y[i] - up2[(size_t)i * itot + kc] * y[i + 1];
  y0s[g * K + kk] = y[0];
  __syncthreads();
  rhs[g * K + kk] = rlast - A * y[G - 2] - A * y0s[((g + 1) % Q) * K + kk];
  __syncthreads();
  if (g == 0) {
    const double A2 = rc2[4 * kc + 0], den2 = rc2[4 * kc + 2];
    const bool pin = rc2[4 * kc + 3] != 0.;
    double zprev = rhs[kk] * s_ri[kk];
    ts[kk] = zprev;
    for (int q = 1; q < Q - 1; q++) {
      zprev = (rhs[q * K + kk] - A2 * zprev) * s_ri[q * K + kk];
      ts[q * K + kk] = zprev;
    }
    for (int q = Q - 3; q >= 0; q--) {
      zprev = ts[q * K + kk] - s_ru[q * K + kk] * zprev;
      ts[q * K + kk] = zprev;
    }
    const double num = rhs[(Q - 1) * K + kk] - A2 * ts[kk] - A2 * ts[(Q - 2) * K + kk];
    const double last = pin ? 0. : num / den2;
    for (int q = 0; q < Q - 1; q++) ts[q * K + kk] = ts[q * K + kk] + last * s_rq[q * K + kk];
    ts[(Q - 1) * K + kk] = last;
  }
  __syncthreads();
  if (!on) return;
  const double tl = ts[((g + Q - 1) % Q) * K + kk], tr = ts[g * K + kk];
#pragma unroll
  for (int i = 0; i < G - 1; i++) {
    const double v = y[i] + tl * phi2[(size_t)i * itot + k] + tr * phi2[(size_t)(G - 2 - i) * itot + k];
    iface[(size_t)(g * G + i) * itot + k] = v;
    if (iface_f) iface_f[(size_t)(g * G + i) * itot + k] = eifd::d2f(v);
  }
  iface[(size_t)(g * G + G - 1) * itot + k] = tr;
  if (iface_f) iface_f[(size_t)(g * G + G - 1) * itot + k] = eifd::d2f(tr);
}

// columns per block of k_tdm_reduced that fit its shared memory
static int red_cols(int nblk) {
  for (int cols = 16; cols >= 1; cols /= 2) {
    if (sizeof(double) * ((size_t)3 * nblk * cols + cols) <= 227 * 1024) return cols;
  }
  return 0;
}
static size_t red_smem_bytes(int nblk, int cols) { return sizeof(double) * ((size_t)3 * nblk * cols + cols); }

// fallback for column lengths without a suitable block size: the reference's
// sequential cyclic algorithm per wavenumber on global memory
__global__ void k_tdm_serial(double *__restrict__ qhat, double *__restrict__ scratch, const double *__restrict__ lam,
                             double l, int itot, int jtot, int ld) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= itot) return;
  const int n = jtot;
  const double c = -l - l + lam[k];
  double *u0 = scratch + k;                     // [i*itot + k]
  double *q1 = scratch + (size_t)n * itot + k;  // [i*itot + k]
  auto Q = [&](int i) -> double & { return qhat[(size_t)i * ld + k]; };
  auto U0 = [&](int i) -> double & { return u0[(size_t)i * itot]; };
  auto Q1 = [&](int i) -> double & { return q1[(size_t)i * itot]; };
  for (int i = 0; i < n - 1; i++) Q1(i) = i == 0 ? -l : (i == n - 2 ? -l : 0.);
  // Thomas on rows 0..n-2 for q and q1 together (same factors)
  U0(0) = l / c;
  Q(0) = Q(0) / c;
  Q1(0) = Q1(0) / c;
  for (int i = 1; i <= n - 2; i++) {
    double val = c - l * U0(i - 1);
    if (fabs(val) < 2.220446049250313e-16) {
      U0(i) = 0.; Q(i) = 0.; Q1(i) = 0.;
    } else {
      val = 1. / val;
      U0(i) = val * l;
      Q(i) = val * (Q(i) - l * Q(i - 1));
      Q1(i) = val * (Q1(i) - l * Q1(i - 1));
    }
  }
  for (int i = n - 3; i >= 0; i--) {
    Q(i) -= U0(i) * Q(i + 1);
    Q1(i) -= U0(i) * Q1(i + 1);
  }
  const double num = Q(n - 1) - l * Q(0) - l * Q(n - 2);
  const double den = c + l * Q1(0) + l * Q1(n - 2);
  const double last = (k == 0 || fabs(den) < 2.220446049250313e-16) ? 0. : num / den;
  Q(n - 1) = last;
  for (int i = 0; i <= n - 2; i++) Q(i) = Q(i) + last * Q1(i);
}

struct Dct3Args {
  const double *qhat, *iface, *g;
  double *psi;
  const double2 *tw, *rot, *wn;
  FftDesc fd;
  int itot, jtot, ld, blk, nblk;
};

// block reconstruction + DCT-III + scaling of one row (compute_potential.c:118-137)
__global__ void __launch_bounds__(256) k_dct3(Dct3Args a) {
  extern __shared__ double2 sm[];
  const int n = a.itot, m = n / 2, ld = a.ld;
  double *xr = reinterpret_cast<double *>(sm + 2 * m);
  const int j = 1 + blockIdx.x;
  const int jr = j - 1;  // 0-based row in the tridiagonal systems
  const double *row = a.qhat + (size_t)jr * ld;
  if (a.blk > 0) {
    const int M = a.blk;
    const int b = jr / M, r = jr % M;
    const int bm = (b + a.nblk - 1) % a.nblk;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      double v;
      if (r == M - 1) {
        v = __ldg(a.iface + (size_t)b * n + k);
      } else {
        const double gl = __ldg(a.g + (size_t)r * n + k);
        const double gr = __ldg(a.g + (size_t)(M - 2 - r) * n + k);
        v = __ldg(row + k) + __ldg(a.iface + (size_t)bm * n + k) * gl + __ldg(a.iface + (size_t)b * n + k) * gr;
      }
      xr[k] = v;
    }
  } else {
    for (int k = threadIdx.x; k < n; k += blockDim.x) xr[k] = __ldg(row + k);
  }
  __syncthreads();
  double2 *x = sm, *y = sm + m;
  // W[t] = exp(i pi t / 2n) (x[t] - i x[n-t]); Z[s] = (W[s] + W[s+m]) + i (W[s] - W[s+m]) exp(2 pi i s / n)
  for (int s = threadIdx.x; s < m; s += blockDim.x) {
    const int t0 = s, t1 = s + m;
    const double2 r0 = conjd(__ldg(a.rot + t0)), r1 = conjd(__ldg(a.rot + t1));
    const double2 w0 = cmul(r0, make_double2(xr[t0], t0 == 0 ? 0. : -xr[n - t0]));
    const double2 w1 = cmul(r1, make_double2(xr[t1], -xr[n - t1]));
    const double2 sum = cadd(w0, w1);
    const double2 dif = cmul(csub(w0, w1), conjd(__ldg(a.wn + s)));
    x[s] = make_double2(sum.x - dif.y, sum.y + dif.x);
  }
  __syncthreads();
  const double2 *z = fft_smem(x, y, a.fd, a.tw, +1);
  const double scale = 1. / (2. * n);
  double *prow = a.psi + (size_t)j * ld;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    // y[2t] = w[t], y[2t+1] = w[n-1-t]; w[2s] = Re z[s], w[2s+1] = Im z[s]
    const int t = (i & 1) ? n - 1 - (i >> 1) : (i >> 1);
    const double w = (t & 1) ? z[t >> 1].y : z[t >> 1].x;
    const double v = w * scale;
    prow[i + 1] = v;
    if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld + i + 1] = v;
    if (j == a.jtot) a.psi[i + 1] = v;
    if (i == 0) {
      prow[0] = v;
      if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld] = v;
      if (j == a.jtot) a.psi[0] = v;
    }
    if (i == n - 1) {
      prow[n + 1] = v;
      if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld + n + 1] = v;
      if (j == a.jtot) a.psi[n + 1] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// Complex double-float arithmetic (eif_df.cuh) for the mixed-precision form.
using namespace eifdf;
struct CDF { DF re, im; };

__device__ __forceinline__ CDF cdf_add(CDF a, CDF b) { return CDF{df_add_nw(a.re, b.re), df_add_nw(a.im, b.im)}; }
__device__ __forceinline__ CDF cdf_sub(CDF a, CDF b) {
  return CDF{df_add_nw(a.re, df_neg(b.re)), df_add_nw(a.im, df_neg(b.im))};
}
// x.hi y.hi + s u.hi v.hi formed exactly (two products, one TwoSum), the
// cross and trailing terms accumulated in single precision with FMAs
__device__ __forceinline__ DF df_dot2(DF x, DF y, DF u, DF v, float sgn) {
  const float p1 = x.hi * y.hi, p2 = sgn * (u.hi * v.hi);
  const float e1 = fmaf(x.hi, y.hi, -p1), e2 = fmaf(sgn * u.hi, v.hi, -p2);
  const DF s = two_sum(p1, p2);
  float t = fmaf(x.hi, y.lo, e1);
  t = fmaf(x.lo, y.hi, t);
  t = fmaf(sgn * u.hi, v.lo, t);
  t = fmaf(sgn * u.lo, v.hi, t);
  t = t + e2 + s.lo;
  return fast_sum(s.hi, t);
}
__device__ __forceinline__ CDF cdf_mul(CDF a, CDF b) {
  return CDF{df_dot2(a.re, b.re, a.im, b.im, -1.f), df_dot2(a.re, b.im, a.im, b.re, 1.f)};
}
__device__ __forceinline__ CDF cdf_conj(CDF a) { return CDF{a.re, df_neg(a.im)}; }
__device__ __forceinline__ CDF cdf_mul_i(CDF a, int sign) {
  return sign > 0 ? CDF{df_neg(a.im), a.re} : CDF{a.im, df_neg(a.re)};
}
__device__ __forceinline__ CDF cdf_load(const float4 *t, int k) {
  const float4 v = __ldg(t + k);
  return CDF{DF{v.x, v.y}, DF{v.z, v.w}};
}

// double-float version of fft_smem (same Stockham radix-4/2/3 schedule)
__device__ CDF *fft_smem_df(CDF *x, CDF *y, const FftDesc &d, const float4 *__restrict__ tw, int sign) {
  const int m = d.m;
  int L = 1;
  for (int s = 0; s < d.nfac; s++) {
    const int R = d.fac[s];
    const int Ls = L * R;
    const int nb = m / R;
    const int tws = m / Ls;
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
      const int k = j % L;
      const int blk = j / L;
      CDF a[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        if (r < R) {
          CDF v = x[j + r * nb];
          if (r > 0 && k > 0) {
            CDF w = cdf_load(tw, r * k * tws);
            if (sign > 0) w = cdf_conj(w);
            v = cdf_mul(v, w);
          }
          a[r] = v;
        }
      }
      const int o = blk * Ls + k;
      if (R == 4) {
        const CDF s02 = cdf_add(a[0], a[2]), d02 = cdf_sub(a[0], a[2]);
        const CDF s13 = cdf_add(a[1], a[3]), d13 = cdf_mul_i(cdf_sub(a[1], a[3]), sign);
        y[o] = cdf_add(s02, s13);
        y[o + L] = cdf_add(d02, d13);
        y[o + 2 * L] = cdf_sub(s02, s13);
        y[o + 3 * L] = cdf_sub(d02, d13);
      } else if (R == 2) {
        y[o] = cdf_add(a[0], a[1]);
        y[o + L] = cdf_sub(a[0], a[1]);
      } else {  // R == 3: w = -1/2 + i sign sqrt(3)/2
        const CDF t = cdf_add(a[1], a[2]);
        const CDF u = cdf_sub(a[1], a[2]);
        const CDF base = cdf_sub(a[0], CDF{df_scale(t.re, 0.5f), df_scale(t.im, 0.5f)});
        const DF s3 = DF{0.8660253882408142f, 1.5543625053737742e-08f};  // sqrt(3)/2 as a float pair
        const DF ss = sign > 0 ? s3 : df_neg(s3);
        const CDF rot = CDF{df_neg(df_mul(ss, u.im)), df_mul(ss, u.re)};
        y[o] = cdf_add(a[0], t);
        y[o + L] = cdf_add(base, rot);
        y[o + 2 * L] = cdf_sub(base, rot);
      }
    }
    __syncthreads();
    CDF *t = x;
    x = y;
    y = t;
    L = Ls;
  }
  return x;
}

struct Dct2ArgsDF {
  const double *ux, *uy;
  const float *dux, *duy;   // IBM field response in single precision
  const float *coef;   // [12 + 2 rk] = hi, lo of 1/(gamma dt)
  double *qhat;             // double, or (hi, lo) float pairs when qdf is set
  const float4 *tw, *rot, *wn;
  FftDesc fd;
  DF rdx, rdy;
  int itot, jtot, ld, with_ibm, rk, qdf;
};

// RHS + DCT-II of one row in double-float arithmetic (compute_potential.c:70-92)
__global__ void __launch_bounds__(256) k_dct2_df(Dct2ArgsDF a) {
  extern __shared__ CDF smd[];
  const int n = a.itot, m = n / 2, ld = a.ld;
  DF *q = reinterpret_cast<DF *>(smd + 2 * m);
  const int j = 1 + blockIdx.x;
  const DF inv = DF{__ldg(a.coef + 12 + 2 * a.rk), __ldg(a.coef + 13 + 2 * a.rk)};
  for (int i = 1 + threadIdx.x; i <= n; i += blockDim.x) {
    // differences of neighbouring doubles (exact), then double-float
    DF dux_ = df_of(__ldg(a.ux + ux_idx(i + 1, j, ld)) - __ldg(a.ux + ux_idx(i, j, ld)));
    DF duy_ = df_of(__ldg(a.uy + uy_idx(i, j + 1, ld)) - __ldg(a.uy + uy_idx(i, j, ld)));
    if (a.with_ibm) {
      // (u + (d0 + de)/2) - (u + (dw + d0)/2) with single-precision field values:
      // the increments (de - dw)/2 and (en - ds)/2 as exact float sums
      const int c = uy_idx(i, j, ld);
      const float dw = (i >= 2) ? __ldg(a.dux + c - 1) : -__ldg(a.dux + c);
      const float de = (i + 1 <= n) ? __ldg(a.dux + c + 1) : -__ldg(a.dux + c);
      dux_ = df_add_nw(dux_, df_scale(two_sum(de, -dw), 0.5f));
      duy_ = df_add_nw(duy_, df_scale(two_sum(__ldg(a.duy + c + ld), -__ldg(a.duy + c - ld)), 0.5f));
    }
    q[i - 1] = df_mul(inv, df_add_nw(df_mul(dux_, a.rdx), df_mul(duy_, a.rdy)));
  }
  __syncthreads();
  CDF *x = smd, *y = smd + m;
  for (int s = threadIdx.x; s < m; s += blockDim.x) {
    const int t0 = 2 * s, t1 = 2 * s + 1;
    const DF v0 = t0 < m ? q[2 * t0] : q[2 * (n - 1 - t0) + 1];
    const DF v1 = t1 < m ? q[2 * t1] : q[2 * (n - 1 - t1) + 1];
    x[s] = CDF{v0, v1};
  }
  __syncthreads();
  const CDF *Z = fft_smem_df(x, y, a.fd, a.tw, -1);
  double *out = a.qhat + (size_t)(j - 1) * ld;
  // outputs k and n - k share the half-length spectrum values (conjugate pair)
  for (int kk = threadIdx.x; kk <= m; kk += blockDim.x) {
    const CDF zk = Z[kk % m];
    const CDF zm = cdf_conj(Z[(m - kk) % m]);
    const CDF sm = cdf_add(zk, zm), df = cdf_sub(zk, zm);
    const CDF e = CDF{df_scale(sm.re, 0.5f), df_scale(sm.im, 0.5f)};
    const CDF o = CDF{df_scale(df.im, 0.5f), df_scale(df_neg(df.re), 0.5f)};  // (zk - zm) / 2i
    const CDF v = cdf_add(e, cdf_mul(cdf_load(a.wn, kk), o));
    {
      const CDF r = cdf_load(a.rot, kk);
      const DF o0 = df_scale(df_dot2(r.re, v.re, r.im, v.im, -1.f), 2.f);
      if (a.qdf) reinterpret_cast<float2 *>(out)[kk] = make_float2(o0.hi, o0.lo);
      else out[kk] = df_to_double(o0);
    }
    if (kk > 0 && kk < m) {
      // v conjugated for k = n - kk
      const CDF r = cdf_load(a.rot, n - kk);
      const DF o1 = df_scale(df_dot2(r.re, v.re, r.im, df_neg(v.im), -1.f), 2.f);
      if (a.qdf) reinterpret_cast<float2 *>(out)[n - kk] = make_float2(o1.hi, o1.lo);
      else out[n - kk] = df_to_double(o1);
    }
  }
}

struct Dct3ArgsDF {
  const double *qhat, *iface;   // qhat: double, or (hi, lo) float pairs when qdf is set
  const float2 *g;   // tdm_g as (hi, lo)
  double *psi;
  const float4 *tw, *rot, *wn;
  FftDesc fd;
  DF scale;   // 1 / (2 itot)
  int itot, jtot, ld, blk, nblk, qdf;
};

// block reconstruction + DCT-III + scaling of one row, double-float arithmetic
__global__ void __launch_bounds__(256) k_dct3_df(Dct3ArgsDF a) {
  extern __shared__ CDF smd[];
  const int n = a.itot, m = n / 2, ld = a.ld;
  DF *xr = reinterpret_cast<DF *>(smd + 2 * m);
  const int j = 1 + blockIdx.x;
  const int jr = j - 1;
  const double *row = a.qhat + (size_t)jr * ld;
  if (a.blk > 0) {
    const int M = a.blk;
    const int b = jr / M, r = jr % M;
    const int bm = (b + a.nblk - 1) % a.nblk;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      DF v;
      if (r == M - 1) {
        v = df_of(__ldg(a.iface + (size_t)b * n + k));
      } else {
        // y + s_left g + s_right h in double-float from the double-precision block solution
        const float2 gl = __ldg(a.g + (size_t)r * n + k);
        const float2 gr = __ldg(a.g + (size_t)(M - 2 - r) * n + k);
        DF yv;
        if (a.qdf) {
          const float2 t = __ldg(reinterpret_cast<const float2 *>(row) + k);
          yv = DF{t.x, t.y};
        } else {
          yv = df_of(__ldg(row + k));
        }
        v = df_add_nw(df_add_nw(yv, df_mul(df_of(__ldg(a.iface + (size_t)bm * n + k)), DF{gl.x, gl.y})),
                      df_mul(df_of(__ldg(a.iface + (size_t)b * n + k)), DF{gr.x, gr.y}));
      }
      xr[k] = v;
    }
  } else {
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      if (a.qdf) {
        const float2 t = __ldg(reinterpret_cast<const float2 *>(row) + k);
        xr[k] = DF{t.x, t.y};
      } else {
        xr[k] = df_of(__ldg(row + k));
      }
    }
  }
  __syncthreads();
  CDF *x = smd, *y = smd + m;
  for (int s = threadIdx.x; s < m; s += blockDim.x) {
    const int t0 = s, t1 = s + m;
    const CDF r0 = cdf_conj(cdf_load(a.rot, t0)), r1 = cdf_conj(cdf_load(a.rot, t1));
    const CDF w0 = cdf_mul(r0, CDF{xr[t0], t0 == 0 ? DF{0.f, 0.f} : df_neg(xr[n - t0])});
    const CDF w1 = cdf_mul(r1, CDF{xr[t1], df_neg(xr[n - t1])});
    const CDF sum = cdf_add(w0, w1);
    const CDF dif = cdf_mul(cdf_sub(w0, w1), cdf_conj(cdf_load(a.wn, s)));
    x[s] = CDF{df_add_nw(sum.re, df_neg(dif.im)), df_add_nw(sum.im, dif.re)};
  }
  __syncthreads();
  const CDF *z = fft_smem_df(x, y, a.fd, a.tw, +1);
  double *prow = a.psi + (size_t)j * ld;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = (i & 1) ? n - 1 - (i >> 1) : (i >> 1);
    const DF w = (t & 1) ? z[t >> 1].im : z[t >> 1].re;
    const double v = df_to_double(df_mul(w, a.scale));
    prow[i + 1] = v;
    if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld + i + 1] = v;
    if (j == a.jtot) a.psi[i + 1] = v;
    if (i == 0) {
      prow[0] = v;
      if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld] = v;
      if (j == a.jtot) a.psi[0] = v;
    }
    if (i == n - 1) {
      prow[n + 1] = v;
      if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld + n + 1] = v;
      if (j == a.jtot) a.psi[n + 1] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// Register-radix double-float FFT for power-of-two half lengths m (V <= m <= 512 V).
//
// T = m/V threads own one row; each holds V complex values in registers (V = 8 or
// 16). The Stockham passes are radix V (16 = 4 x 4 and 8 = 4 x 2 splits with
// constant inner twiddles) and, when log2 m is not a multiple of log2 V, one last
// pass of a smaller radix R in which each thread does V/R butterflies. Every pass
// reads its inputs, waits for the whole CTA, and writes its outputs back into the
// same row buffer, so one buffer of m values (padded by one value every V against
// bank conflicts) serves the transform. Sums inside a pass keep the trailing part
// unnormalised (a TwoSum of the leading parts, the trailing parts added in single
// precision); values are renormalised once before they are stored. The error stays
// below a small multiple of 2^-47 of the norm of the inputs, as in the radix-4
// version.
template <int V> __device__ __forceinline__ int padv(int i) { return i + (i >> (V == 16 ? 4 : 3)); }

__device__ __forceinline__ DF dfl_add(DF x, DF y) {
  const DF s = two_sum(x.hi, y.hi);
  return DF{s.hi, s.lo + (x.lo + y.lo)};
}
__device__ __forceinline__ DF dfl_sub(DF x, DF y) {
  const DF s = two_sum(x.hi, -y.hi);
  return DF{s.hi, s.lo + (x.lo - y.lo)};
}
// x y + sgn u v with exact leading products (df_dot2 without the final renormalisation)
__device__ __forceinline__ DF dfl_dot2(DF x, DF y, DF u, DF v, float sgn) {
  const float p1 = x.hi * y.hi, p2 = sgn * (u.hi * v.hi);
  const float e1 = fmaf(x.hi, y.hi, -p1), e2 = fmaf(sgn * u.hi, v.hi, -p2);
  const DF s = two_sum(p1, p2);
  float t = fmaf(x.hi, y.lo, e1);
  t = fmaf(x.lo, y.hi, t);
  t = fmaf(sgn * u.hi, v.lo, t);
  t = fmaf(sgn * u.lo, v.hi, t);
  return DF{s.hi, t + e2 + s.lo};
}
__device__ __forceinline__ DF dfl_mulc(DF x, DF c) {
  const float p = x.hi * c.hi;
  const float e = fmaf(x.hi, c.lo, fmaf(x.lo, c.hi, fmaf(x.hi, c.hi, -p)));
  return DF{p, e};
}
__device__ __forceinline__ CDF cl_add(CDF a, CDF b) { return CDF{dfl_add(a.re, b.re), dfl_add(a.im, b.im)}; }
__device__ __forceinline__ CDF cl_sub(CDF a, CDF b) { return CDF{dfl_sub(a.re, b.re), dfl_sub(a.im, b.im)}; }
__device__ __forceinline__ CDF cl_norm(CDF a) { return CDF{fast_sum(a.re.hi, a.re.lo), fast_sum(a.im.hi, a.im.lo)}; }
// a w for a twiddle w = (c, s) given as float pairs
__device__ __forceinline__ CDF cl_mul(CDF a, float4 w) {
  const DF c = DF{w.x, w.y}, s = DF{w.z, w.w};
  return CDF{dfl_dot2(a.re, c, a.im, s, -1.f), dfl_dot2(a.re, s, a.im, c, 1.f)};
}
// multiplication by S i
template <int S> __device__ __forceinline__ CDF cl_mul_si(CDF a) {
  return S > 0 ? CDF{df_neg(a.im), a.re} : CDF{a.im, df_neg(a.re)};
}
// sqrt(2)/2 and cos, sin of pi/8 as float pairs
__device__ __forceinline__ DF k_h() { return DF{0x1.6a09e6p-1f, 0x1.9fcef4p-27f}; }
__device__ __forceinline__ DF k_c1() { return DF{0x1.d906bcp-1f, 0x1.e651a8p-26f}; }
__device__ __forceinline__ DF k_s1() { return DF{0x1.87de2ap-2f, 0x1.abaa58p-28f}; }
// multiplication by exp(S i pi/4) = (sqrt(2)/2)(1 + S i)
template <int S> __device__ __forceinline__ CDF cl_mul_w8(CDF a) {
  const DF re = S > 0 ? dfl_sub(a.re, a.im) : dfl_add(a.re, a.im);
  const DF im = S > 0 ? dfl_add(a.im, a.re) : dfl_sub(a.im, a.re);
  return CDF{dfl_mulc(re, k_h()), dfl_mulc(im, k_h())};
}
// multiplication by c + S i s
template <int S> __device__ __forceinline__ CDF cl_mul_cs(CDF a, DF c, DF s) {
  return CDF{dfl_dot2(a.re, c, a.im, s, -(float)S), dfl_dot2(a.im, c, a.re, s, (float)S)};
}

// radix-4 butterfly on v[o], v[o + st], v[o + 2 st], v[o + 3 st], outputs in natural order
template <int S, int O, int ST, int N> __device__ __forceinline__ void dft4(CDF (&v)[N]) {
  const CDF s02 = cl_add(v[O], v[O + 2 * ST]), d02 = cl_sub(v[O], v[O + 2 * ST]);
  const CDF s13 = cl_add(v[O + ST], v[O + 3 * ST]), d13 = cl_mul_si<S>(cl_sub(v[O + ST], v[O + 3 * ST]));
  v[O] = cl_add(s02, s13);
  v[O + ST] = cl_add(d02, d13);
  v[O + 2 * ST] = cl_sub(s02, s13);
  v[O + 3 * ST] = cl_sub(d02, d13);
}

// 16-point DFT of v (sign S), result in natural order
template <int S> __device__ __forceinline__ void dft16(CDF (&v)[16]) {
  // n = 4 n1 + n2: transforms over n1 for each n2, result A[n2][k1] in v[n2 + 4 k1]
  dft4<S, 0, 4>(v);
  dft4<S, 1, 4>(v);
  dft4<S, 2, 4>(v);
  dft4<S, 3, 4>(v);
  // inner twiddles W16^(n2 k1)
  v[5] = cl_mul_cs<S>(v[5], k_c1(), k_s1());                 // W^1
  v[6] = cl_mul_w8<S>(v[6]);                                 // W^2
  v[7] = cl_mul_cs<S>(v[7], k_s1(), k_c1());                 // W^3
  v[9] = cl_mul_w8<S>(v[9]);                                 // W^2
  v[10] = cl_mul_si<S>(v[10]);                               // W^4
  v[11] = cl_mul_si<S>(cl_mul_w8<S>(v[11]));                 // W^6
  v[13] = cl_mul_cs<S>(v[13], k_s1(), k_c1());               // W^3
  v[14] = cl_mul_si<S>(cl_mul_w8<S>(v[14]));                 // W^6
  {
    const CDF w = cl_mul_cs<S>(v[15], k_c1(), k_s1());       // W^9 = -W^1
    v[15] = CDF{df_neg(w.re), df_neg(w.im)};
  }
  // transforms over n2 for each k1: X[k1 + 4 k2] lands in v[4 k1 + k2]
  dft4<S, 0, 1>(v);
  dft4<S, 4, 1>(v);
  dft4<S, 8, 1>(v);
  dft4<S, 12, 1>(v);
  // transpose the 4 x 4 index so that v[k] = X[k]
  CDF t;
  t = v[1]; v[1] = v[4]; v[4] = t;
  t = v[2]; v[2] = v[8]; v[8] = t;
  t = v[3]; v[3] = v[12]; v[12] = t;
  t = v[6]; v[6] = v[9]; v[9] = t;
  t = v[7]; v[7] = v[13]; v[13] = t;
  t = v[11]; v[11] = v[14]; v[14] = t;
}

// 8-point DFT of v[G], ..., v[G + 7] (sign S), result in natural order
template <int S, int G, int N> __device__ __forceinline__ void dft8(CDF (&v)[N]) {
  // n = 2 n1 + n2, k = k1 + 4 k2: transforms over n1, A[n2][k1] in v[G + n2 + 2 k1]
  dft4<S, G, 2>(v);
  dft4<S, G + 1, 2>(v);
  v[G + 3] = cl_mul_w8<S>(v[G + 3]);                         // W8^1
  v[G + 5] = cl_mul_si<S>(v[G + 5]);                         // W8^2
  v[G + 7] = cl_mul_si<S>(cl_mul_w8<S>(v[G + 7]));           // W8^3
  CDF w[8];
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    w[k1] = cl_add(v[G + 2 * k1], v[G + 2 * k1 + 1]);
    w[k1 + 4] = cl_sub(v[G + 2 * k1], v[G + 2 * k1 + 1]);
  }
#pragma unroll
  for (int k = 0; k < 8; k++) v[G + k] = w[k];
}

template <int S, int V> __device__ __forceinline__ void dft_full(CDF (&v)[V]) {
  if constexpr (V == 16) dft16<S>(v);
  else dft8<S, 0>(v);
}

// the last pass: radix R (< V) butterflies on groups of R consecutive values
template <int S, int R, int V> __device__ __forceinline__ void dft_small(CDF (&v)[V]) {
  if constexpr (R == 2) {
#pragma unroll
    for (int q = 0; q < V / 2; q++) {
      const CDF a = v[2 * q], b = v[2 * q + 1];
      v[2 * q] = cl_add(a, b);
      v[2 * q + 1] = cl_sub(a, b);
    }
  } else if constexpr (R == 4) {
    dft4<S, 0, 1>(v);
    dft4<S, 4, 1>(v);
    if constexpr (V == 16) {
      dft4<S, 8, 1>(v);
      dft4<S, 12, 1>(v);
    }
  } else {
    dft8<S, 0>(v);
    if constexpr (V == 16) dft8<S, 8>(v);
  }
}

template <int S> __device__ __forceinline__ float4 twiddle(const float4 *__restrict__ tw, int e) {
  float4 w = __ldg(tw + e);
  if (S > 0) { w.z = -w.z; w.w = -w.w; }
  return w;
}

template <int S, int R, int V>
__device__ __forceinline__ void fft_last(CDF *buf, CDF (&v)[V], int t, int T, int L, const float4 *__restrict__ tw) {
  // L R = m: butterfly j (< L) reads and writes j + u L, twiddles w^(u j)
#pragma unroll
  for (int q = 0; q < V / R; q++) {
    const int j = t + q * T;
#pragma unroll
    for (int u = 0; u < R; u++) {
      CDF x = buf[padv<V>(j + u * L)];
      if (u > 0 && j > 0) x = cl_mul(x, twiddle<S>(tw, u * j));
      v[q * R + u] = x;
    }
  }
  dft_small<S, R, V>(v);
#pragma unroll
  for (int q = 0; q < V / R; q++) {
    const int j = t + q * T;
#pragma unroll
    for (int u = 0; u < R; u++) buf[padv<V>(j + u * L)] = cl_norm(v[q * R + u]);
  }
}

// Transform of one row: v holds the inputs x[t + u T] of thread t on entry; on
// exit the spectrum is in buf (padded layout) and visible to the whole CTA.
template <int S, int V>
__device__ void fft_row(CDF *buf, CDF (&v)[V], int t, int T, int m, const float4 *__restrict__ tw) {
  constexpr int LGV = V == 16 ? 4 : 3;
  dft_full<S, V>(v);
  __syncthreads();
#pragma unroll
  for (int u = 0; u < V; u++) buf[padv<V>(V * t + u)] = cl_norm(v[u]);
  __syncthreads();
  int L = V, lgL = LGV;
  while (L * V <= m) {
    const int k = t & (L - 1), blk = t >> lgL;
    const int tws = m >> (lgL + LGV);
#pragma unroll
    for (int u = 0; u < V; u++) {
      CDF x = buf[padv<V>(t + u * T)];
      if (u > 0 && k > 0) x = cl_mul(x, twiddle<S>(tw, u * k * tws));
      v[u] = x;
    }
    dft_full<S, V>(v);
    __syncthreads();
    const int o = blk * L * V + k;
#pragma unroll
    for (int u = 0; u < V; u++) buf[padv<V>(o + u * L)] = cl_norm(v[u]);
    __syncthreads();
    L <<= LGV;
    lgL += LGV;
  }
  const int R = m / L;
  if (R > 1) {
    if (R == 2) fft_last<S, 2, V>(buf, v, t, T, L, tw);
    else if (R == 4) fft_last<S, 4, V>(buf, v, t, T, L, tw);
    else if constexpr (V == 16) fft_last<S, 8, V>(buf, v, t, T, L, tw);
    __syncthreads();
  }
}

struct FftShape {
  int T, lgT, rows;   // threads per row, log2 T, rows per CTA
};

// values per thread of the register-radix transforms
constexpr int FFT_V = 8;
constexpr int FFT_CTA = 128;

// RHS + DCT-II of rows (compute_potential.c:70-92), register-radix transform
template <int V>
__global__ void __launch_bounds__(FFT_CTA, 8) k_dct2_dfr(Dct2ArgsDF a, FftShape sh) {
  extern __shared__ float4 sm4[];
  const int n = a.itot, m = n / 2, ld = a.ld;
  const int T = sh.T;
  const int rloc = threadIdx.x >> sh.lgT, t = threadIdx.x & (T - 1);
  const int jr = blockIdx.x * sh.rows + rloc;
  const bool live = jr < a.jtot;
  const int j = 1 + jr;
  CDF *buf = reinterpret_cast<CDF *>(sm4) + rloc * (m + m / V);
  DF *vq = reinterpret_cast<DF *>(buf);
  if (live) {
    // (1/(gamma dt)) / dx and (1/(gamma dt)) / dy
    const DF inv = DF{__ldg(a.coef + 12 + 2 * a.rk), __ldg(a.coef + 13 + 2 * a.rk)};
    const DF ax = df_mul(inv, a.rdx), ay = df_mul(inv, a.rdy);
#pragma unroll 4
    for (int i0 = t; i0 < n; i0 += T) {
      const int i = i0 + 1;
      // differences of neighbouring doubles (exact), split into float pairs
      const float2 sx = eifd::split(__ldg(a.ux + ux_idx(i + 1, j, ld)) - __ldg(a.ux + ux_idx(i, j, ld)));
      const float2 sy = eifd::split(__ldg(a.uy + uy_idx(i, j + 1, ld)) - __ldg(a.uy + uy_idx(i, j, ld)));
      DF dux_ = DF{sx.x, sx.y}, duy_ = DF{sy.x, sy.y};
      if (a.with_ibm) {
        // (u + (d0 + de)/2) - (u + (dw + d0)/2) with single-precision field values:
        // the increments (de - dw)/2 and (en - ds)/2 as exact float sums
        const int c = uy_idx(i, j, ld);
        const float dw = (i >= 2) ? __ldg(a.dux + c - 1) : -__ldg(a.dux + c);
        const float de = (i + 1 <= n) ? __ldg(a.dux + c + 1) : -__ldg(a.dux + c);
        dux_ = dfl_add(dux_, df_scale(two_sum(de, -dw), 0.5f));
        duy_ = dfl_add(duy_, df_scale(two_sum(__ldg(a.duy + c + ld), -__ldg(a.duy + c - ld)), 0.5f));
      }
      // Makhoul order: q[2t] -> v[t], q[2t + 1] -> v[n - 1 - t]
      const int vpos = (i0 & 1) ? n - 1 - (i0 >> 1) : (i0 >> 1);
      const DF q = dfl_add(dfl_mulc(dux_, ax), dfl_mulc(duy_, ay));
      vq[vpos] = fast_sum(q.hi, q.lo);
    }
  }
  __syncthreads();
  CDF v[V];
#pragma unroll
  for (int u = 0; u < V; u++) v[u] = buf[t + u * T];   // z[s] = v[2s] + i v[2s+1], unpadded
  fft_row<-1, V>(buf, v, t, T, m, a.tw);
  if (!live) return;
  double *out = a.qhat + (size_t)jr * ld;
#pragma unroll 2
  for (int kk = t; kk <= m; kk += T) {
    const CDF zk = buf[padv<V>(kk & (m - 1))];
    const CDF zm = cdf_conj(buf[padv<V>((m - kk) & (m - 1))]);
    const CDF sm = cl_add(zk, zm), df = cl_sub(zk, zm);
    const CDF e = CDF{df_scale(sm.re, 0.5f), df_scale(sm.im, 0.5f)};
    const CDF o = CDF{df_scale(df.im, 0.5f), df_scale(df_neg(df.re), 0.5f)};  // (zk - zm) / 2i
    const CDF vv = cl_add(e, cl_mul(o, __ldg(a.wn + kk)));
    // rot[kk] = (c, s); rot[n - kk] = -i conj(rot[kk]) = (-s, -c)
    const float4 r = __ldg(a.rot + kk);
    const DF rc = DF{r.x, r.y}, rs = DF{r.z, r.w};
    const DF o0 = df_scale(dfl_dot2(rc, vv.re, rs, vv.im, -1.f), 2.f);
    const DF o1 = df_scale(dfl_dot2(rs, vv.re, rc, vv.im, 1.f), -2.f);
    const bool pair = kk > 0 && kk < m;
    if (a.qdf) {
      float2 *outf = reinterpret_cast<float2 *>(out);
      const DF n0 = fast_sum(o0.hi, o0.lo);
      outf[kk] = make_float2(n0.hi, n0.lo);
      if (pair) {
        const DF n1 = fast_sum(o1.hi, o1.lo);
        outf[n - kk] = make_float2(n1.hi, n1.lo);
      }
    } else {
      out[kk] = df_to_double(o0);
      if (pair) out[n - kk] = df_to_double(o1);
    }
  }
}

// block reconstruction + DCT-III + scaling of rows, register-radix transform
template <int V>
__global__ void __launch_bounds__(FFT_CTA, 8) k_dct3_dfr(Dct3ArgsDF a, FftShape sh) {
  extern __shared__ float4 sm4[];
  const int n = a.itot, m = n / 2, ld = a.ld;
  const int T = sh.T;
  const int rloc = threadIdx.x >> sh.lgT, t = threadIdx.x & (T - 1);
  const int jr = blockIdx.x * sh.rows + rloc;
  const bool live = jr < a.jtot;
  const int j = 1 + jr;
  CDF *buf = reinterpret_cast<CDF *>(sm4) + rloc * (m + m / V);
  DF *xr = reinterpret_cast<DF *>(buf);
  if (live) {
    const double *row = a.qhat + (size_t)jr * ld;
    if (a.blk > 0) {
      const int M = a.blk;
      const int b = jr / M, r = jr % M;
      const int bm = (b + a.nblk - 1) % a.nblk;
#pragma unroll 4
      for (int k = t; k < n; k += T) {
        DF val;
        if (r == M - 1) {
          val = df_of(__ldg(a.iface + (size_t)b * n + k));
        } else {
          // y + s_left g + s_right h in double-float from the double-precision block solution
          const float2 gl = __ldg(a.g + (size_t)r * n + k);
          const float2 gr = __ldg(a.g + (size_t)(M - 2 - r) * n + k);
          const float2 y = a.qdf ? __ldg(reinterpret_cast<const float2 *>(row) + k) : eifd::split(__ldg(row + k));
          const float2 sl = eifd::split(__ldg(a.iface + (size_t)bm * n + k));
          const float2 sr = eifd::split(__ldg(a.iface + (size_t)b * n + k));
          const DF acc = dfl_add(dfl_add(DF{y.x, y.y}, dfl_mulc(DF{sl.x, sl.y}, DF{gl.x, gl.y})),
                                 dfl_mulc(DF{sr.x, sr.y}, DF{gr.x, gr.y}));
          val = fast_sum(acc.hi, acc.lo);
        }
        xr[k] = val;
      }
    } else {
      for (int k = t; k < n; k += T) {
        if (a.qdf) {
          const float2 q = __ldg(reinterpret_cast<const float2 *>(row) + k);
          xr[k] = DF{q.x, q.y};
        } else {
          xr[k] = df_of(__ldg(row + k));
        }
      }
    }
  }
  __syncthreads();
  CDF v[V];
#pragma unroll
  for (int u = 0; u < V; u++) {
    const int s = t + u * T;
    const int t0 = s, t1 = s + m;
    float4 r0 = __ldg(a.rot + t0), r1 = __ldg(a.rot + t1), wn = __ldg(a.wn + s);
    r0.z = -r0.z; r0.w = -r0.w;
    r1.z = -r1.z; r1.w = -r1.w;
    wn.z = -wn.z; wn.w = -wn.w;
    const CDF w0 = cl_mul(CDF{xr[t0], t0 == 0 ? DF{0.f, 0.f} : df_neg(xr[n - t0])}, r0);
    const CDF w1 = cl_mul(CDF{xr[t1], df_neg(xr[n - t1])}, r1);
    const CDF sum = cl_add(w0, w1);
    const CDF dif = cl_mul(cl_sub(w0, w1), wn);
    v[u] = CDF{dfl_sub(sum.re, dif.im), dfl_add(sum.im, dif.re)};
  }
  fft_row<1, V>(buf, v, t, T, m, a.tw);
  if (!live) return;
  double *prow = a.psi + (size_t)j * ld;
  for (int i = t; i < n; i += T) {
    const int tt = (i & 1) ? n - 1 - (i >> 1) : (i >> 1);
    const CDF zz = buf[padv<V>(tt >> 1)];
    const DF w = (tt & 1) ? zz.im : zz.re;
    const double val = df_to_double(dfl_mulc(w, a.scale));
    prow[i + 1] = val;
    if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld + i + 1] = val;
    if (j == a.jtot) a.psi[i + 1] = val;
    if (i == 0) {
      prow[0] = val;
      if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld] = val;
      if (j == a.jtot) a.psi[0] = val;
    }
    if (i == n - 1) {
      prow[n + 1] = val;
      if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld + n + 1] = val;
      if (j == a.jtot) a.psi[n + 1] = val;
    }
  }
}

// Interior Thomas solve of one block in double-float arithmetic (mixed form): the
// right-hand side and the block solution are (hi, lo) float pairs in the qhat
// buffer, the pivots 1/d_i and modified upper diagonals are float-pair tables, and
// the two values the reduced system needs are written in double. The blocks are
// diagonally dominant (|c| >= 2 l), so the recurrences carry the pairs' 2^-48
// relative error without amplification.
template <int M>
__global__ void __launch_bounds__(256) k_tdm_local_df(float2 *__restrict__ qhat, const float2 *__restrict__ inv,
                                                     const float2 *__restrict__ up, double *__restrict__ iface_a,
                                                     double *__restrict__ first, DF l, int itot, int nblk, int ld) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (k >= itot) return;
  DF v[M - 1];
  const size_t base = (size_t)b * M * ld + k;
#pragma unroll
  for (int r = 0; r < M - 1; r++) {
    const float2 t = qhat[base + (size_t)r * ld];
    v[r] = DF{t.x, t.y};
  }
  const float2 rif = qhat[base + (size_t)(M - 1) * ld];
  {
    const float2 iv = __ldg(inv + k);
    const DF t = dfl_mulc(v[0], DF{iv.x, iv.y});
    v[0] = fast_sum(t.hi, t.lo);
  }
#pragma unroll
  for (int r = 1; r < M - 1; r++) {
    const float2 iv = __ldg(inv + r * itot + k);
    const DF t = dfl_mulc(dfl_sub(v[r], dfl_mulc(v[r - 1], l)), DF{iv.x, iv.y});
    v[r] = fast_sum(t.hi, t.lo);
  }
#pragma unroll
  for (int r = M - 3; r >= 0; r--) {
    const float2 u = __ldg(up + r * itot + k);
    const DF t = dfl_sub(v[r], dfl_mulc(v[r + 1], DF{u.x, u.y}));
    v[r] = fast_sum(t.hi, t.lo);
  }
#pragma unroll
  for (int r = 0; r < M - 1; r++) qhat[base + (size_t)r * ld] = make_float2(v[r].hi, v[r].lo);
  // interface equation: r_iface - l y[M-2] (this block) - l y[0] (next block)
  iface_a[(size_t)b * itot + k] = df_to_double(dfl_sub(DF{rif.x, rif.y}, dfl_mulc(v[M - 2], l)));
  first[(size_t)b * itot + k] = df_to_double(v[0]);
}

// ---------------------------------------------------------------------------
// Single-precision solve with one refinement (mixed form, power-of-two half lengths
// with the block tridiagonal solver). The Poisson equation L psi = q (q the
// divergence of u** over gamma dt, compute_potential.c:70-134) is solved twice with
// single-precision transforms and block Thomas sweeps (the reduced cyclic systems of
// the interface values stay in double precision):
//   pass 1: L psi1 = q,               psi1 stored as float
//   pass 2: L psi2 = q - L psi1,      the residual formed in double-float arithmetic
//                                      from the exact double differences of u** and the
//                                      float values of psi1
// and psi = psi1 + psi2 is kept as the float pair (psi1, psi2). A single-precision
// solve leaves a residual of about 1e-6 (smooth right-hand sides: 1e-2) of |q|; the
// refinement solves for that residual and leaves about 1e-12 (1e-8).
struct CF { float re, im; };
__device__ __forceinline__ CF cf_add(CF a, CF b) { return CF{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ CF cf_sub(CF a, CF b) { return CF{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ CF cf_mul(CF a, float2 w) {
  return CF{fmaf(a.re, w.x, -a.im * w.y), fmaf(a.re, w.y, a.im * w.x)};
}
template <int S> __device__ __forceinline__ CF cf_mul_si(CF a) { return S > 0 ? CF{-a.im, a.re} : CF{a.im, -a.re}; }
// multiplication by exp(S i pi/4) = (sqrt(2)/2)(1 + S i)
template <int S> __device__ __forceinline__ CF cf_mul_w8(CF a) {
  const float h = 0.70710678118654752f;
  return S > 0 ? CF{(a.re - a.im) * h, (a.im + a.re) * h} : CF{(a.re + a.im) * h, (a.im - a.re) * h};
}
// radix-4 butterfly on v[o], v[o + st], v[o + 2 st], v[o + 3 st], outputs in natural order
template <int S, int O, int ST, int N> __device__ __forceinline__ void dft4_f(CF (&v)[N]) {
  const CF s02 = cf_add(v[O], v[O + 2 * ST]), d02 = cf_sub(v[O], v[O + 2 * ST]);
  const CF s13 = cf_add(v[O + ST], v[O + 3 * ST]), d13 = cf_mul_si<S>(cf_sub(v[O + ST], v[O + 3 * ST]));
  v[O] = cf_add(s02, s13);
  v[O + ST] = cf_add(d02, d13);
  v[O + 2 * ST] = cf_sub(s02, s13);
  v[O + 3 * ST] = cf_sub(d02, d13);
}
// 8-point DFT of v (sign S), result in natural order (n = 2 n1 + n2, k = k1 + 4 k2)
template <int S> __device__ __forceinline__ void dft8_f(CF (&v)[8]) {
  dft4_f<S, 0, 2>(v);
  dft4_f<S, 1, 2>(v);
  v[3] = cf_mul_w8<S>(v[3]);
  v[5] = cf_mul_si<S>(v[5]);
  v[7] = cf_mul_si<S>(cf_mul_w8<S>(v[7]));
  CF w[8];
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    w[k1] = cf_add(v[2 * k1], v[2 * k1 + 1]);
    w[k1 + 4] = cf_sub(v[2 * k1], v[2 * k1 + 1]);
  }
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = w[k];
}
// The single-precision transforms are instantiated for each power-of-two half length
// m = 2^LGM (8 <= m <= 8 FFT_CTA): thread counts, pass lengths and strides are compile-time
// constants, so the shared-memory offsets are immediates. The twiddles are read from a
// table laid out in pass order (pass_twiddles below): for the radix-8 pass of length L,
// butterfly k reads its seven twiddles w^(u k m / 8L), u = 1..7, as consecutive values.
constexpr int ilog2c(int x) { return x <= 1 ? 0 : 1 + ilog2c(x / 2); }
// offset of the twiddles of the radix-8 pass of length L (L = 8, 64, ...) in the table;
// the last pass's twiddles follow those of all radix-8 passes
constexpr int twp_off(int L) { return L <= 8 ? 0 : twp_off(L / 8) + 7 * (L / 8); }
__device__ __forceinline__ int padv8(int i) { return i + (i >> 3); }
template <int S> __device__ __forceinline__ float2 twiddle_p(const float2 *__restrict__ p) {
  float2 w = __ldg(p);
  if (S > 0) w.y = -w.y;
  return w;
}
// the last pass of radix R = 2 or 4 (L = M / R): butterfly j = t + q T (q < 8/R) reads and
// writes j + u L; its twiddles w^(u j), u = 1..R-1, are twp[(R-1) j + u - 1]
template <int S, int R, int M>
__device__ __forceinline__ void fft_last_f(CF *buf, CF (&v)[8], int t, const float2 *__restrict__ twp) {
  constexpr int T = M / 8, L = M / R, SL = L + L / 8;
  static_assert(L % 8 == 0, "the last pass follows a radix-8 pass");
#pragma unroll
  for (int q = 0; q < 8 / R; q++) {
    const int j = t + q * T;
    const int jb = padv8(j);
#pragma unroll
    for (int u = 0; u < R; u++) {
      CF x = buf[jb + u * SL];
      if (u > 0 && j > 0) x = cf_mul(x, twiddle_p<S>(twp + (R - 1) * j + u - 1));
      v[q * R + u] = x;
    }
  }
  if constexpr (R == 2) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const CF a = v[2 * q], b = v[2 * q + 1];
      v[2 * q] = cf_add(a, b);
      v[2 * q + 1] = cf_sub(a, b);
    }
  } else {
    dft4_f<S, 0, 1>(v);
    dft4_f<S, 4, 1>(v);
  }
#pragma unroll
  for (int q = 0; q < 8 / R; q++) {
    const int jb = padv8(t + q * T);
#pragma unroll
    for (int u = 0; u < R; u++) buf[jb + u * SL] = v[q * R + u];
  }
}
// the Stockham passes from length L on: radix 8 while 8 L <= M, then radix M / L
template <int S, int M, int L>
__device__ __forceinline__ void fft_passes_f(CF *buf, CF (&v)[8], int t, const float2 *__restrict__ twp) {
  constexpr int T = M / 8;
  if constexpr (L * 8 <= M) {
    static_assert(T % 8 == 0 && L % 8 == 0, "radix-8 passes need 8 | T and 8 | L");
    constexpr int LG = ilog2c(L), ST = T + T / 8, SL = L + L / 8;
    const int k = t & (L - 1), blk = t >> LG;
    const float2 *w = twp + twp_off(L) + 7 * k;
    const int ib = padv8(t);
#pragma unroll
    for (int u = 0; u < 8; u++) {
      CF x = buf[ib + u * ST];
      if (u > 0 && k > 0) x = cf_mul(x, twiddle_p<S>(w + u - 1));
      v[u] = x;
    }
    dft8_f<S>(v);
    __syncthreads();
    const int ob = padv8(blk * L * 8 + k);
#pragma unroll
    for (int u = 0; u < 8; u++) buf[ob + u * SL] = v[u];
    __syncthreads();
    fft_passes_f<S, M, L * 8>(buf, v, t, twp);
  } else if constexpr (M / L > 1) {
    fft_last_f<S, M / L, M>(buf, v, t, twp + twp_off(L));
    __syncthreads();
  }
}
// Stockham transform of one row of M = 8 T values (radix-8 passes, then radix 2 or 4):
// v holds the inputs x[t + u T] of thread t on entry; on exit the spectrum is in buf
// (padded layout) and visible to the whole CTA
template <int S, int M>
__device__ void fft_row_f(CF *buf, CF (&v)[8], int t, const float2 *__restrict__ twp) {
  dft8_f<S>(v);
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 8; u++) buf[9 * t + u] = v[u];   // padded index of 8 t + u
  __syncthreads();
  fft_passes_f<S, M, 8>(buf, v, t, twp);
}

struct Dct2ArgsF {
  const double *ux, *uy;
  const float *dux, *duy;   // IBM field response in single precision
  const float *coef;        // [12 + 2 rk], [13 + 2 rk]: 1/(gamma dt) as a float pair
  const float *psi1;        // refinement pass: the first solution (uy layout), else null
  float2 *qdf;              // q as (hi, lo) pairs: written by the first pass, read by the second
  float *q;                 // transformed right-hand side, rows of pitch ld floats
  const float2 *tw, *rot, *wn;   // tw: twiddles in pass order (pass_twiddles)
  DF rdx, rdy, rdx2, rdy2;  // 1/dx, 1/dy, 1/dx^2, 1/dy^2
  int itot, jtot, ld, with_ibm, rk;
};

// right-hand side (or the residual of the first solution) + single-precision DCT-II
// of rows; one row of m = itot/2 complex values per T = m/8 threads
// (itot = 2 m, m = 2^LGM); capped at 32 registers for 16 resident CTAs per SM: measured
// faster than 40 registers and 12 CTAs
template <int LGM>
__global__ void __launch_bounds__(FFT_CTA, 16) k_dct2_f(Dct2ArgsF a) {
  extern __shared__ float4 sm4[];
  constexpr int m = 1 << LGM, n = 2 * m, T = m / 8, ROWS = FFT_CTA / T;
  const int ld = a.ld;
  const int rloc = threadIdx.x >> (LGM - 3), t = threadIdx.x & (T - 1);
  const int jr = blockIdx.x * ROWS + rloc;
  const bool live = jr < a.jtot;
  const int j = 1 + jr;
  CF *buf = reinterpret_cast<CF *>(sm4) + rloc * (m + m / 8);
  float *vq = reinterpret_cast<float *>(buf);
  if (live && !a.psi1) {
    // (1/(gamma dt)) / dx and (1/(gamma dt)) / dy
    const DF inv = DF{__ldg(a.coef + 12 + 2 * a.rk), __ldg(a.coef + 13 + 2 * a.rk)};
    const DF ax = df_mul(inv, a.rdx), ay = df_mul(inv, a.rdy);
    float2 *qrow = a.qdf + (size_t)jr * ld;
#pragma unroll 4
    for (int i0 = t; i0 < n; i0 += T) {
      const int i = i0 + 1;
      const int c = uy_idx(i, j, ld);
      // differences of neighbouring doubles as float pairs, from their integer splits
      // (no double arithmetic): exact leading parts, trailing parts to 2^-48 of |u|
      const float2 ue = eifd::split(__ldg(a.ux + ux_idx(i + 1, j, ld))), uw = eifd::split(__ldg(a.ux + ux_idx(i, j, ld)));
      const float2 vn = eifd::split(__ldg(a.uy + c + ld)), vs = eifd::split(__ldg(a.uy + c));
      DF dux_ = dfl_sub(DF{ue.x, ue.y}, DF{uw.x, uw.y}), duy_ = dfl_sub(DF{vn.x, vn.y}, DF{vs.x, vs.y});
      if (a.with_ibm) {
        // (u + (d0 + de)/2) - (u + (dw + d0)/2): the increments (de - dw)/2, (en - ds)/2
        const float dw = (i >= 2) ? __ldg(a.dux + c - 1) : -__ldg(a.dux + c);
        const float de = (i + 1 <= n) ? __ldg(a.dux + c + 1) : -__ldg(a.dux + c);
        dux_ = dfl_add(dux_, df_scale(two_sum(de, -dw), 0.5f));
        duy_ = dfl_add(duy_, df_scale(two_sum(__ldg(a.duy + c + ld), -__ldg(a.duy + c - ld)), 0.5f));
      }
      const DF qq = dfl_add(dfl_mulc(dux_, ax), dfl_mulc(duy_, ay));
      const DF q = fast_sum(qq.hi, qq.lo);
      qrow[i0] = make_float2(q.hi, q.lo);
      // Makhoul order: q[2t] -> v[t], q[2t + 1] -> v[n - 1 - t]
      vq[(i0 & 1) ? n - 1 - (i0 >> 1) : (i0 >> 1)] = q.hi;
    }
  } else if (live) {
    // residual q - L psi1: the first differences of float neighbours are exact pairs
    const float2 *qrow = a.qdf + (size_t)jr * ld;
#pragma unroll 4
    for (int i0 = t; i0 < n; i0 += T) {
      const int c = uy_idx(i0 + 1, j, ld);
      const float2 qv = __ldg(qrow + i0);
      const float p0 = __ldg(a.psi1 + c);
      const DF dxx = dfl_sub(two_sum(__ldg(a.psi1 + c + 1), -p0), two_sum(p0, -__ldg(a.psi1 + c - 1)));
      const DF dyy = dfl_sub(two_sum(__ldg(a.psi1 + c + ld), -p0), two_sum(p0, -__ldg(a.psi1 + c - ld)));
      const DF r = dfl_sub(DF{qv.x, qv.y}, dfl_add(dfl_mulc(dxx, a.rdx2), dfl_mulc(dyy, a.rdy2)));
      vq[(i0 & 1) ? n - 1 - (i0 >> 1) : (i0 >> 1)] = r.hi + r.lo;
    }
  }
  __syncthreads();
  CF v[8];
#pragma unroll
  for (int u = 0; u < 8; u++) v[u] = buf[t + u * T];   // z[s] = v[2s] + i v[2s+1], unpadded
  fft_row_f<-1, m>(buf, v, t, a.tw);
  if (!live) return;
  float *out = a.q + (size_t)jr * ld;
#pragma unroll 2
  for (int kk = t; kk <= m; kk += T) {
    const CF zk = buf[padv<8>(kk & (m - 1))];
    const CF zm0 = buf[padv<8>((m - kk) & (m - 1))];
    const CF zm = CF{zm0.re, -zm0.im};
    const CF sm = cf_add(zk, zm), df = cf_sub(zk, zm);
    const CF e = CF{0.5f * sm.re, 0.5f * sm.im};
    const CF o = CF{0.5f * df.im, -0.5f * df.re};   // (zk - zm) / 2i
    const CF vv = cf_add(e, cf_mul(o, __ldg(a.wn + kk)));
    // rot[kk] = (c, s); rot[n - kk] = -i conj(rot[kk]) = (-s, -c)
    const float2 r = __ldg(a.rot + kk);
    out[kk] = 2.f * fmaf(r.x, vv.re, -r.y * vv.im);
    if (kk > 0 && kk < m) out[n - kk] = -2.f * fmaf(r.y, vv.re, r.x * vv.im);
  }
}

// block Thomas sweep of one block and wavenumber column in single precision (the
// blocks are diagonally dominant); the two values the reduced system needs in double
template <int M>
__global__ void __launch_bounds__(256) k_tdm_local_f(float *__restrict__ q, const float *__restrict__ inv,
                                                    const float *__restrict__ up, double *__restrict__ iface_a,
                                                    double *__restrict__ first, float l, int itot, int nblk, int ld) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (k >= itot) return;
  float v[M - 1];
  const size_t base = (size_t)b * M * ld + k;
#pragma unroll
  for (int r = 0; r < M - 1; r++) v[r] = q[base + (size_t)r * ld];
  const float rif = q[base + (size_t)(M - 1) * ld];
  v[0] = v[0] * __ldg(inv + k);
#pragma unroll
  for (int r = 1; r < M - 1; r++) v[r] = fmaf(-l, v[r - 1], v[r]) * __ldg(inv + r * itot + k);
#pragma unroll
  for (int r = M - 3; r >= 0; r--) v[r] = fmaf(-__ldg(up + r * itot + k), v[r + 1], v[r]);
#pragma unroll
  for (int r = 0; r < M - 1; r++) q[base + (size_t)r * ld] = v[r];
  // interface equation: r_iface - l y[M-2] (this block) - l y[0] (next block)
  iface_a[(size_t)b * itot + k] = eifd::f2d(fmaf(-l, v[M - 2], rif));
  first[(size_t)b * itot + k] = eifd::f2d(v[0]);
}

struct Dct3ArgsF {
  const float *q;        // block solutions, rows of pitch ld floats
  const float *iface;    // solved interface values [block][k], rounded to float by the reduced solve
  const float *g;        // left responses of the block interior [r][k]
  float *psi;            // output (uy layout, with halo rows and ghost columns)
  const float2 *tw, *rot, *wn;   // tw: twiddles in pass order (pass_twiddles)
  float scale;           // 1/(2 itot)
  int itot, jtot, ld, blk, nblk;
};

// block reconstruction + single-precision DCT-III + scaling of rows (compute_potential.c:120-134)
// (itot = 2 m, m = 2^LGM); capped at 48 registers for 10 resident CTAs per SM: measured
// faster than 53 registers and 9 CTAs
template <int LGM>
__global__ void __launch_bounds__(FFT_CTA, 10) k_dct3_f(Dct3ArgsF a) {
  extern __shared__ float4 sm4[];
  constexpr int m = 1 << LGM, n = 2 * m, T = m / 8, ROWS = FFT_CTA / T;
  const int ld = a.ld;
  const int rloc = threadIdx.x >> (LGM - 3), t = threadIdx.x & (T - 1);
  const int jr = blockIdx.x * ROWS + rloc;
  const bool live = jr < a.jtot;
  const int j = 1 + jr;
  CF *buf = reinterpret_cast<CF *>(sm4) + rloc * (m + m / 8);
  float *xr = reinterpret_cast<float *>(buf);
  if (live) {
    const float *row = a.q + (size_t)jr * ld;
    const int M = a.blk;
    const int b = jr / M, r = jr % M;
    const int bm = (b + a.nblk - 1) % a.nblk;
#pragma unroll 4
    for (int k = t; k < n; k += T) {
      float val;
      if (r == M - 1) {
        val = __ldg(a.iface + (size_t)b * n + k);
      } else {
        // y + s_left g + s_right h (h = g reversed, the blocks are symmetric)
        const float gl = __ldg(a.g + (size_t)r * n + k), gr = __ldg(a.g + (size_t)(M - 2 - r) * n + k);
        const float sl = __ldg(a.iface + (size_t)bm * n + k);
        const float sr = __ldg(a.iface + (size_t)b * n + k);
        val = fmaf(sr, gr, fmaf(sl, gl, __ldg(row + k)));
      }
      xr[k] = val;
    }
  }
  __syncthreads();
  CF v[8];
#pragma unroll
  for (int u = 0; u < 8; u++) {
    const int s = t + u * T;
    const int t0 = s, t1 = s + m;
    float2 r0 = __ldg(a.rot + t0), r1 = __ldg(a.rot + t1), wn = __ldg(a.wn + s);
    r0.y = -r0.y;
    r1.y = -r1.y;
    wn.y = -wn.y;
    const CF w0 = cf_mul(CF{xr[t0], t0 == 0 ? 0.f : -xr[n - t0]}, r0);
    const CF w1 = cf_mul(CF{xr[t1], -xr[n - t1]}, r1);
    const CF sum = cf_add(w0, w1);
    const CF dif = cf_mul(cf_sub(w0, w1), wn);
    v[u] = CF{sum.re - dif.im, sum.im + dif.re};
  }
  fft_row_f<1, m>(buf, v, t, a.tw);
  if (!live) return;
  float *prow = a.psi + (size_t)j * ld;
  for (int i = t; i < n; i += T) {
    const int tt = (i & 1) ? n - 1 - (i >> 1) : (i >> 1);
    const CF zz = buf[padv<8>(tt >> 1)];
    const float val = ((tt & 1) ? zz.im : zz.re) * a.scale;
    prow[i + 1] = val;
    if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld + i + 1] = val;
    if (j == a.jtot) a.psi[i + 1] = val;
    if (i == 0) {
      prow[0] = val;
      if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld] = val;
      if (j == a.jtot) a.psi[0] = val;
    }
    if (i == n - 1) {
      prow[n + 1] = val;
      if (j == 1) a.psi[(size_t)(a.jtot + 1) * ld + n + 1] = val;
      if (j == a.jtot) a.psi[n + 1] = val;
    }
  }
}

// psi as doubles: psi1 + psi2 (float pair) or the double field itself
__global__ void k_psi_pair_to_double(const float *__restrict__ p1, const float *__restrict__ p2,
                                     double *__restrict__ out, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    out[t] = eifd::f2d(p1[t]) + eifd::f2d(p2[t]);
}

// launch shape of the register-radix transforms, or T = 0 when m is not supported
// (not a power of two, or more than FFT_CTA threads per row)
FftShape fftr_shape(int m) {
  FftShape s{0, 0, 0};
  if (m < FFT_V || m > FFT_V * FFT_CTA || (m & (m - 1)) != 0) return s;
  s.T = m / FFT_V;
  while ((1 << s.lgT) < s.T) s.lgT++;
  s.rows = FFT_CTA / s.T;
  return s;
}
size_t fftr_smem(int m, int rows) { return sizeof(float4) * (size_t)rows * (m + m / FFT_V); }

// The twiddles w^e (w = exp(-2 pi i / m), tw[e] for e < m) of the single-precision
// transforms in the order fft_passes_f reads them: for each radix-8 pass of length
// L = 8, 64, ... (8 L <= m) and each butterfly k < L the seven values w^(u k m / 8L),
// u = 1..7; then, when the last pass has radix R = m / L > 1, for each butterfly j < L
// the R - 1 values w^(u j). Values are copied, not recomputed: the transforms read the
// same floats as from tw itself.
std::vector<float2> pass_twiddles(const std::vector<float2> &tw, int m) {
  std::vector<float2> out;
  int L = 8;
  for (; L * 8 <= m; L *= 8)
    for (int k = 0; k < L; k++)
      for (int u = 1; u < 8; u++) out.push_back(tw[(size_t)u * k * (m / (8 * L))]);
  const int R = m / L;
  if (R > 1)
    for (int j = 0; j < L; j++)
      for (int u = 1; u < R; u++) out.push_back(tw[(size_t)u * j]);
  if (out.empty()) out.push_back(tw[0]);   // m = 8: one radix-8 stage, no twiddles
  return out;
}

bool factorize(int m, int *fac, int *nfac) {
  int k = 0;
  while (m % 4 == 0) { fac[k++] = 4; m /= 4; }
  while (m % 2 == 0) { fac[k++] = 2; m /= 2; }
  while (m % 3 == 0) { fac[k++] = 3; m /= 3; }
  *nfac = k;
  return m == 1 && k <= 16;
}

// Thomas factors of a constant-coefficient tridiagonal matrix of size n
void thomas_factors(int n, double l, double c, double *inv, double *up) {
  inv[0] = 1. / c;
  up[0] = l * inv[0];
  for (int i = 1; i < n; i++) {
    inv[i] = 1. / (c - l * up[i - 1]);
    up[i] = l * inv[i];
  }
}

void thomas_apply(int n, double l, const double *inv, const double *up, double *q) {
  q[0] = q[0] * inv[0];
  for (int i = 1; i < n; i++) q[i] = (q[i] - l * q[i - 1]) * inv[i];
  for (int i = n - 2; i >= 0; i--) q[i] = q[i] - up[i] * q[i + 1];
}

}  // namespace

namespace eif {

int poisson_init(eif_ctx *c) {
  PoissonPlan &pp = c->pp;
  const int n = c->itot, jt = c->jtot;
  if (n % 2 != 0) return fail(c, EIF_ERR_ARG, "itot must be even (got %d)", n);
  pp.n = n;
  pp.m = n / 2;
  if (!factorize(pp.m, pp.fac, &pp.nfac)) return fail(c, EIF_ERR_ARG, "itot/2 must be of the form 2^a 3^b (got %d)", pp.m);
  const long double PI = 3.141592653589793238462643383279502884L;
  std::vector<double2> tw(pp.m), rot(n), wn(n);
  for (int k = 0; k < pp.m; k++) {
    const long double t = -2.L * PI * k / pp.m;
    tw[k] = make_double2((double)cosl(t), (double)sinl(t));
  }
  for (int k = 0; k < n; k++) {
    const long double h = -PI * k / (2.L * n);
    rot[k] = make_double2((double)cosl(h), (double)sinl(h));
    const long double t = -2.L * PI * k / n;
    wn[k] = make_double2((double)cosl(t), (double)sinl(t));
  }
  // tridiagonal coefficients (compute_potential.c:103-112)
  const double dx = c->dx, dy = c->dy;
  const double l = 1. / dy / dy;
  std::vector<double> lam(n);
  for (int k = 0; k < n; k++) {
    const double s = sin(M_PI * k / (2. * n));
    lam[k] = -4. / (dx * dx) * (s * s);
  }
  pp.blk = 0;
  pp.nblk = 1;
  const int cand[3] = {EIF_TDM_M, 8, 4};
  for (int ci = 0; ci < 3; ci++) {
    if (jt % cand[ci] == 0 && jt / cand[ci] >= 3) { pp.blk = cand[ci]; pp.nblk = jt / cand[ci]; break; }
  }
  auto up_load = [&](void **dst, const void *src, size_t bytes) -> cudaError_t {
    cudaError_t e = cudaMalloc(dst, bytes);
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
  };
  EIF_CK(c, up_load((void **)&pp.tw, tw.data(), sizeof(double2) * pp.m));
  {
    // the same twiddles as float pairs for the double-float (mixed-precision) transforms
    auto pair = [&](long double t) {
      const float hi = (float)t;
      return std::make_pair(hi, (float)(t - (long double)hi));
    };
    auto df_table = [&](int len, long double step, float4 **dst) -> int {
      std::vector<float4> v(len);
      for (int k = 0; k < len; k++) {
        const auto re = pair(cosl(step * k)), im = pair(sinl(step * k));
        v[k] = make_float4(re.first, re.second, im.first, im.second);
      }
      EIF_CK(c, up_load((void **)dst, v.data(), sizeof(float4) * len));
      return EIF_OK;
    };
    int rc;
    if ((rc = df_table(pp.m, -2.L * PI / pp.m, &pp.tw_f))) return rc;
    if ((rc = df_table(n, -PI / (2.L * n), &pp.rot_f))) return rc;
    if ((rc = df_table(n, -2.L * PI / n, &pp.wn_f))) return rc;
    // single-precision twiddles of the refined solve, rounded from long double
    auto f_values = [&](int len, long double step) {
      std::vector<float2> v(len);
      for (int k = 0; k < len; k++) v[k] = make_float2((float)cosl(step * k), (float)sinl(step * k));
      return v;
    };
    auto f_table = [&](int len, long double step, float2 **dst) -> int {
      const std::vector<float2> v = f_values(len, step);
      EIF_CK(c, up_load((void **)dst, v.data(), sizeof(float2) * len));
      return EIF_OK;
    };
    {
      const std::vector<float2> tw = pass_twiddles(f_values(pp.m, -2.L * PI / pp.m), pp.m);
      EIF_CK(c, up_load((void **)&pp.tw2, tw.data(), sizeof(float2) * tw.size()));
    }
    if ((rc = f_table(n, -PI / (2.L * n), &pp.rot2))) return rc;
    if ((rc = f_table(n, -2.L * PI / n, &pp.wn2))) return rc;
  }
  EIF_CK(c, up_load((void **)&pp.rot, rot.data(), sizeof(double2) * n));
  EIF_CK(c, up_load((void **)&pp.wn, wn.data(), sizeof(double2) * n));
  EIF_CK(c, up_load((void **)&pp.lam, lam.data(), sizeof(double) * n));
  if (pp.blk > 0) {
    const int M = pp.blk, P = pp.nblk;
    std::vector<double> inv((size_t)(M - 1) * n), up((size_t)(M - 1) * n), g((size_t)(M - 1) * n);
    std::vector<double> rinv((size_t)P * n), rup((size_t)P * n), rq1((size_t)P * n), rcoef((size_t)4 * n);
    std::vector<double> ti(M), tu(M), tg(M), ri(P), ru(P), rq(P);
    // second level: groups of G2 (16, 8 or 4) with 3 <= Q2 = P / G2 <= 32, smallest G2 + Q2
    int G2 = 0, Q2 = 0;
    for (int gsz : {16, 8, 4}) {
      if (P % gsz != 0) continue;
      const int q = P / gsz;
      if (q < 3 || q > 32) continue;
      if (G2 == 0 || gsz + q < G2 + Q2) { G2 = gsz; Q2 = q; }
    }
    pp.g2 = G2;
    pp.q2 = Q2;
    const size_t l2 = G2 > 0 ? (size_t)std::max(G2, Q2) * n : 1;
    std::vector<double> inv2(l2), up2(l2), phi2(l2), ri2(l2), ru2(l2), rq2(l2), rc2(G2 > 0 ? (size_t)4 * n : 1);
    std::vector<double> t2i(std::max(G2, 1)), t2u(std::max(G2, 1)), t2g(std::max(G2, 1));
    std::vector<double> q2i(std::max(Q2, 1)), q2u(std::max(Q2, 1)), q2q(std::max(Q2, 1));
    for (int k = 0; k < n; k++) {
      const double cc = -l - l + lam[k];
      thomas_factors(M - 1, l, cc, ti.data(), tu.data());
      for (int i = 0; i < M - 1; i++) tg[i] = 0.;
      tg[0] = -l;
      thomas_apply(M - 1, l, ti.data(), tu.data(), tg.data());
      for (int i = 0; i < M - 1; i++) {
        inv[(size_t)i * n + k] = ti[i];
        up[(size_t)i * n + k] = tu[i];
        g[(size_t)i * n + k] = tg[i];
      }
      // reduced cyclic system A s_{b-1} + B s_b + A s_{b+1} = R_b
      const double A = l * tg[M - 2];
      const double B = cc + 2. * l * tg[0];
      thomas_factors(P - 1, A, B, ri.data(), ru.data());
      for (int b = 0; b < P - 1; b++) rq[b] = 0.;
      rq[0] = -A;
      rq[P - 2] += -A;
      thomas_apply(P - 1, A, ri.data(), ru.data(), rq.data());
      for (int b = 0; b < P - 1; b++) {
        rinv[(size_t)b * n + k] = ri[b];
        rup[(size_t)b * n + k] = ru[b];
        rq1[(size_t)b * n + k] = rq[b];
      }
      rcoef[4 * k + 0] = A;
      rcoef[4 * k + 1] = B;
      rcoef[4 * k + 2] = B + A * rq[0] + A * rq[P - 2];
      rcoef[4 * k + 3] = k == 0 ? 1. : 0.;
      if (G2 > 0) {
        // second level: interior factors and left response of a group, then the
        // cyclic system of the Q second-level interface values
        thomas_factors(G2 - 1, A, B, t2i.data(), t2u.data());
        for (int i = 0; i < G2 - 1; i++) t2g[i] = 0.;
        t2g[0] = -A;
        thomas_apply(G2 - 1, A, t2i.data(), t2u.data(), t2g.data());
        for (int i = 0; i < G2 - 1; i++) {
          inv2[(size_t)i * n + k] = t2i[i];
          up2[(size_t)i * n + k] = t2u[i];
          phi2[(size_t)i * n + k] = t2g[i];
        }
        const double A2 = A * t2g[G2 - 2];
        const double B2 = B + 2. * A * t2g[0];
        thomas_factors(Q2 - 1, A2, B2, q2i.data(), q2u.data());
        for (int q = 0; q < Q2 - 1; q++) q2q[q] = 0.;
        q2q[0] = -A2;
        q2q[Q2 - 2] += -A2;
        thomas_apply(Q2 - 1, A2, q2i.data(), q2u.data(), q2q.data());
        for (int q = 0; q < Q2 - 1; q++) {
          ri2[(size_t)q * n + k] = q2i[q];
          ru2[(size_t)q * n + k] = q2u[q];
          rq2[(size_t)q * n + k] = q2q[q];
        }
        rc2[4 * k + 0] = A2;
        rc2[4 * k + 1] = B2;
        rc2[4 * k + 2] = B2 + A2 * q2q[0] + A2 * q2q[Q2 - 2];
        rc2[4 * k + 3] = k == 0 ? 1. : 0.;
      }
    }
    EIF_CK(c, up_load((void **)&pp.tdm_inv, inv.data(), sizeof(double) * inv.size()));
    EIF_CK(c, up_load((void **)&pp.tdm_up, up.data(), sizeof(double) * up.size()));
    EIF_CK(c, up_load((void **)&pp.tdm_g, g.data(), sizeof(double) * g.size()));
    {
      std::vector<float2> gdf(g.size());
      for (size_t q = 0; q < g.size(); q++) {
        const float hi = (float)g[q];
        gdf[q] = make_float2(hi, (float)(g[q] - (double)hi));
      }
      EIF_CK(c, up_load((void **)&pp.tdm_g_df, gdf.data(), sizeof(float2) * gdf.size()));
      auto pairs = [](const std::vector<double> &v) {
        std::vector<float2> o(v.size());
        for (size_t q = 0; q < v.size(); q++) {
          const float hi = (float)v[q];
          o[q] = make_float2(hi, (float)(v[q] - (double)hi));
        }
        return o;
      };
      const std::vector<float2> invdf = pairs(inv), updf = pairs(up);
      EIF_CK(c, up_load((void **)&pp.tdm_inv_df, invdf.data(), sizeof(float2) * invdf.size()));
      EIF_CK(c, up_load((void **)&pp.tdm_up_df, updf.data(), sizeof(float2) * updf.size()));
      const std::vector<float> invf(inv.begin(), inv.end()), upf(up.begin(), up.end()), gf(g.begin(), g.end());
      EIF_CK(c, up_load((void **)&pp.tdm_inv_f, invf.data(), sizeof(float) * invf.size()));
      EIF_CK(c, up_load((void **)&pp.tdm_up_f, upf.data(), sizeof(float) * upf.size()));
      EIF_CK(c, up_load((void **)&pp.tdm_g_f, gf.data(), sizeof(float) * gf.size()));
    }
    EIF_CK(c, up_load((void **)&pp.red_inv, rinv.data(), sizeof(double) * rinv.size()));
    EIF_CK(c, up_load((void **)&pp.red_up, rup.data(), sizeof(double) * rup.size()));
    EIF_CK(c, up_load((void **)&pp.red_q1, rq1.data(), sizeof(double) * rq1.size()));
    EIF_CK(c, up_load((void **)&pp.red_coef, rcoef.data(), sizeof(double) * rcoef.size()));
    if (G2 > 0) {
      EIF_CK(c, up_load((void **)&pp.r2_inv, inv2.data(), sizeof(double) * l2));
      EIF_CK(c, up_load((void **)&pp.r2_up, up2.data(), sizeof(double) * l2));
      EIF_CK(c, up_load((void **)&pp.r2_phi, phi2.data(), sizeof(double) * l2));
      EIF_CK(c, up_load((void **)&pp.r2_qinv, ri2.data(), sizeof(double) * l2));
      EIF_CK(c, up_load((void **)&pp.r2_qup, ru2.data(), sizeof(double) * l2));
      EIF_CK(c, up_load((void **)&pp.r2_q1, rq2.data(), sizeof(double) * l2));
      EIF_CK(c, up_load((void **)&pp.r2_coef, rc2.data(), sizeof(double) * rc2.size()));
    }
    EIF_CK(c, cudaMalloc((void **)&pp.ywork, sizeof(double) * 2 * (size_t)P * n));
  } else {
    EIF_CK(c, cudaMalloc((void **)&pp.ywork, sizeof(double) * 2 * (size_t)jt * n));
  }
  const int rcols = red_cols(pp.blk > 0 ? pp.nblk : 1);
  if (rcols == 0) return fail(c, EIF_ERR_ARG, "jtot %d needs too many tridiagonal blocks", jt);
  const size_t red_smem = red_smem_bytes(pp.blk > 0 ? pp.nblk : 1, rcols);
  if (red_smem > 48 * 1024) {
    EIF_CK(c, cudaFuncSetAttribute(k_tdm_reduced, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)red_smem));
  }
  const size_t smem = sizeof(double2) * 2 * pp.m + sizeof(double) * n;
  if (smem > 48 * 1024) {
    EIF_CK(c, cudaFuncSetAttribute(k_dct2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    EIF_CK(c, cudaFuncSetAttribute(k_dct3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    EIF_CK(c, cudaFuncSetAttribute(k_dct2_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    EIF_CK(c, cudaFuncSetAttribute(k_dct3_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  {
    const FftShape sh = fftr_shape(pp.m);
    const size_t smr = sh.T > 0 ? fftr_smem(pp.m, sh.rows) : 0;
    if (smr > 48 * 1024) {
      EIF_CK(c, cudaFuncSetAttribute(k_dct2_dfr<FFT_V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr));
      EIF_CK(c, cudaFuncSetAttribute(k_dct3_dfr<FFT_V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr));
    }
    // the refined single-precision solve: power-of-two half lengths with the block solver
    c->psi_pair = c->cfg.precision == EIF_PREC_MIXED && sh.T > 0 && pp.blk > 0;
    if (c->psi_pair) {
      EIF_CK(c, cudaMalloc((void **)&pp.qdf, sizeof(float2) * (size_t)c->ld * jt));
      EIF_CK(c, cudaMalloc((void **)&pp.iface_f, sizeof(float) * (size_t)pp.nblk * n));
    }
  }
  return EIF_OK;
}

void poisson_free(eif_ctx *c) {
  PoissonPlan &pp = c->pp;
  void *ptrs[] = {pp.r2_inv, pp.r2_up, pp.r2_phi, pp.r2_qinv, pp.r2_qup, pp.r2_q1, pp.r2_coef,
                  pp.tw, pp.rot, pp.wn, pp.tw_f, pp.rot_f, pp.wn_f, pp.lam, pp.tdm_inv, pp.tdm_up, pp.tdm_g, pp.tdm_g_df, pp.tdm_inv_df, pp.tdm_up_df,
                  pp.red_inv, pp.red_up, pp.red_q1, pp.red_coef, pp.ywork, pp.tw2, pp.rot2, pp.wn2, pp.tdm_inv_f,
                  pp.tdm_up_f, pp.tdm_g_f, pp.qdf, pp.iface_f};
  for (void *p : ptrs) if (p) cudaFree(p);
  pp = PoissonPlan{};
}

static int fft_threads(int m) { return m >= 512 ? 256 : (m >= 128 ? 128 : 64); }

// the reduced cyclic systems of the interface values (double precision), in place in iface
static int reduced_solve(eif_ctx *c, double *iface, double *first, float *iface_f) {
  PoissonPlan &pp = c->pp;
  const int n = c->itot;
  const double l = 1. / c->dy / c->dy;
  if (pp.g2 > 0) {
    const int Q = pp.q2;
    const size_t sm = red2_smem_bytes(Q);
    const dim3 grid((n + RED2_K - 1) / RED2_K);
    if (pp.g2 == 16) {
      k_tdm_reduced2<16><<<grid, RED2_K * Q, sm, c->stream>>>(iface, first, pp.red_coef, pp.r2_inv, pp.r2_up, pp.r2_phi,
                                                          pp.r2_qinv, pp.r2_qup, pp.r2_q1, pp.r2_coef, l, n, pp.nblk, Q,
                                                         iface_f);
    } else if (pp.g2 == 8) {
      k_tdm_reduced2<8><<<grid, RED2_K * Q, sm, c->stream>>>(iface, first, pp.red_coef, pp.r2_inv, pp.r2_up, pp.r2_phi,
                                                         pp.r2_qinv, pp.r2_qup, pp.r2_q1, pp.r2_coef, l, n, pp.nblk, Q,
                                                         iface_f);
    } else {
      k_tdm_reduced2<4><<<grid, RED2_K * Q, sm, c->stream>>>(iface, first, pp.red_coef, pp.r2_inv, pp.r2_up, pp.r2_phi,
                                                         pp.r2_qinv, pp.r2_qup, pp.r2_q1, pp.r2_coef, l, n, pp.nblk, Q,
                                                         iface_f);
    }
  } else {
    const int rcols = red_cols(pp.nblk);
    k_tdm_reduced<<<(n + rcols - 1) / rcols, RED_THREADS, red_smem_bytes(pp.nblk, rcols), c->stream>>>(
        iface, first, pp.red_inv, pp.red_up, pp.red_q1, pp.red_coef, l, n, pp.nblk, rcols, iface_f);
  }
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

// one launch of the single-precision DCT-II (a) or DCT-III (b) instance for m = 2^lgm
static void launch_dct_f(int lgm, unsigned blocks, size_t smem, cudaStream_t s, const Dct2ArgsF *a,
                         const Dct3ArgsF *b) {
#define EIF_DCT_F_CASE(L)                                          \
  case L:                                                          \
    if (a) k_dct2_f<L><<<blocks, FFT_CTA, smem, s>>>(*a);          \
    else k_dct3_f<L><<<blocks, FFT_CTA, smem, s>>>(*b);            \
    break;
  switch (lgm) {
    EIF_DCT_F_CASE(3) EIF_DCT_F_CASE(4) EIF_DCT_F_CASE(5) EIF_DCT_F_CASE(6)
    EIF_DCT_F_CASE(7) EIF_DCT_F_CASE(8) EIF_DCT_F_CASE(9) EIF_DCT_F_CASE(10)
    default: break;
  }
#undef EIF_DCT_F_CASE
}

// the mixed form's Poisson solve: two single-precision passes, the second on the
// double-float residual of the first (see k_dct2_f); psi1, psi2 into the psi buffer
static int potential_refined(eif_ctx *c, int rk, bool with_ibm) {
  PoissonPlan &pp = c->pp;
  const int n = c->itot, jt = c->jtot;
  const FftShape sh = fftr_shape(pp.m);
  static_assert(FFT_V * FFT_CTA == 1 << 10, "instances of the single-precision transforms: m = 2^3 .. 2^10");
  const int lgm = sh.lgT + 3;   // m = 8 T, T = 2^lgT
  const size_t smem = sizeof(CF) * (size_t)sh.rows * (pp.m + pp.m / 8);
  auto dfpair = [](double v) {
    const float hi = (float)v;
    return DF{hi, (float)(v - (double)hi)};
  };
  float *qf = reinterpret_cast<float *>(c->qhat);
  float *psi1 = reinterpret_cast<float *>(c->psi), *psi2 = psi1 + c->nfield;
  double *iface = pp.ywork;
  double *first = pp.ywork + (size_t)pp.nblk * n;
  const float lf = (float)(1. / c->dy / c->dy);
  const int tt = c->tiles.tdm;
  const dim3 gt((n + tt - 1) / tt, pp.nblk);
  const unsigned blocks = (unsigned)((jt + sh.rows - 1) / sh.rows);
  for (int pass = 0; pass < 2; pass++) {
    Dct2ArgsF a;
    a.ux = c->ux[c->cur]; a.uy = c->uy[c->cur];
    a.dux = reinterpret_cast<const float *>(c->dux); a.duy = reinterpret_cast<const float *>(c->duy);
    a.coef = c->d_coef;
    a.psi1 = pass ? psi1 : nullptr;
    a.qdf = pp.qdf;
    a.q = qf;
    a.tw = pp.tw2; a.rot = pp.rot2; a.wn = pp.wn2;
    a.rdx = dfpair(1. / c->dx); a.rdy = dfpair(1. / c->dy);
    a.rdx2 = dfpair(1. / (c->dx * c->dx)); a.rdy2 = dfpair(1. / (c->dy * c->dy));
    a.itot = n; a.jtot = jt; a.ld = c->ld; a.with_ibm = with_ibm ? 1 : 0; a.rk = rk;
    {
      EIF_PROF(c, "poisson_dct2", 1);
      launch_dct_f(lgm, blocks, smem, c->stream, &a, nullptr);
      EIF_LAUNCH_CK(c);
    }
    {
      EIF_PROF(c, "poisson_tdm", 2);
      if (pp.blk == 16) {
        k_tdm_local_f<16><<<gt, tt, 0, c->stream>>>(qf, pp.tdm_inv_f, pp.tdm_up_f, iface, first, lf, n, pp.nblk, c->ld);
      } else if (pp.blk == 8) {
        k_tdm_local_f<8><<<gt, tt, 0, c->stream>>>(qf, pp.tdm_inv_f, pp.tdm_up_f, iface, first, lf, n, pp.nblk, c->ld);
      } else {
        k_tdm_local_f<4><<<gt, tt, 0, c->stream>>>(qf, pp.tdm_inv_f, pp.tdm_up_f, iface, first, lf, n, pp.nblk, c->ld);
      }
      EIF_LAUNCH_CK(c);
      int rc = reduced_solve(c, iface, first, pp.iface_f);
      if (rc) return rc;
    }
    Dct3ArgsF b;
    b.q = qf; b.iface = pp.iface_f; b.g = pp.tdm_g_f;
    b.psi = pass ? psi2 : psi1;
    b.tw = pp.tw2; b.rot = pp.rot2; b.wn = pp.wn2;
    b.scale = (float)(1. / (2. * n));
    b.itot = n; b.jtot = jt; b.ld = c->ld; b.blk = pp.blk; b.nblk = pp.nblk;
    EIF_PROF(c, "poisson_dct3", 1);
    launch_dct_f(lgm, blocks, smem, c->stream, nullptr, &b);
    EIF_LAUNCH_CK(c);
  }
  return EIF_OK;
}

int launch_psi_to_double(eif_ctx *c, double *dst) {
  if (!c->psi_pair) {
    EIF_CK(c, cudaMemcpyAsync(dst, c->psi, sizeof(double) * c->nfield, cudaMemcpyDeviceToDevice, c->stream));
    return EIF_OK;
  }
  const float *p1 = reinterpret_cast<const float *>(c->psi);
  k_psi_pair_to_double<<<c->sms * 4, 256, 0, c->stream>>>(p1, p1 + c->nfield, dst, c->nfield);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

int launch_potential(eif_ctx *c, int rk, bool with_ibm) {
  PoissonPlan &pp = c->pp;
  const int n = c->itot, jt = c->jtot;
  FftDesc fd;
  fd.m = pp.m;
  fd.nfac = pp.nfac;
  for (int s = 0; s < 16; s++) fd.fac[s] = pp.fac[s];
  const size_t smem = sizeof(double2) * 2 * pp.m + sizeof(double) * n;
  const int thr = fft_threads(pp.m);
  const bool mixed = c->cfg.precision == EIF_PREC_MIXED;
  auto dfpair = [](double v) {
    const float hi = (float)v;
    return DF{hi, (float)(v - (double)hi)};
  };
  if (c->psi_pair) return potential_refined(c, rk, with_ibm);
  if (mixed) {
    Dct2ArgsDF a;
    a.ux = c->ux[c->cur]; a.uy = c->uy[c->cur];
    a.dux = reinterpret_cast<const float *>(c->dux); a.duy = reinterpret_cast<const float *>(c->duy);
    a.coef = c->d_coef;
    a.qhat = c->qhat;
    a.tw = pp.tw_f; a.rot = pp.rot_f; a.wn = pp.wn_f;
    a.fd = fd;
    a.rdx = dfpair(1. / c->dx); a.rdy = dfpair(1. / c->dy);
    a.itot = n; a.jtot = jt; a.ld = c->ld; a.with_ibm = with_ibm ? 1 : 0; a.rk = rk;
    a.qdf = pp.blk > 0 ? 1 : 0;   // the block solver reads and writes float pairs
    EIF_PROF(c, "poisson_dct2", 1);
    const FftShape sh = fftr_shape(pp.m);
    if (sh.T > 0) {
      k_dct2_dfr<FFT_V><<<(jt + sh.rows - 1) / sh.rows, sh.T * sh.rows, fftr_smem(pp.m, sh.rows), c->stream>>>(a, sh);
    } else {
      k_dct2_df<<<jt, thr, smem, c->stream>>>(a);
    }
    EIF_LAUNCH_CK(c);
  } else {
    Dct2Args a;
    a.ux = c->ux[c->cur]; a.uy = c->uy[c->cur];
    a.dux = c->dux; a.duy = c->duy; a.dt = c->d_scal;
    a.qhat = c->qhat;
    a.tw = pp.tw; a.rot = pp.rot; a.wn = pp.wn;
    a.fd = fd;
    a.gamma = rk_coef(rk).gamma;
    a.rdx = 1. / c->dx; a.rdy = 1. / c->dy;
    a.itot = n; a.jtot = jt; a.ld = c->ld; a.with_ibm = with_ibm ? 1 : 0;
    a.rhs = c->adj_rhs;
    EIF_PROF(c, "poisson_dct2", 1);
    k_dct2<<<jt, thr, smem, c->stream>>>(a);
    EIF_LAUNCH_CK(c);
  }
  const double l = 1. / c->dy / c->dy;
  double *iface = pp.ywork;
  double *first = pp.ywork + (size_t)pp.nblk * n;
  if (pp.blk > 0) {
    EIF_PROF(c, "poisson_tdm", 2);
    // one thread per wavenumber column; the threads per block come from the tuner
    const int tt = c->tiles.tdm;
    dim3 g((n + tt - 1) / tt, pp.nblk);
    if (mixed) {
      float2 *qf = reinterpret_cast<float2 *>(c->qhat);
      const DF ldf = dfpair(l);
      if (pp.blk == 16) {
        k_tdm_local_df<16><<<g, tt, 0, c->stream>>>(qf, pp.tdm_inv_df, pp.tdm_up_df, iface, first, ldf, n, pp.nblk, c->ld);
      } else if (pp.blk == 8) {
        k_tdm_local_df<8><<<g, tt, 0, c->stream>>>(qf, pp.tdm_inv_df, pp.tdm_up_df, iface, first, ldf, n, pp.nblk, c->ld);
      } else {
        k_tdm_local_df<4><<<g, tt, 0, c->stream>>>(qf, pp.tdm_inv_df, pp.tdm_up_df, iface, first, ldf, n, pp.nblk, c->ld);
      }
    } else if (pp.blk == 16) {
      k_tdm_local<16><<<g, tt, 0, c->stream>>>(c->qhat, pp.tdm_inv, pp.tdm_up, iface, first, l, n, pp.nblk, c->ld);
    } else if (pp.blk == 8) {
      k_tdm_local<8><<<g, tt, 0, c->stream>>>(c->qhat, pp.tdm_inv, pp.tdm_up, iface, first, l, n, pp.nblk, c->ld);
    } else {
      k_tdm_local<4><<<g, tt, 0, c->stream>>>(c->qhat, pp.tdm_inv, pp.tdm_up, iface, first, l, n, pp.nblk, c->ld);
    }
    EIF_LAUNCH_CK(c);
    if (pp.g2 > 0) {
      const int Q = pp.q2;
      const size_t sm = red2_smem_bytes(Q);
      const dim3 grid((n + RED2_K - 1) / RED2_K);
      if (pp.g2 == 16) {
        k_tdm_reduced2<16><<<grid, RED2_K * Q, sm, c->stream>>>(iface, first, pp.red_coef, pp.r2_inv, pp.r2_up, pp.r2_phi,
                                                            pp.r2_qinv, pp.r2_qup, pp.r2_q1, pp.r2_coef, l, n,
                                                            pp.nblk, Q, nullptr);
      } else if (pp.g2 == 8) {
        k_tdm_reduced2<8><<<grid, RED2_K * Q, sm, c->stream>>>(iface, first, pp.red_coef, pp.r2_inv, pp.r2_up, pp.r2_phi,
                                                           pp.r2_qinv, pp.r2_qup, pp.r2_q1, pp.r2_coef, l, n,
                                                           pp.nblk, Q, nullptr);
      } else {
        k_tdm_reduced2<4><<<grid, RED2_K * Q, sm, c->stream>>>(iface, first, pp.red_coef, pp.r2_inv, pp.r2_up, pp.r2_phi,
                                                           pp.r2_qinv, pp.r2_qup, pp.r2_q1, pp.r2_coef, l, n,
                                                           pp.nblk, Q, nullptr);
      }
    } else {
      const int rcols = red_cols(pp.nblk);
      k_tdm_reduced<<<(n + rcols - 1) / rcols, RED_THREADS, red_smem_bytes(pp.nblk, rcols), c->stream>>>(
          iface, first, pp.red_inv, pp.red_up, pp.red_q1, pp.red_coef, l, n, pp.nblk, rcols, nullptr);
    }
    EIF_LAUNCH_CK(c);
  } else {
    EIF_PROF(c, "poisson_tdm", 1);
    k_tdm_serial<<<(n + 63) / 64, 64, 0, c->stream>>>(c->qhat, pp.ywork, pp.lam, l, n, jt, c->ld);
    EIF_LAUNCH_CK(c);
  }
  if (mixed) {
    Dct3ArgsDF a;
    a.qhat = c->qhat; a.iface = iface; a.g = pp.tdm_g_df;
    a.psi = c->psi;
    a.tw = pp.tw_f; a.rot = pp.rot_f; a.wn = pp.wn_f;
    a.fd = fd;
    a.scale = dfpair(1. / (2. * n));
    a.itot = n; a.jtot = jt; a.ld = c->ld; a.blk = pp.blk; a.nblk = pp.nblk;
    a.qdf = pp.blk > 0 ? 1 : 0;
    EIF_PROF(c, "poisson_dct3", 1);
    const FftShape sh = fftr_shape(pp.m);
    if (sh.T > 0) {
      k_dct3_dfr<FFT_V><<<(jt + sh.rows - 1) / sh.rows, sh.T * sh.rows, fftr_smem(pp.m, sh.rows), c->stream>>>(a, sh);
    } else {
      k_dct3_df<<<jt, thr, smem, c->stream>>>(a);
    }
    EIF_LAUNCH_CK(c);
  } else {
    Dct3Args a;
    a.qhat = c->qhat; a.iface = iface; a.g = pp.tdm_g;
    a.psi = c->psi;
    a.tw = pp.tw; a.rot = pp.rot; a.wn = pp.wn;
    a.fd = fd;
    a.itot = n; a.jtot = jt; a.ld = c->ld; a.blk = pp.blk; a.nblk = pp.nblk;
    EIF_PROF(c, "poisson_dct3", 1);
    k_dct3<<<jt, thr, smem, c->stream>>>(a);
    EIF_LAUNCH_CK(c);
  }
  return EIF_OK;
}

}  // namespace eif
