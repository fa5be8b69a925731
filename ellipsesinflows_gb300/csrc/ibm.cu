// Immersed-boundary kernels: smoothed indicator, momentum exchange and the
// volume integrals of the particle interiors.
//
// Reference functions restated here (NaokiHori/EllipsesInFlows):
//   suspensions_decide_loop_size   src/suspensions/auxiliary.c:11-17
//   compute_signed_dist            src/suspensions/auxiliary.c:19-47
//   suspensions_s_weight/v_weight  src/suspensions/auxiliary.c:51-59
//   mass, moment of inertia        src/suspensions/auxiliary.c:63-75
//   find_normal_t, compute_ex/ey   src/ellipse.c:7-65
//   kernel_exchange_momentum       src/suspensions/exchange.c:13-88
//   compute_inertia                src/suspensions/inertia.c:9-70
//
// Work decomposition. For every particle the reference visits, for the
// periodic images -1, 0, +1, the cells of a clipped bounding box. Here every
// box row is one task (rows wider than CHUNK cells are cut into segments of
// CHUNK cells); tasks are numbered in the reference's (image, j, i) order. One
// warp evaluates one task (two cells per lane) inside a persistent grid sized
// to the SM count, so particles of any size keep all SMs busy. Per-particle sums are reduced per chunk with warp shuffles and
// then per particle over its chunks in a fixed order: results are
// deterministic. The momentum exchange also stores each box cell's field
// contribution in a scratch buffer; a tile gather then adds, for every cell,
// the contributions of all covering boxes in (particle, image) order, which
// is the reference's accumulation order (exchange.c:71-72), without atomics.
#ifndef EIF_CHECK
#define EIF_CHECK 1
#endif
#include "eif_internal.cuh"
#include <cfloat>
#include <vector>
#include <algorithm>
#include <cmath>

namespace {

constexpr int CHUNK = 64;       // cells per warp task (a box row, or a segment of one)
__device__ __host__ __forceinline__ int box_segs(int w) { return (w + CHUNK - 1) / CHUNK; }
constexpr int NEXTRA = 3;       // auxiliary.c:8
constexpr double BETA = 2.;     // auxiliary.c:49
constexpr int GTX = 128, GTY = 8, GTHREADS = 256;  // gather tile and block
constexpr int GCOLS = 64;   // columns covered by the threads of one pass (GTX / GCOLS passes)
constexpr int LMAX = 256;       // gather entries staged in shared memory at a time (GTHREADS)

// per-particle geometry needed by a box cell evaluation
struct Ell {
  double a, b, px, py, cz, sz;   // semi-axes, centre, cos(-az), sin(-az)
  double kex, key, ab2;          // a(1-(b/a)^2), b(1-(a/b)^2), a*a+b*b
};

__device__ __forceinline__ Ell make_ell(double a, double b, double px, double py, double az) {
  Ell e;
  e.a = a; e.b = b; e.px = px; e.py = py;
  sincos(-az, &e.sz, &e.cz);
  e.kex = a * (1. - (b / a) * (b / a));
  e.key = b * (1. - (a / b) * (a / b));
  e.ab2 = a * a + b * b;
  return e;
}

// ellipse.c:30-65 (x_, y_ in the body frame)
__device__ __forceinline__ double normal_t(const Ell &e, double x_, double y_) {
  const double px = fabs(x_), py = fabs(y_);
  double t = 0.25 * M_PI;
  for (int n = 0;; n++) {
    double st, ct;
    sincos(t, &st, &ct);
    const double x = e.a * ct, y = e.b * st;
    const double ex = e.kex * (ct * ct * ct);
    const double ey = e.key * (st * st * st);
    const double rx = x - ex, ry = y - ey;
    const double qx = px - ex, qy = py - ey;
    const double r = sqrt(ry * ry + rx * rx);
    const double q = sqrt(qy * qy + qx * qx);
    const double dc = r * asin((rx * qy - ry * qx) / (r * q));
    const double dt = dc / sqrt(e.ab2 - x * x - y * y);
    t += dt;
    t = fmin(0.5 * M_PI, t);
    t = fmax(0., t);
    if (fabs(dt) < 1.e-8) break;
    if (n > EIF_NORMAL_MAX_ITER - 1) break;
  }
  if (x_ < 0.) t = M_PI - t;
  if (y_ < 0.) t = -t;
  return t;
}

// auxiliary.c:19-47, in units of the grid size h (rh = 1/h), from the body-frame
// offset (x_, y_) = R(-az) (x - px, y - py)
__device__ __forceinline__ double signed_dist_body(const Ell &e, double x_, double y_, double rh) {
  const double f0 = 1. - (x_ / e.a) * (x_ / e.a) - (y_ / e.b) * (y_ / e.b);
  const double sign = f0 > 0. ? 1. : -1.;
  const double t = normal_t(e, x_, y_);
  double st, ct;
  sincos(t, &st, &ct);
  const double dxx = e.a * ct - x_, dyy = e.b * st - y_;
  return sign * sqrt(dxx * dxx + dyy * dyy) * rh;
}

// Cells far from the interface. With rho = sqrt((x/a)^2 + (y/b)^2) (the gauge of
// the ellipse, Lipschitz with constant 1/min(a,b)) the distance to the boundary is
// at least min(a,b) |rho - 1|, and at least r - max(a,b) outside / min(a,b) - r
// inside (r = |(x, y)|). When that bound times 2/h reaches the value at which
// tanh rounds to +-1 in the working precision, the weights are exactly those of
// the saturated tanh and the normal-foot iteration is not needed. row_chords
// turns these bounds into column ranges of a box row.
//
// double-precision tanh(2d) equals +-1 exactly for |2d| >= 20 (the correction
// 2/(exp(2|x|)+1) is below half an ulp of 1); with a margin for rounding of the bound
constexpr double FAR_CELLS_D = 10.5;
constexpr float FAR_CELLS_F = 5.f;

// auxiliary.c:11-17
__device__ __forceinline__ void loop_size(int lb, int ub, double h, double r, double gc, int &mn, int &mx) {
  mn = (int)(floor((gc - r) / h) - NEXTRA);
  mx = (int)(ceil((gc + r) / h) + NEXTRA);
  mn = mn < lb ? lb : mn;
  mx = mx > ub ? ub : mx;
}

__device__ __forceinline__ double pmass(double den, double a, double b) { return den * (M_PI * a * b); }
__device__ __forceinline__ double pmoi(double den, double a, double b) {
  return 0.25 * pmass(den, a, b) * (a * a + b * b);
}

// sizes of the buffers the IBM kernels touch (used by EIF_CHECK builds)
struct Bounds {
  long long P, box, off, partial, wbuf, field, xc, yc;
  unsigned long long *rec;
};

// Per-particle single-precision parameters of the mixed-precision indicator,
// PF_WORDS words per particle (see k_boxes).
constexpr int PF_WORDS = 28;
enum { PF_A, PF_B, PF_CZ, PF_SZ, PF_KEX, PF_KEY, PF_RPM, PF_RPIM, PF_UX, PF_UY, PF_VZ, PF_GX, PF_I0,
       PF_J0, PF_GY = PF_J0 + 3,
       // quadratic form of the ellipse in the lab frame and the far-cell scales (row_chords)
       PF_AL = PF_GY + 3, PF_KA, PF_DE, PF_SO2, PF_SI2, PF_RO2 };
static_assert(PF_RO2 < PF_WORDS && PF_WORDS % 4 == 0, "per-particle parameter block");

struct BoxArgs {
  const double *P;
  int pcap, np, itot, jtot, use_increment;
  double dx, dy, ly, yf1;
  float *pf;                // PF_WORDS per particle, or null (double-precision form)
  int *box, *nchunk;
  const int *bd_off_base;   // start of the buffer nchunk points into
  // inside the sub-iteration loop of a step graph: the loop's counter. In the first
  // sub-iteration the increments are zero, the positions are X and the boxes built at
  // X before the loop are still in place, so the box kernels return at once.
  const unsigned *iter;
  Bounds bd;
};

// Per-particle boxes of the three periodic images and their task counts, and the
// single-precision parameters. The double-precision work of one particle is a long
// chain (divisions, sincos) and the FP64 pipe takes a warp instruction at a time, so
// the work is split into eight parts run by different warps (grid row blockIdx.y),
// each over 32 particles: rows 0-2 the boxes of images -1, 0, +1 (their task counts
// are added to nchunk, zeroed before the launch), rows 3-7 groups of parameters
// (mixed form only).
constexpr int BOX_PARTS = 8;
__global__ void __launch_bounds__(32) k_boxes(BoxArgs a) {
  if (a.iter && *a.iter == 0u) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int sub = blockIdx.y;
  const double *P = a.P;
  const int pc = a.pcap;
  bool on = n < a.np;
  if (on && !EIF_CHK(a.bd.rec, EIF_P_DY * pc + n, a.bd.P, 1)) on = false;
  int tasks = 0;
  if (on) {
    const double pa = P[EIF_P_A * pc + n], pb = P[EIF_P_B * pc + n];
    double px = P[EIF_P_X * pc + n], py = P[EIF_P_Y * pc + n];
    if (a.use_increment) {
      px = px + P[EIF_P_DX * pc + n];
      py = py + P[EIF_P_DY * pc + n];
    }
    const double r = fmax(pa, pb);
    float *q = a.pf ? a.pf + (size_t)PF_WORDS * n : nullptr;
    if (sub < 3) {
      const int per = sub - 1;
      int imin, imax, jmin, jmax;
      loop_size(1, a.itot, a.dx, r, px, imin, imax);
      loop_size(1, a.jtot, a.dy, r, py + a.ly * per - a.yf1, jmin, jmax);
      if (EIF_CHK(a.bd.rec, 12 * n + 4 * sub + 3, a.bd.box, 2)) {
        int *bx = a.box + 12 * n + 4 * sub;
        bx[0] = imin; bx[1] = imax; bx[2] = jmin; bx[3] = jmax;
        if (imax >= imin && jmax >= jmin) tasks = (jmax - jmin + 1) * box_segs(imax - imin + 1);
      }
    } else if (q && sub == 3) {
      // orientation and the quadratic form rho^2 = al X^2 + 2 ka X Y + de Y^2 of the
      // ellipse for lab-frame offsets (X, Y)
      double az = P[EIF_P_AZ * pc + n];
      if (a.use_increment) az = az + P[EIF_P_DAZ * pc + n];
      double sz, cz;
      sincos(-az, &sz, &cz);
      q[PF_CZ] = (float)cz;
      q[PF_SZ] = (float)sz;
      q[PF_AL] = (float)(cz * cz / (pa * pa) + sz * sz / (pb * pb));
      q[PF_KA] = (float)(cz * sz * (1. / (pb * pb) - 1. / (pa * pa)));
      q[PF_DE] = (float)(sz * sz / (pa * pa) + cz * cz / (pb * pb));
    } else if (q && sub == 4) {
      q[PF_A] = (float)pa;
      q[PF_B] = (float)pb;
      q[PF_KEX] = (float)(pa * (1. - (pb / pa) * (pb / pa)));
      q[PF_KEY] = (float)(pb * (1. - (pa / pb) * (pa / pb)));
    } else if (q && sub == 5) {
      const double den = P[EIF_P_DEN * pc + n];
      q[PF_RPM] = (float)(1. / pmass(den, pa, pb));
      q[PF_RPIM] = (float)(1. / pmoi(den, pa, pb));
      q[PF_UX] = (float)P[EIF_P_UX * pc + n];
      q[PF_UY] = (float)P[EIF_P_UY * pc + n];
      q[PF_VZ] = (float)P[EIF_P_VZ * pc + n];
    } else if (q && sub == 6) {
      // cell centres XC(i) = (i - 1/2) dx, YC(j) = (j - 1/2) dy: offsets in grid units are
      // (i - i0) - gx and (j - j0[m]) - gy[m] for the periodic images m = -1, 0, +1
      const double sx = px / a.dx;
      const int i0 = (int)floor(sx);
      q[PF_GX] = (float)(sx - i0 + 0.5);
      q[PF_I0] = __int_as_float(i0);
      for (int m = 0; m < 3; m++) {
        const double sy = (py + a.ly * (m - 1)) / a.dy;
        const int j0 = (int)floor(sy);
        q[PF_J0 + m] = __int_as_float(j0);
        q[PF_GY + m] = (float)(sy - j0 + 0.5);
      }
    } else if (q && sub == 7) {
      // far-cell scales (row_chords)
      const double mn = fmin(pa, pb), mx = fmax(pa, pb);
      const double md = FAR_CELLS_F * fmin(a.dx, a.dy);
      const double so = 1. + md / mn, si = 1. - md / mn;
      q[PF_SO2] = (float)(so * so);
      q[PF_SI2] = si > 0. ? (float)(si * si) : -1.f;
      q[PF_RO2] = (float)((mx + md) * (mx + md));
    }
  }
  if (on && tasks && EIF_CHK(a.bd.rec, (a.nchunk - a.bd_off_base) + n, a.bd.off, 3)) atomicAdd(a.nchunk + n, tasks);
}

// exclusive scan of the chunk counts (one block); off[np] = total
__global__ void k_scan(const int *__restrict__ cnt, int *__restrict__ off, int np, Bounds bd,
                       const unsigned *__restrict__ iter) {
  if (iter && *iter == 0u) return;
  __shared__ int s[1024];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < np; base += 1024) {
    const int t = base + threadIdx.x;
    const int v = (t < np && EIF_CHK(bd.rec, (cnt - off) + t, bd.off, 4)) ? cnt[t] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int add = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += add;
      __syncthreads();
    }
    if (t < np && EIF_CHK(bd.rec, t, bd.off, 5)) off[t] = carry + s[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += s[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0 && EIF_CHK(bd.rec, np, bd.off, 6)) off[np] = carry;
}

// A particle's tasks: image by image, row by row, segment by segment.
struct RowTask {
  int img, j, ib, ie;   // image -1..1, row, first and last column of the segment
};
// one image's box (columns bi0..bi1, rows bj0..bj1): true when task r lies in it,
// otherwise r is reduced by the image's task count
__device__ __forceinline__ bool row_task_in(int4 b, int img, int &r, RowTask &t) {
  const int w = b.y - b.x + 1, h = b.w - b.z + 1;
  if (w <= 0 || h <= 0) return false;
  const int segs = box_segs(w);
  const int cnt = h * segs;
  if (r >= cnt) {
    r -= cnt;
    return false;
  }
  const int row = segs == 1 ? r : r / segs;
  const int seg = r - row * segs;
  t.img = img;
  t.j = b.z + row;
  t.ib = b.x + seg * CHUNK;
  t.ie = min(t.ib + CHUNK - 1, b.y);
  return true;
}
// task r of a particle whose image boxes are bm, b0, bp (images -1, 0, +1)
__device__ __forceinline__ bool row_task(int4 bm, int4 b0, int4 bp, int r, RowTask &t) {
  return row_task_in(bm, -1, r, t) || row_task_in(b0, 0, r, t) || row_task_in(bp, 1, r, t);
}

// The task table: one int4 per task (chunk) {particle, row, first column, last
// column * 4 + image + 1}, so that a kernel finds its task's geometry with one
// load instead of a chain of dependent loads (owner, boxes, offsets). One warp
// per particle.
__global__ void k_task_table(const int *__restrict__ box, const int *__restrict__ off, int4 *__restrict__ tdesc,
                             int np, Bounds bd, int cap, const unsigned *__restrict__ iter) {
  if (iter && *iter == 0u) return;
  const int n = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (n >= np) return;
  const int4 *b4 = reinterpret_cast<const int4 *>(box + 12 * n);
  const int4 bA = b4[0], bB = b4[1], bC = b4[2];
  const int c0 = off[n], c1 = off[n + 1];
  for (int c = c0 + lane; c < c1; c += 32) {
    RowTask t;
    int4 d = make_int4(-1, 0, 0, 0);
    if (row_task(bA, bB, bC, c - c0, t)) d = make_int4(n, t.j, t.ib, t.ie * 4 + t.img + 1);
    if (EIF_CHK(bd.rec, c, cap, 59)) tdesc[c] = d;
  }
}
// The same table with the task offsets formed in the same kernel, for particle
// counts up to TT_MAX_NP: every block sums the task counts of the particles before
// its own (a few thousand integers from L2), then each warp writes its particle's
// offset and table entries. Replaces k_scan + k_task_table (one launch and one
// single-block pass fewer on the path of every box build).
constexpr int TT_WARPS = 8;
constexpr int TT_MAX_NP = 8192;
__global__ void __launch_bounds__(TT_WARPS * 32) k_task_table_scan(const int *__restrict__ box, const int *__restrict__ cnt,
                                                                  int *__restrict__ off, int4 *__restrict__ tdesc, int np,
                                                                  Bounds bd, int cap, const unsigned *__restrict__ iter) {
  if (iter && *iter == 0u) return;
  __shared__ int red[TT_WARPS], wcnt[TT_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n0 = blockIdx.x * TT_WARPS;
  int s = 0;
  for (int q = threadIdx.x; q < n0; q += blockDim.x) s += cnt[q];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const int n = n0 + w;
  const int my = n < np ? cnt[n] : 0;
  if (lane == 0) {
    red[w] = s;
    wcnt[w] = my;
  }
  __syncthreads();
  int c0 = 0;
#pragma unroll
  for (int q = 0; q < TT_WARPS; q++) c0 += red[q] + (q < w ? wcnt[q] : 0);
  if (n >= np) return;
  if (lane == 0) {
    if (EIF_CHK(bd.rec, n, bd.off, 5)) off[n] = c0;
    if (n == np - 1 && EIF_CHK(bd.rec, np, bd.off, 6)) off[np] = c0 + my;
  }
  const int4 *b4 = reinterpret_cast<const int4 *>(box + 12 * n);
  const int4 bA = b4[0], bB = b4[1], bC = b4[2];
  for (int c = c0 + lane; c < c0 + my; c += 32) {
    RowTask t;
    int4 d = make_int4(-1, 0, 0, 0);
    if (row_task(bA, bB, bC, c - c0, t)) d = make_int4(n, t.j, t.ib, t.ie * 4 + t.img + 1);
    if (EIF_CHK(bd.rec, c, cap, 59)) tdesc[c] = d;
  }
}
__device__ __forceinline__ bool task_of(int4 d, int np, RowTask &t) {
  t.j = d.y;
  t.ib = d.z;
  t.ie = d.w >> 2;
  t.img = (d.w & 3) - 1;
  return d.x >= 0 && d.x < np;
}

// The far-cell bounds above along one row, as ranges of the lab-frame offset
// X from the centre at the row's offset Y: cells outside (olo, ohi) are far
// outside (rho >= so or r >= ro), cells in [ilo, ihi] are far inside (rho <= si;
// the disc r <= mn - md lies inside that ellipse). rho^2 = al X^2 + 2 ka X Y + de Y^2.
template <typename T>
__device__ __forceinline__ void row_chords(T al, T ka, T de, T so2, T si2, T ro2, T Y, T &olo, T &ohi, T &ilo,
                                           T &ihi) {
  const T big = T(1e30);
  olo = big; ohi = -big; ilo = big; ihi = -big;
  const T bY = ka * Y;
  const T Do = bY * bY - al * (de * Y * Y - so2);
  const T c2 = ro2 - Y * Y;
  if (Do > T(0) && c2 > T(0)) {
    const T sq = sqrt(Do), xc = sqrt(c2);
    olo = fmax((-bY - sq) / al, -xc);
    ohi = fmin((-bY + sq) / al, xc);
  }
  if (si2 > T(0)) {
    const T Di = bY * bY - al * (de * Y * Y - si2);
    if (Di >= T(0)) {
      const T sq = sqrt(Di);
      ilo = (-bY - sq) / al;
      ihi = (-bY + sq) / al;
    }
  }
}

struct WorkArgs {
  const double *P;
  const double *ux, *uy, *xc, *yc, *dt;
  const int *box, *off;
  double *partial;   // 3 per chunk
  double2 *wbuf;     // CHUNK per chunk (exchange only)
  int pcap, np, ld, mode, cn;   // mode 0: inertia (cn), 1: exchange
  double dx, dy, ly, h;
  const float *pf;       // per-particle single-precision parameters (mixed form)
  const int4 *tdesc;     // task table (k_task_table)
  const float *coef;     // single-precision dt products; [9] = 1/dt
  float rh_f, dx_f, dy_f, dxdy_f;
  // Indicator weights of the cells at the positions X are kept in wcache (one per
  // task slot, like wbuf) and reused by the evaluations that see the same
  // geometry: wmode 0 computes, 1 computes and stores, 2 loads; when iter is set
  // (the sub-iteration loop of a step graph) the kernel loads in the first
  // sub-iteration (*iter == 0, increments still zero) and computes afterwards.
  void *wcache;
  int wmode;
  const unsigned *iter;
  int gate;   // with iter (mixed form): 1 runs only in the first sub-iteration, 2 only afterwards
  int weights_only;   // exchange (double precision): the cell contributions are the weights (w, w)
  // box cells whose geometry is evaluated and, of those, the near cells that run the
  // normal-foot iteration, added to count[0] and count[1] (null: not counted)
  unsigned long long *count;
  Bounds bd;
};

// One warp per row task: indicator weights, partial sums, and (for the exchange)
// per-cell field contributions.
__global__ void __launch_bounds__(256) k_ibm_work(WorkArgs a) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int total = EIF_CHK(a.bd.rec, a.np, a.bd.off, 10) ? __ldg(a.off + a.np) : 0;
  const double rh = 1. / a.h;
  const double dxdy = a.dx * a.dy;
  const double dtv = a.mode == 1 ? __ldg(a.dt) : 0.;
  const double md = FAR_CELLS_D * a.h;
  const int pc = a.pcap, ld = a.ld;
  const int wmode = a.iter ? (*a.iter == 0u ? 2 : 0) : a.wmode;
  double *wcache = static_cast<double *>(a.wcache);
  // per warp: body-frame offsets of its near cells, overwritten by their weights
  __shared__ double2 slot_buf[8][CHUNK];
  double2 *slots = slot_buf[threadIdx.x >> 5];
  for (int c = warp; c < total; c += nwarps) {
    if (!EIF_CHK(a.bd.rec, c, a.bd.partial / 3, 21)) continue;
    const int4 dsc = __ldg(a.tdesc + c);
    const int n = dsc.x;
    if (!EIF_CHK(a.bd.rec, n, a.np, 11)) continue;
    if (!EIF_CHK(a.bd.rec, EIF_P_VZ * pc + n, a.bd.P, 13)) continue;
    RowTask t;
    const bool task = task_of(dsc, a.np, t) && EIF_CHK(a.bd.rec, t.j, a.bd.yc - 1, 15);
    const double *P = a.P;
    const double pden = __ldg(P + EIF_P_DEN * pc + n), pa = __ldg(P + EIF_P_A * pc + n), pb = __ldg(P + EIF_P_B * pc + n);
    double px = __ldg(P + EIF_P_X * pc + n), py = __ldg(P + EIF_P_Y * pc + n), paz = __ldg(P + EIF_P_AZ * pc + n);
    if (a.mode == 0) {
      // inertia.c:29-31: positions at k + increment
      px = px + __ldg(P + EIF_P_DX * pc + n);
      py = py + __ldg(P + EIF_P_DY * pc + n);
      paz = paz + __ldg(P + EIF_P_DAZ * pc + n);
    }
    const double pm = pmass(pden, pa, pb);
    const double pim = pmoi(pden, pa, pb);
    const double pux = __ldg(P + EIF_P_UX * pc + n), puy = __ldg(P + EIF_P_UY * pc + n), pvz = __ldg(P + EIF_P_VZ * pc + n);
    const Ell e = make_ell(pa, pb, px, py, paz);
    const double py_ = py + a.ly * (task ? t.img : 0);
    const int j = task ? t.j : 1;
    const double y = __ldg(a.yc + j);
    const double Y = y - py_;
    int rank[2];
    bool cin[2];
    double th2[2];
    unsigned near_mask[2];
    if (wmode == 2) {
      // weights of the same geometry from an earlier evaluation
#pragma unroll
      for (int half = 0; half < CHUNK / 32; half++) {
        const int i = (task ? t.ib : 1) + half * 32 + lane;
        bool in = task && i <= t.ie;
        if (in) {
          in = EIF_CHK(a.bd.rec, i, a.bd.xc - 1, 14) && EIF_CHK(a.bd.rec, j * ld + i, a.bd.field, 16) &&
               EIF_CHK(a.bd.rec, (j + 1) * ld + i, a.bd.field, 17) &&
               EIF_CHK(a.bd.rec, j * ld + (i - 1), a.bd.field, 18) &&
               EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, a.bd.wbuf, 22);
        }
        cin[half] = in;
        th2[half] = in ? wcache[(size_t)c * CHUNK + half * 32 + lane] : 0.;
      }
    } else {
    // far cells of this row (row_chords), in single precision: the far distance
    // (10.5 cells) exceeds the saturation distance of tanh (9.53 cells) by far more
    // than the rounding of the column bounds
    float olo, ohi, ilo, ihi;
    {
      const float fa = eifd::d2f(pa), fb = eifd::d2f(pb), cz = eifd::d2f(e.cz), sz = eifd::d2f(e.sz);
      const float mn = fminf(fa, fb), mx = fmaxf(fa, fb), fmd = eifd::d2f(md);
      const float so = 1.f + fmd / mn, si = 1.f - fmd / mn;
      const float al = cz * cz / (fa * fa) + sz * sz / (fb * fb);
      const float ka = cz * sz * (1.f / (fb * fb) - 1.f / (fa * fa));
      const float de = sz * sz / (fa * fa) + cz * cz / (fb * fb);
      row_chords(al, ka, de, so * so, si > 0.f ? si * si : -1.f, (mx + fmd) * (mx + fmd), eifd::d2f(Y), olo, ohi,
                 ilo, ihi);
    }
    // pass 1: cells of the row, far cells settled, body-frame offsets of the near ones
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      bool in = task && i <= t.ie;
      if (in) {
        in = EIF_CHK(a.bd.rec, i, a.bd.xc - 1, 14) && EIF_CHK(a.bd.rec, j * ld + i, a.bd.field, 16) &&
             EIF_CHK(a.bd.rec, (j + 1) * ld + i, a.bd.field, 17) && EIF_CHK(a.bd.rec, j * ld + (i - 1), a.bd.field, 18);
      }
      cin[half] = in;
      bool near = false;
      double x_ = 0., y_ = 0.;
      th2[half] = 0.;
      if (in) {
        const double X = __ldg(a.xc + i) - e.px;
        const float Xf = eifd::d2f(X);
        // reference sign convention: +1 inside (auxiliary.c:36-38); tanh saturated
        const int side = !(Xf > olo && Xf < ohi) ? -1 : ((Xf >= ilo && Xf <= ihi) ? 1 : 0);
        th2[half] = (double)side;
        near = side == 0;
        x_ = e.cz * X - e.sz * Y;
        y_ = e.sz * X + e.cz * Y;
      }
      near_mask[half] = __ballot_sync(0xffffffffu, near);
      rank[half] = (half ? __popc(near_mask[0]) : 0) + __popc(near_mask[half] & ((1u << lane) - 1u));
      if (near) slots[rank[half]] = make_double2(x_, y_);
    }
    // pass 2: the near cells, packed onto consecutive lanes
    const int nnear = __popc(near_mask[0]) + __popc(near_mask[1]);
    if (a.count) {
      const unsigned in0 = __ballot_sync(0xffffffffu, cin[0]), in1 = __ballot_sync(0xffffffffu, cin[1]);
      if (lane == 0) {
        atomicAdd(a.count, (unsigned long long)(__popc(in0) + __popc(in1)));
        atomicAdd(a.count + 1, (unsigned long long)nnear);
      }
    }
    __syncwarp();
    for (int k = lane; k < nnear; k += 32) {
      const double2 o = slots[k];
      slots[k].x = tanh(BETA * signed_dist_body(e, o.x, o.y, rh));
    }
    __syncwarp();
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++)
      if ((near_mask[half] >> lane) & 1u) th2[half] = slots[rank[half]].x;
    __syncwarp();
    if (wmode == 1) {
#pragma unroll
      for (int half = 0; half < CHUNK / 32; half++)
        if (EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, a.bd.wbuf, 23))
          wcache[(size_t)c * CHUNK + half * 32 + lane] = th2[half];
    }
    }
    double s0 = 0., s1 = 0., s2 = 0.;
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      double2 contrib = make_double2(0., 0.);
      // cells of weight exactly zero (inertia: far outside; exchange: any far cell) are skipped
      const double th_ = th2[half];
      const bool live = a.mode == 0 ? th_ != -1. : fabs(th_) != 1.;
      if (cin[half] && live) {
        const double x = __ldg(a.xc + i);
        const double th = th_;
        const double uxf = 0.5 * (__ldg(a.ux + j * ld + (i - 1)) + __ldg(a.ux + j * ld + i));
        const double uyf = 0.5 * (__ldg(a.uy + j * ld + i) + __ldg(a.uy + (j + 1) * ld + i));
        if (a.mode == 0) {
          // inertia.c:51-59
          const double w = 0.5 * (1. + th);
          const double valx = w * 0.5 * (2. * uxf) * dxdy;
          const double valy = w * 0.5 * (2. * uyf) * dxdy;
          s0 += valx / pm;
          s1 += valy / pm;
          s2 += (-(y - py_) * valx / pim) + ((x - px) * valy / pim);
        } else {
          // exchange.c:61-76
          const double w = 0.5 * BETA * (1. - th * th);
          const double uxp = pux - pvz * (y - py_);
          const double uyp = puy + pvz * (x - px);
          const double fx = w * (uxp - uxf) / dtv;
          const double fy = w * (uyp - uyf) / dtv;
          contrib = a.weights_only ? make_double2(w, w) : make_double2(fx * dtv, fy * dtv);
          const double Fx = fx * a.dx * a.dy, Fy = fy * a.dx * a.dy;
          s0 += -(Fx / pm);
          s1 += -(Fy / pm);
          s2 += ((y - py_) * Fx / pim) - ((x - px) * Fy / pim);
        }
      }
      if (a.mode == 1 && EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, a.bd.wbuf, 19))
        a.wbuf[(size_t)c * CHUNK + half * 32 + lane] = contrib;
    }
    s0 = eifd::warp_sum(s0);
    s1 = eifd::warp_sum(s1);
    s2 = eifd::warp_sum(s2);
    if (lane == 0 && EIF_CHK(a.bd.rec, 3LL * c + 2, a.bd.partial, 20)) {
      a.partial[3 * (size_t)c + 0] = s0;
      a.partial[3 * (size_t)c + 1] = s1;
      a.partial[3 * (size_t)c + 2] = s2;
    }
  }
}

// ---------------------------------------------------------------------------
// Single-precision indicator (EIF_PREC_MIXED). Cell offsets from the particle
// centre are formed in grid units, (x - px)/dx = (i - i0) - g with the integer
// i0 and the fraction g computed once per chunk in double precision, so the
// per-cell arithmetic is single precision without cancellation. The normal
// foot iteration is the reference's (ellipse.c:30-65) with a stopping threshold
// suited to single precision.
// The distance at the foot is stationary in t, so an angle error dt changes it by
// O(a dt^2): stopping once the step is below 1e-3 leaves distance errors near 1e-9
// cells (checked against fully converged iterations over the aspect ratios 1-3).
constexpr float NORMAL_TOL_F = 1.e-3f;
constexpr int NORMAL_MAX_F = 24;

struct EllF {
  float a, b, cz, sz, kex, key;
};

// The reference's iteration (ellipse.c:30-65) in single precision. Its fixed point
// is the normal foot whatever the accuracy of the intermediate sin/cos, square
// roots and arcsine, so the loop uses the hardware approximations (__sincosf,
// rsqrtf) and the Taylor polynomial x + x^3/6 + 3x^5/40 of asin (odd, increasing
// and zero only at zero like asin, so the step keeps its sign and vanishes at the
// foot); the distance at the converged angle is evaluated with the accurate
// sincosf, and the distance is stationary in the angle.
__device__ __forceinline__ float normal_t_f(const EllF &e, float x_, float y_) {
  const float px = fabsf(x_), py = fabsf(y_);
  float t = 0.78539816339744831f;
  for (int n = 0; n < NORMAL_MAX_F; n++) {
    float st, ct;
    __sincosf(t, &st, &ct);
    const float x = e.a * ct, y = e.b * st;
    const float ex = e.kex * (ct * ct * ct), ey = e.key * (st * st * st);
    const float rx = x - ex, ry = y - ey, qx = px - ex, qy = py - ey;
    const float r2 = ry * ry + rx * rx, q2 = qy * qy + qx * qx;
    const float arg = fminf(fmaxf((rx * qy - ry * qx) * rsqrtf(r2 * q2), -1.f), 1.f);
    const float a2 = arg * arg;
    const float dc = r2 * rsqrtf(r2) * (arg * fmaf(a2, fmaf(a2, 0.075f, 0.16666667f), 1.f));
    // a^2 + b^2 - x^2 - y^2 written without cancellation
    const float dt = dc * rsqrtf(e.a * e.a * (st * st) + e.b * e.b * (ct * ct));
    t += dt;
    t = fminf(1.5707963267948966f, t);
    t = fmaxf(0.f, t);
    if (fabsf(dt) < NORMAL_TOL_F) break;
  }
  if (x_ < 0.f) t = 3.14159265358979323846f - t;
  if (y_ < 0.f) t = -t;
  return t;
}

// tanh(2 d / h) of the signed distance (positive inside), d from the body-frame
// offset; tanh through one exponential, accurate to a few units of 1e-7 absolute
__device__ __forceinline__ float indicator_f(const EllF &e, float x_, float y_, float rh) {
  const float f0 = 1.f - (x_ / e.a) * (x_ / e.a) - (y_ / e.b) * (y_ / e.b);
  const float t = normal_t_f(e, x_, y_);
  float st, ct;
  sincosf(t, &st, &ct);
  const float dxx = e.a * ct - x_, dyy = e.b * st - y_;
  // |2d/h|; tanh is 1 in single precision beyond 10, the clamp keeps exp finite
  const float z = fminf(2.f * sqrtf(dxx * dxx + dyy * dyy) * rh, 20.f);
  const float ez = __expf(2.f * z);
  const float th = __fdividef(ez - 1.f, ez + 1.f);
  return f0 > 0.f ? th : -th;
}

// one warp per row task, single precision (see k_ibm_work)
__global__ void __launch_bounds__(256, 3) k_ibm_work_f(WorkArgs a) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int total = EIF_CHK(a.bd.rec, a.np, a.bd.off, 50) ? __ldg(a.off + a.np) : 0;
  const float rh = a.rh_f, dxf = a.dx_f, dyf = a.dy_f, dxdy = a.dxdy_f;
  const float rdtv = a.mode == 1 ? __ldg(a.coef + 9) : 0.f;
  const int ld = a.ld;
  float2 *wb = reinterpret_cast<float2 *>(a.wbuf);
  if (a.gate && ((a.gate == 1) != (*a.iter == 0u))) return;
  const int wmode = a.wmode;
  float *wcache = static_cast<float *>(a.wcache);
  // per warp: body-frame offsets of its near cells, overwritten by their weights
  __shared__ float2 slot_buf[8][CHUNK];
  float2 *slots = slot_buf[threadIdx.x >> 5];
  // the next task's table entry is loaded while the current task is processed
  int4 nxt = make_int4(-1, 0, 0, 0);
  if (warp < total && EIF_CHK(a.bd.rec, warp, a.bd.partial / 3, 51)) nxt = __ldg(a.tdesc + warp);
  for (int c = warp; c < total; c += nwarps) {
    const int4 dsc = nxt;
    if (c + nwarps < total && EIF_CHK(a.bd.rec, c + nwarps, a.bd.partial / 3, 51)) nxt = __ldg(a.tdesc + c + nwarps);
    const int n = dsc.x;
    if (!EIF_CHK(a.bd.rec, n, a.np, 52)) continue;
    RowTask t;
    const bool task = task_of(dsc, a.np, t);
    const float4 *q4 = reinterpret_cast<const float4 *>(a.pf + (size_t)PF_WORDS * n);
    const float4 qA = __ldg(q4), qB = __ldg(q4 + 1), qC = __ldg(q4 + 2), qD = __ldg(q4 + 3), qE = __ldg(q4 + 4);
    const float4 qF = __ldg(q4 + 5), qG = __ldg(q4 + 6);
    EllF e;
    e.a = qA.x; e.b = qA.y; e.cz = qA.z; e.sz = qA.w; e.kex = qB.x; e.key = qB.y;
    const float rpm = qB.z, rpim = qB.w, pux = qC.x, puy = qC.y, pvz = qC.z, gx = qC.w;
    const int i0 = __float_as_int(qD.x);
    const int m = task ? t.img + 1 : 1;
    // image row origin and fraction selected without a local array
    const int j0i = __float_as_int(m == 0 ? qD.y : (m == 1 ? qD.z : qD.w));
    const float gyi = m == 0 ? qE.x : (m == 1 ? qE.y : qE.z);
    const int j = task ? t.j : 1;
    const float Y = ((float)(j - j0i) - gyi) * dyf;
    int rank[2];
    float cX[2], th2[2];
    bool cin[2];
    unsigned near_mask[2];
    if (wmode == 2) {
      // weights of the same geometry from an earlier evaluation
#pragma unroll
      for (int half = 0; half < CHUNK / 32; half++) {
        const int i = (task ? t.ib : 1) + half * 32 + lane;
        bool in = task && i <= t.ie;
        if (in) {
          in = EIF_CHK(a.bd.rec, j * ld + i, a.bd.field, 54) && EIF_CHK(a.bd.rec, (j + 1) * ld + i, a.bd.field, 55) &&
               EIF_CHK(a.bd.rec, j * ld + (i - 1), a.bd.field, 56) &&
               EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, 2 * a.bd.wbuf, 59);
        }
        cin[half] = in;
        cX[half] = ((float)(i - i0) - gx) * dxf;
        th2[half] = in ? wcache[(size_t)c * CHUNK + half * 32 + lane] : 0.f;
      }
    } else {
    // far cells of this row (PF_AL .. PF_RO2: al, ka, de, so^2, si^2, ro^2)
    float olo, ohi, ilo, ihi;
    row_chords(qE.w, qF.x, qF.y, qF.z, qF.w, qG.x, Y, olo, ohi, ilo, ihi);
    // pass 1: cells of the row, far cells settled, body-frame offsets of the near ones
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      bool in = task && i <= t.ie;
      if (in) {
        in = EIF_CHK(a.bd.rec, j * ld + i, a.bd.field, 54) && EIF_CHK(a.bd.rec, (j + 1) * ld + i, a.bd.field, 55) &&
             EIF_CHK(a.bd.rec, j * ld + (i - 1), a.bd.field, 56);
      }
      cin[half] = in;
      bool near = false;
      float x_ = 0.f, y_ = 0.f;
      const float X = ((float)(i - i0) - gx) * dxf;
      cX[half] = X;
      th2[half] = 0.f;
      if (in) {
        const int side = !(X > olo && X < ohi) ? -1 : ((X >= ilo && X <= ihi) ? 1 : 0);
        th2[half] = (float)side;
        near = side == 0;
        x_ = e.cz * X - e.sz * Y;
        y_ = e.sz * X + e.cz * Y;
      }
      near_mask[half] = __ballot_sync(0xffffffffu, near);
      rank[half] = (half ? __popc(near_mask[0]) : 0) + __popc(near_mask[half] & ((1u << lane) - 1u));
      if (near) slots[rank[half]] = make_float2(x_, y_);
    }
    // pass 2: the near cells, packed onto consecutive lanes
    const int nnear = __popc(near_mask[0]) + __popc(near_mask[1]);
    if (a.count) {
      const unsigned in0 = __ballot_sync(0xffffffffu, cin[0]), in1 = __ballot_sync(0xffffffffu, cin[1]);
      if (lane == 0) {
        atomicAdd(a.count, (unsigned long long)(__popc(in0) + __popc(in1)));
        atomicAdd(a.count + 1, (unsigned long long)nnear);
      }
    }
    __syncwarp();
    for (int k = lane; k < nnear; k += 32) {
      const float2 o = slots[k];
      slots[k].x = indicator_f(e, o.x, o.y, rh);
    }
    __syncwarp();
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++)
      if ((near_mask[half] >> lane) & 1u) th2[half] = slots[rank[half]].x;
    __syncwarp();
    if (wmode == 1) {
#pragma unroll
      for (int half = 0; half < CHUNK / 32; half++)
        if (EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, 2 * a.bd.wbuf, 60))
          wcache[(size_t)c * CHUNK + half * 32 + lane] = th2[half];
    }
    }
    float sacc0 = 0.f, sacc1 = 0.f, sacc2 = 0.f;
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      float2 contrib = make_float2(0.f, 0.f);
      // cells of weight exactly zero (inertia: far outside; exchange: any far cell) are skipped
      const float th_ = th2[half];
      const bool live = a.mode == 0 ? th_ != -1.f : fabsf(th_) != 1.f;
      if (cin[half] && live) {
        const float X = cX[half], th = th_;
        const float uxs = eifd::d2f(__ldg(a.ux + j * ld + (i - 1))) + eifd::d2f(__ldg(a.ux + j * ld + i));
        const float uys = eifd::d2f(__ldg(a.uy + j * ld + i)) + eifd::d2f(__ldg(a.uy + (j + 1) * ld + i));
        if (a.mode == 0) {
          const float w = 0.5f * (1.f + th);
          const float valx = w * 0.5f * uxs * dxdy;
          const float valy = w * 0.5f * uys * dxdy;
          sacc0 += valx * rpm;
          sacc1 += valy * rpm;
          sacc2 += (-Y * valx + X * valy) * rpim;
        } else {
          const float w = 1.f - th * th;
          const float uxp = pux - pvz * Y;
          const float uyp = puy + pvz * X;
          const float gxv = w * (uxp - 0.5f * uxs);   // fx * dt
          const float gyv = w * (uyp - 0.5f * uys);   // fy * dt
          contrib = make_float2(gxv, gyv);
          const float Fx = gxv * rdtv * dxdy, Fy = gyv * rdtv * dxdy;
          sacc0 -= Fx * rpm;
          sacc1 -= Fy * rpm;
          sacc2 += (Y * Fx - X * Fy) * rpim;
        }
      }
      if (a.mode == 1 && EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, 2 * a.bd.wbuf, 57))
        wb[(size_t)c * CHUNK + half * 32 + lane] = contrib;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sacc0 += __shfl_xor_sync(0xffffffffu, sacc0, o);
      sacc1 += __shfl_xor_sync(0xffffffffu, sacc1, o);
      sacc2 += __shfl_xor_sync(0xffffffffu, sacc2, o);
    }
    if (lane == 0 && EIF_CHK(a.bd.rec, 3LL * c + 2, a.bd.partial, 58)) {
      // single-precision partial sums, reduced per particle by k_chunk_reduce_f
      float *pf3 = reinterpret_cast<float *>(a.partial);
      pf3[3 * (size_t)c + 0] = sacc0;
      pf3[3 * (size_t)c + 1] = sacc1;
      pf3[3 * (size_t)c + 2] = sacc2;
    }
  }
}

// The mixed form's evaluation with cached weights (wmode 2 of k_ibm_work_f): the
// same sums and field contributions, without the geometry work, so it runs with
// few registers and many resident warps, which hide the latency of its loads.
__global__ void __launch_bounds__(256, 6) k_ibm_sum_f(WorkArgs a) {
  if (a.gate && ((a.gate == 1) != (*a.iter == 0u))) return;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int total = EIF_CHK(a.bd.rec, a.np, a.bd.off, 70) ? __ldg(a.off + a.np) : 0;
  const float dxf = a.dx_f, dyf = a.dy_f, dxdy = a.dxdy_f;
  const float rdtv = a.mode == 1 ? __ldg(a.coef + 9) : 0.f;
  const int ld = a.ld;
  float2 *wb = reinterpret_cast<float2 *>(a.wbuf);
  const float *wcache = static_cast<const float *>(a.wcache);
  // the next task's table entry and cached weights are loaded while the current task
  // is processed, so that its field loads need not wait for them
  int4 nxt = make_int4(-1, 0, 0, 0);
  float nth0 = 0.f, nth1 = 0.f;
  if (warp < total && EIF_CHK(a.bd.rec, warp, a.bd.partial / 3, 71) &&
      EIF_CHK(a.bd.rec, (long long)warp * CHUNK + CHUNK - 1, 2 * a.bd.wbuf, 77)) {
    nxt = __ldg(a.tdesc + warp);
    nth0 = wcache[(size_t)warp * CHUNK + lane];
    nth1 = wcache[(size_t)warp * CHUNK + 32 + lane];
  }
  for (int c = warp; c < total; c += nwarps) {
    const int4 dsc = nxt;
    const float th_pre[2] = {nth0, nth1};
    const int cn = c + nwarps;
    if (cn < total && EIF_CHK(a.bd.rec, cn, a.bd.partial / 3, 71) &&
        EIF_CHK(a.bd.rec, (long long)cn * CHUNK + CHUNK - 1, 2 * a.bd.wbuf, 77)) {
      nxt = __ldg(a.tdesc + cn);
      nth0 = wcache[(size_t)cn * CHUNK + lane];
      nth1 = wcache[(size_t)cn * CHUNK + 32 + lane];
    }
    const int n = dsc.x;
    if (!EIF_CHK(a.bd.rec, n, a.np, 72)) continue;
    RowTask t;
    const bool task = task_of(dsc, a.np, t);
    const float4 *q4 = reinterpret_cast<const float4 *>(a.pf + (size_t)PF_WORDS * n);
    const float4 qB = __ldg(q4 + 1), qC = __ldg(q4 + 2), qD = __ldg(q4 + 3), qE = __ldg(q4 + 4);
    const float rpm = qB.z, rpim = qB.w, pux = qC.x, puy = qC.y, pvz = qC.z, gx = qC.w;
    const int i0 = __float_as_int(qD.x);
    const int m = task ? t.img + 1 : 1;
    const int j0i = __float_as_int(m == 0 ? qD.y : (m == 1 ? qD.z : qD.w));
    const float gyi = m == 0 ? qE.x : (m == 1 ? qE.y : qE.z);
    const int j = task ? t.j : 1;
    const float Y = ((float)(j - j0i) - gyi) * dyf;
    float sacc0 = 0.f, sacc1 = 0.f, sacc2 = 0.f;
#pragma unroll 1
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      const long long slot = (long long)c * CHUNK + half * 32 + lane;
      bool in = task && i <= t.ie;
      if (in) {
        in = EIF_CHK(a.bd.rec, j * ld + i, a.bd.field, 74) && EIF_CHK(a.bd.rec, (j + 1) * ld + i, a.bd.field, 75) &&
             EIF_CHK(a.bd.rec, j * ld + (i - 1), a.bd.field, 76);
      }
      float2 contrib = make_float2(0.f, 0.f);
      const float th = in ? th_pre[half] : 0.f;
      // cells of weight exactly zero (inertia: far outside; exchange: any far cell) are skipped
      const bool live = in && (a.mode == 0 ? th != -1.f : fabsf(th) != 1.f);
      if (live) {
        const float X = ((float)(i - i0) - gx) * dxf;
        const float uxs = eifd::d2f(__ldg(a.ux + j * ld + (i - 1))) + eifd::d2f(__ldg(a.ux + j * ld + i));
        const float uys = eifd::d2f(__ldg(a.uy + j * ld + i)) + eifd::d2f(__ldg(a.uy + (j + 1) * ld + i));
        if (a.mode == 0) {
          const float w = 0.5f * (1.f + th);
          const float valx = w * 0.5f * uxs * dxdy;
          const float valy = w * 0.5f * uys * dxdy;
          sacc0 += valx * rpm;
          sacc1 += valy * rpm;
          sacc2 += (-Y * valx + X * valy) * rpim;
        } else {
          const float w = 1.f - th * th;
          const float uxp = pux - pvz * Y;
          const float uyp = puy + pvz * X;
          const float gxv = w * (uxp - 0.5f * uxs);   // fx * dt
          const float gyv = w * (uyp - 0.5f * uys);   // fy * dt
          contrib = make_float2(gxv, gyv);
          const float Fx = gxv * rdtv * dxdy, Fy = gyv * rdtv * dxdy;
          sacc0 -= Fx * rpm;
          sacc1 -= Fy * rpm;
          sacc2 += (Y * Fx - X * Fy) * rpim;
        }
      }
      if (a.mode == 1 && EIF_CHK(a.bd.rec, slot, 2 * a.bd.wbuf, 78)) wb[slot] = contrib;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sacc0 += __shfl_xor_sync(0xffffffffu, sacc0, o);
      sacc1 += __shfl_xor_sync(0xffffffffu, sacc1, o);
      sacc2 += __shfl_xor_sync(0xffffffffu, sacc2, o);
    }
    if (lane == 0 && EIF_CHK(a.bd.rec, 3LL * c + 2, a.bd.partial, 79)) {
      // single-precision partial sums, reduced per particle by k_chunk_reduce_f
      float *pf3 = reinterpret_cast<float *>(a.partial);
      pf3[3 * (size_t)c + 0] = sacc0;
      pf3[3 * (size_t)c + 1] = sacc1;
      pf3[3 * (size_t)c + 2] = sacc2;
    }
  }
}

// per-particle sums over chunks in a fixed order (warp per particle)
__global__ void k_chunk_reduce(const double *__restrict__ partial, const int *__restrict__ off, double *__restrict__ P,
                               int pcap, int np, int f0, int f1, int f2, Bounds bd) {
  const int lane = threadIdx.x & 31;
  const int n = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (n >= np) return;
  if (!EIF_CHK(bd.rec, n + 1, bd.off, 30)) return;
  const int c0 = off[n], c1 = off[n + 1];
  double s0 = 0., s1 = 0., s2 = 0.;
  for (int c = c0 + lane; c < c1; c += 32) {
    if (!EIF_CHK(bd.rec, 3LL * c + 2, bd.partial, 31)) break;
    s0 += partial[3 * (size_t)c + 0];
    s1 += partial[3 * (size_t)c + 1];
    s2 += partial[3 * (size_t)c + 2];
  }
  s0 = eifd::warp_sum(s0);
  s1 = eifd::warp_sum(s1);
  s2 = eifd::warp_sum(s2);
  if (lane == 0 && EIF_CHK(bd.rec, f2 * pcap + n, bd.P, 32)) {
    P[f0 * pcap + n] = s0;
    P[f1 * pcap + n] = s1;
    P[f2 * pcap + n] = s2;
  }
}

// The same per-particle sums from the single-precision partials of the mixed form,
// accumulated in double-float arithmetic (TwoSum) on the FP32 pipe: the sum of at most
// a few hundred floats is kept to about 48 bits, and the result is rounded once to
// double.
__global__ void k_chunk_reduce_f(const float *__restrict__ partial, const int *__restrict__ off, double *__restrict__ P,
                                 int pcap, int np, int f0, int f1, int f2, Bounds bd) {
  const int lane = threadIdx.x & 31;
  const int n = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (n >= np) return;
  if (!EIF_CHK(bd.rec, n + 1, bd.off, 33)) return;
  const int c0 = off[n], c1 = off[n + 1];
  float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
  for (int c = c0 + lane; c < c1; c += 32) {
    if (!EIF_CHK(bd.rec, 3LL * c + 2, 2 * bd.partial, 34)) break;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float v = partial[3 * (size_t)c + k];
      const float s = h[k] + v, bb = s - h[k];
      l[k] += (h[k] - (s - bb)) + (v - bb);
      h[k] = s;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float vh = __shfl_xor_sync(0xffffffffu, h[k], o), vl = __shfl_xor_sync(0xffffffffu, l[k], o);
      const float s = h[k] + vh, bb = s - h[k];
      l[k] += ((h[k] - (s - bb)) + (vh - bb)) + vl;
      h[k] = s;
    }
  }
  if (lane == 0 && EIF_CHK(bd.rec, f2 * pcap + n, bd.P, 35)) {
    P[f0 * pcap + n] = eifd::f2d(h[0]) + eifd::f2d(l[0]);
    P[f1 * pcap + n] = eifd::f2d(h[1]) + eifd::f2d(l[1]);
    P[f2 * pcap + n] = eifd::f2d(h[2]) + eifd::f2d(l[2]);
  }
}

// Ordered lists of the (particle, image) boxes that reach each band of GTY rows,
// built once per exchange; entry = 3 * particle + image index, in entry order.
// Step 1 (one thread per particle): every box sets its bit in the bitmap of each
// band it reaches (atomicOr: the result does not depend on the order). Step 2
// (one warp per band): the band's set bits are compacted in index order.
__global__ void k_band_marks(const int *__restrict__ box, const int *__restrict__ off, int np, int jtot,
                             unsigned *__restrict__ marks, int words, int4 *__restrict__ edesc, Bounds bd) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= np) return;
  const int nbands = (jtot + GTY - 1) / GTY;
  const int *bx = box + 12 * n;
  int tasks_q = 0;   // tasks of the earlier images
  const int off_n = off[n];
#pragma unroll
  for (int q = 0; q < 3; q++) {
    const int bi0 = bx[4 * q], bi1 = bx[4 * q + 1], bj0 = bx[4 * q + 2], bj1 = bx[4 * q + 3];
    const bool nonempty = bi1 >= bi0 && bj1 >= bj0;
    const int e = 3 * n + q;
    // the entry's box and where its rows start in the scratch buffer (a box row
    // occupies segs * CHUNK slots)
    if (EIF_CHK(bd.rec, 2LL * e + 1, 6LL * np, 47)) {
      edesc[2 * e] = nonempty ? make_int4(bi0, bi1, bj0, bj1) : make_int4(1, 0, 1, 0);
      edesc[2 * e + 1] = make_int4(nonempty ? box_segs(bi1 - bi0 + 1) * CHUNK : 0, (off_n + tasks_q) * CHUNK, 0, 0);
    }
    if (!nonempty) continue;
    tasks_q += (bj1 - bj0 + 1) * box_segs(bi1 - bi0 + 1);
    const int b0 = max(0, (bj0 - 1) / GTY), b1 = min(nbands - 1, (bj1 - 1) / GTY);
    for (int b = b0; b <= b1; b++) atomicOr(marks + (size_t)b * words + (e >> 5), 1u << (e & 31));
  }
}

__global__ void k_band_lists(const unsigned *__restrict__ marks, int words, int jtot, int *__restrict__ lists,
                             int *__restrict__ counts, int cap, unsigned *__restrict__ flags) {
  const int lane = threadIdx.x & 31;
  const int band = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nbands = (jtot + GTY - 1) / GTY;
  if (band >= nbands) return;
  int count = 0;
  int *out = lists + (size_t)band * cap;
  const unsigned *row = marks + (size_t)band * words;
  for (int base = 0; base < words; base += 32) {
    const int w = base + lane;
    unsigned bits = w < words ? row[w] : 0u;
    const int m = __popc(bits);
    int sc = m;
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, sc, o);
      if (lane >= o) sc += v;
    }
    int pos = count + sc - m;
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1u;
      if (pos < cap) out[pos] = 32 * w + b;
      pos++;
    }
    count += __shfl_sync(0xffffffffu, sc, 31);
  }
  if (lane == 0) {
    counts[band] = count;
    if (count > cap) atomicOr(flags, EIF_FLAG_NOCONV);
  }
}

struct GatherArgs {
  const int4 *edesc;   // per (particle, image) entry: box, then row pitch and scratch offset
  const int *lists, *counts;
  int cap;
  const void *wbuf;
  void *dux, *duy;   // double (FP64 form) or float (mixed form) fields with the same pitch
  unsigned *flags;
  int np, itot, jtot, ld;
  Bounds bd;
};

// field response dux/duy (exchange.c:71-72,80-81): per tile, the entries of the
// band's ordered list that reach the tile's columns are compacted in order into
// shared memory, then every cell sums their contributions in that order
template <typename V2, typename Acc>
__global__ void __launch_bounds__(GTHREADS, 6) k_gather(GatherArgs a) {
  const V2 *wbuf = static_cast<const V2 *>(a.wbuf);
  // compacted entries: columns, rows, row pitch and offset of the box in the scratch buffer
  __shared__ int e_i0[LMAX], e_i1[LMAX], e_j0[LMAX], e_j1[LMAX], e_w[LMAX], e_base[LMAX];
  __shared__ int wcount[GTHREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int i0 = 1 + blockIdx.x * GTX, j0 = 1 + blockIdx.y * GTY;
  const int i1 = min(i0 + GTX - 1, a.itot), j1 = min(j0 + GTY - 1, a.jtot);
  constexpr int NC = (GTX / GCOLS) * 2;
  Acc acc_x[NC], acc_y[NC];
#pragma unroll
  for (int r = 0; r < NC; r++) { acc_x[r] = 0; acc_y[r] = 0; }
  // cells of this thread: (i0 + lx + GCOLS h, j0 + ly0 + 4 r), cell index 2 h + r
  const int lx = threadIdx.x % GCOLS, ly0 = threadIdx.x / GCOLS;  // GTHREADS / GCOLS = 4 rows per pass
  const int band = blockIdx.y;
  const int L = min(__ldg(a.counts + band), a.cap);
  const int *blist = a.lists + (size_t)band * a.cap;
  for (int base = 0; base < L; base += GTHREADS) {
    const int e = base + threadIdx.x;
    int4 b = make_int4(1, 0, 1, 0), w = make_int4(0, 0, 0, 0);
    if (e < L) {
      const int ent = __ldg(blist + e);
      // entry = 3 * particle + image; anything else is recorded and skipped
      if (EIF_CHK(a.bd.rec, ent, 3LL * a.np, 46)) {
        b = __ldg(a.edesc + 2 * ent);
        w = __ldg(a.edesc + 2 * ent + 1);
      }
    }
    const bool keep = b.y >= b.x && b.x <= i1 && b.y >= i0 && b.z <= j1 && b.w >= j0;
    const unsigned mask = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wcount[wid] = __popc(mask);
    __syncthreads();
    int pos = __popc(mask & ((1u << lane) - 1u)), cnt = 0;
#pragma unroll
    for (int q = 0; q < GTHREADS / 32; q++) {
      const int wc = wcount[q];
      pos += q < wid ? wc : 0;
      cnt += wc;
    }
    if (keep) {
      e_i0[pos] = b.x; e_i1[pos] = b.y; e_j0[pos] = b.z; e_j1[pos] = b.w; e_w[pos] = w.x; e_base[pos] = w.y;
    }
    __syncthreads();
    for (int k = 0; k < cnt; k++) {
      const int bi0 = e_i0[k], bi1 = e_i1[k], bj0 = e_j0[k], bj1 = e_j1[k], pw = e_w[k];
      const size_t pbase = (size_t)e_base[k];
#pragma unroll
      for (int q = 0; q < NC; q++) {
        const int i = i0 + lx + GCOLS * (q >> 1), j = j0 + ly0 + 4 * (q & 1);
        if (i >= bi0 && i <= bi1 && j >= bj0 && j <= bj1 &&
            EIF_CHK(a.bd.rec, (long long)(pbase + (size_t)(j - bj0) * pw + (i - bi0)),
                    a.bd.wbuf * (long long)(sizeof(double2) / sizeof(V2)), 41)) {
          const V2 v = wbuf[pbase + (size_t)(j - bj0) * pw + (i - bi0)];
          acc_x[q] += v.x;
          acc_y[q] += v.y;
        }
      }
    }
    __syncthreads();
  }
  // write the tile's interior cells (zero where no box covers); the halo rows and
  // ghost columns are filled afterwards by k_ibm_halo from these cells
  const int ld = a.ld;
#pragma unroll
  for (int q = 0; q < NC; q++) {
    const int i = i0 + lx + GCOLS * (q >> 1), j = j0 + ly0 + 4 * (q & 1);
    if (i > i1 || j > j1) continue;
    const int cidx = j * ld + i;
    if (!EIF_CHK(a.bd.rec, cidx, a.bd.field, 42)) continue;
    static_cast<Acc *>(a.dux)[cidx] = acc_x[q];
    static_cast<Acc *>(a.duy)[cidx] = acc_y[q];
  }
}

// Periodic halo rows (j = 0 <- jtot, j = jtot+1 <- 1) and Neumann ghost columns
// (i = 0 <- 1, i = itot+1 <- itot, corners included) of the IBM field response,
// exchange.c:80-81 with the boundary update of the reference. Every thread reads
// one interior cell and writes one halo cell.
template <typename T>
__global__ void k_ibm_halo(T *__restrict__ dux, T *__restrict__ duy, int itot, int jtot, int ld) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nrow = itot + 2;
  int dst, src;
  if (t < 2 * nrow) {
    const int i = t % nrow, top = t / nrow;
    const int ic = i < 1 ? 1 : (i > itot ? itot : i);
    dst = (top ? jtot + 1 : 0) * ld + i;
    src = (top ? 1 : jtot) * ld + ic;
  } else if (t < 2 * nrow + 2 * jtot) {
    const int u = t - 2 * nrow;
    const int j = 1 + u % jtot, right = u / jtot;
    dst = j * ld + (right ? itot + 1 : 0);
    src = j * ld + (right ? itot : 1);
  } else {
    return;
  }
  dux[dst] = dux[src];
  duy[dst] = duy[src];
}

}  // namespace

namespace eif {

// Bound on the box cells of one particle over its three images. A box spans at
// most 2r/h + 2 + 2*NEXTRA + 1 cells per direction before clipping; the three
// images are shifted by exactly jtot rows, so their clipped row ranges together
// never exceed the unclipped height.
static size_t box_tasks_bound(const eif_ctx *c, double r) {
  const long w = (long)std::ceil(2. * r / c->dx) + 2 + 2 * NEXTRA + 2;
  const long h = (long)std::ceil(2. * r / c->dy) + 2 + 2 * NEXTRA + 2;
  const long wc = std::min<long>(w, c->itot);
  const long hc = std::min<long>(h, 3L * c->jtot);
  return (size_t)hc * (size_t)box_segs((int)wc);
}

// resident CTAs per SM of the IBM work kernels (a host query; done before any graph capture)
int ibm_prepare(eif_ctx *c) {
  int v = 0;
  EIF_CK(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_ibm_work, 256, 0));
  c->ibm_ctas_per_sm[0] = std::max(1, v);
  EIF_CK(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_ibm_work_f, 256, 0));
  c->ibm_ctas_per_sm[1] = std::max(1, v);
  EIF_CK(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_ibm_sum_f, 256, 0));
  c->ibm_ctas_per_sm[2] = std::max(1, v);
  return EIF_OK;
}

// task bound of a particle set, from the radii in the host records (EIF_NFIELDS per particle)
size_t ibm_tasks_needed(const eif_ctx *c, const double *rec, int n) {
  size_t chunks = 0;
  for (int k = 0; k < n; k++) {
    chunks += box_tasks_bound(c, std::max(rec[(size_t)k * EIF_NFIELDS + EIF_P_A], rec[(size_t)k * EIF_NFIELDS + EIF_P_B]));
  }
  return chunks;
}

int ibm_reserve(eif_ctx *c, size_t chunks) {
  // called after a particle push that changed the particle set: size the task and scratch buffers
  ibm_free(c);
  if (c->np == 0) return EIF_OK;
  c->chunk_cap = (int)chunks;
  c->wcap = chunks * CHUNK;
  EIF_CK(c, cudaMalloc((void **)&c->box, sizeof(int) * 12 * c->np));
  EIF_CK(c, cudaMalloc((void **)&c->chunk_off, sizeof(int) * 2 * (c->np + 1)));
  EIF_CK(c, cudaMalloc((void **)&c->partial, sizeof(double) * 3 * chunks));
  EIF_CK(c, cudaMalloc((void **)&c->wbuf, sizeof(double2) * c->wcap));
  EIF_CK(c, cudaMalloc((void **)&c->wcache, sizeof(double) * c->wcap));
  EIF_CK(c, cudaMalloc((void **)&c->pf, sizeof(float) * PF_WORDS * c->np));
  EIF_CK(c, cudaMalloc((void **)&c->tdesc, sizeof(int4) * (size_t)chunks));
  const int nbands = (c->jtot + GTY - 1) / GTY;
  c->band_cap = 3 * c->np;
  EIF_CK(c, cudaMalloc((void **)&c->band_lists, sizeof(int) * (size_t)nbands * c->band_cap));
  EIF_CK(c, cudaMalloc((void **)&c->band_counts, sizeof(int) * (size_t)nbands));
  EIF_CK(c, cudaMalloc((void **)&c->band_marks, sizeof(unsigned) * (size_t)nbands * ((3 * c->np + 31) / 32)));
  EIF_CK(c, cudaMalloc((void **)&c->edesc, sizeof(int4) * 6 * (size_t)c->np));
  return EIF_OK;
}

void ibm_free(eif_ctx *c) {
  if (c->box) cudaFree(c->box);
  if (c->chunk_off) cudaFree(c->chunk_off);
  if (c->partial) cudaFree(c->partial);
  if (c->wbuf) cudaFree(c->wbuf);
  if (c->wcache) cudaFree(c->wcache);
  if (c->pf) cudaFree(c->pf);
  if (c->tdesc) cudaFree(c->tdesc);
  if (c->band_lists) cudaFree(c->band_lists);
  if (c->band_counts) cudaFree(c->band_counts);
  if (c->band_marks) cudaFree(c->band_marks);
  if (c->edesc) cudaFree(c->edesc);
  c->band_lists = nullptr; c->band_counts = nullptr; c->band_marks = nullptr; c->edesc = nullptr;
  c->box = nullptr; c->chunk_off = nullptr; c->partial = nullptr; c->wbuf = nullptr; c->wcache = nullptr;
  c->weights_x_valid = false;
  c->pf = nullptr; c->tdesc = nullptr;
  c->chunk_cap = 0; c->wcap = 0;
}

static Bounds bounds_of(const eif_ctx *c) {
  Bounds b;
  b.P = (long long)EIF_NFIELDS * c->pcap;
  b.box = 12LL * c->np;
  b.off = 2LL * (c->np + 1);
  b.partial = 3LL * c->chunk_cap;
  b.wbuf = (long long)c->wcap;
  b.field = (long long)c->nfield;
  b.xc = c->itot + 3;   // entries 0..itot+1 (EIF_CHK is given xc-1 as the bound of valid i)
  b.yc = c->jtot + 3;
  b.rec = c->d_check;
  return b;
}

static int launch_boxes(eif_ctx *c, bool use_increment) {
  // boxes at the positions X (no increment, or increments known to be zero) are
  // reused until the positions or the particle set change
  const bool x_only = !use_increment || c->incr_zero;
  if (x_only && c->boxes_x_valid) return EIF_OK;
  c->boxes_x_valid = false;
  c->weights_x_valid = false;
  c->bands_x_valid = false;
  BoxArgs b;
  b.bd = bounds_of(c);
  b.bd_off_base = c->chunk_off;
  b.P = c->P; b.pcap = c->pcap; b.np = c->np; b.itot = c->itot; b.jtot = c->jtot;
  b.use_increment = use_increment ? 1 : 0;
  b.dx = c->dx; b.dy = c->dy; b.ly = c->ly; b.yf1 = c->h_yf[0];
  b.box = c->box;
  b.pf = c->cfg.precision == EIF_PREC_MIXED ? c->pf : nullptr;
  b.iter = c->in_loop ? reinterpret_cast<const unsigned *>(c->d_inc + 1) : nullptr;
  int *cnt = c->chunk_off + (c->np + 1);
  b.nchunk = cnt;
  EIF_PROF(c, "ibm_boxes", c->np <= TT_MAX_NP ? 2 : 3);
  EIF_CK(c, cudaMemsetAsync(cnt, 0, sizeof(int) * c->np, c->stream));
  k_boxes<<<dim3((c->np + 31) / 32, b.pf ? BOX_PARTS : 3), 32, 0, c->stream>>>(b);
  EIF_LAUNCH_CK(c);
  if (c->np <= TT_MAX_NP) {
    k_task_table_scan<<<(c->np + TT_WARPS - 1) / TT_WARPS, TT_WARPS * 32, 0, c->stream>>>(
        c->box, cnt, c->chunk_off, c->tdesc, c->np, bounds_of(c), c->chunk_cap, b.iter);
    EIF_LAUNCH_CK(c);
  } else {
    k_scan<<<1, 1024, 0, c->stream>>>(cnt, c->chunk_off, c->np, bounds_of(c), b.iter);
    EIF_LAUNCH_CK(c);
    k_task_table<<<(c->np * 32 + 255) / 256, 256, 0, c->stream>>>(c->box, c->chunk_off, c->tdesc, c->np,
                                                                   bounds_of(c), c->chunk_cap, b.iter);
    EIF_LAUNCH_CK(c);
  }
  c->boxes_x_valid = x_only;
  return EIF_OK;
}

static int launch_work(eif_ctx *c, int mode, int cn) {
  WorkArgs w;
  w.P = c->P; w.ux = c->ux[c->cur]; w.uy = c->uy[c->cur]; w.xc = c->xc; w.yc = c->yc; w.dt = c->d_scal;
  w.box = c->box; w.off = c->chunk_off; w.partial = c->partial; w.wbuf = reinterpret_cast<double2 *>(c->wbuf);
  w.pcap = c->pcap; w.np = c->np; w.ld = c->ld; w.mode = mode; w.cn = cn;
  w.dx = c->dx; w.dy = c->dy; w.ly = c->ly; w.h = std::min(c->dx, c->dy);
  w.bd = bounds_of(c);
  w.pf = c->pf;
  w.tdesc = c->tdesc;
  w.coef = c->d_coef;
  w.rh_f = (float)(1. / w.h);
  w.dx_f = (float)c->dx;
  w.dy_f = (float)c->dy;
  w.dxdy_f = (float)(c->dx * c->dy);
  // weights at the positions X (inertia with zero increments, or the exchange)
  // are stored once and reused while the boxes at X stay valid
  const bool x_only = mode == 1 || c->incr_zero;
  w.wcache = c->wcache;
  w.iter = nullptr;
  w.gate = 0;
  w.weights_only = c->ibm_weights_only ? 1 : 0;
  w.count = c->prof.enabled ? c->d_inc + 3 : nullptr;
  if (c->in_loop) {
    w.wmode = 0;
    w.iter = reinterpret_cast<const unsigned *>(c->d_inc + 1);
  } else if (x_only && c->boxes_x_valid && c->weights_x_valid) {
    w.wmode = 2;
  } else if (x_only && c->boxes_x_valid) {
    w.wmode = 1;
    c->weights_x_valid = true;
  } else {
    w.wmode = 0;
  }
  // persistent grid: as many CTAs as are resident at once (queried once per context)
  const int per_sm_idx = c->cfg.precision == EIF_PREC_MIXED ? 1 : 0;
  if (c->ibm_ctas_per_sm[per_sm_idx] == 0) {
    int rc = ibm_prepare(c);
    if (rc) return rc;
  }
  const int per_sm = c->ibm_ctas_per_sm[per_sm_idx];
  const int blocks = std::max(1, std::min(c->sms * per_sm, (c->chunk_cap * 32 + 255) / 256));
  {
    const bool mixed = c->cfg.precision == EIF_PREC_MIXED;
    // launches that evaluate the indicator geometry are timed as ibm_indicator, those
    // with stored weights (sums and field contributions only) as inertia or exchange
    const bool geometry = w.wmode != 2 && !(mixed && c->in_loop);
    EIF_PROF(c, geometry ? "ibm_indicator" : (mode == 0 ? "ibm_inertia" : "ibm_exchange"),
             mixed && c->in_loop ? 2 : 1);
    if (mixed && c->in_loop) {
      // first sub-iteration: cached weights; later ones: full evaluation (decided on the device)
      WorkArgs w1 = w, w2 = w;
      w1.wmode = 2; w1.gate = 1;
      w2.wmode = 0; w2.gate = 2;
      k_ibm_sum_f<<<c->sms * c->ibm_ctas_per_sm[2], 256, 0, c->stream>>>(w1);
      EIF_LAUNCH_CK(c);
      k_ibm_work_f<<<blocks, 256, 0, c->stream>>>(w2);
    } else if (mixed && w.wmode == 2) {
      k_ibm_sum_f<<<c->sms * c->ibm_ctas_per_sm[2], 256, 0, c->stream>>>(w);
    } else if (mixed) {
      k_ibm_work_f<<<blocks, 256, 0, c->stream>>>(w);
    } else {
      k_ibm_work<<<blocks, 256, 0, c->stream>>>(w);
    }
    EIF_LAUNCH_CK(c);
  }
  const int f0 = mode == 0 ? EIF_P_IUX0 + cn : EIF_P_FUX;
  const int f1 = mode == 0 ? EIF_P_IUY0 + cn : EIF_P_FUY;
  const int f2 = mode == 0 ? EIF_P_IVZ0 + cn : EIF_P_TVZ;
  EIF_PROF(c, "ibm_reduce", 1);
  if (c->cfg.precision == EIF_PREC_MIXED) {
    k_chunk_reduce_f<<<(c->np * 32 + 255) / 256, 256, 0, c->stream>>>(reinterpret_cast<const float *>(c->partial),
                                                                        c->chunk_off, c->P, c->pcap, c->np, f0, f1,
                                                                        f2, bounds_of(c));
  } else {
    k_chunk_reduce<<<(c->np * 32 + 255) / 256, 256, 0, c->stream>>>(c->partial, c->chunk_off, c->P, c->pcap, c->np,
                                                                      f0, f1, f2, bounds_of(c));
  }
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

int launch_inertia(eif_ctx *c, int cn) {
  if (c->np == 0) return EIF_OK;
  int rc = launch_boxes(c, true);
  if (rc) return rc;
  return launch_work(c, 0, cn);
}

static int band_lists_of_boxes(eif_ctx *c);

// ordered box lists per band of GTY rows for the gather, from the boxes at X
int launch_band_lists(eif_ctx *c) {
  if (c->np == 0) return EIF_OK;
  int rc = launch_boxes(c, false);
  if (rc) return rc;
  return band_lists_of_boxes(c);
}

// the band lists of the boxes currently built
static int band_lists_of_boxes(eif_ctx *c) {
  const int nbands = (c->jtot + GTY - 1) / GTY;
  const int words = (3 * c->np + 31) / 32;
  EIF_PROF(c, "ibm_band_lists", 2);
  EIF_CK(c, cudaMemsetAsync(c->band_marks, 0, sizeof(unsigned) * (size_t)nbands * words, c->stream));
  k_band_marks<<<(c->np + 127) / 128, 128, 0, c->stream>>>(c->box, c->chunk_off, c->np, c->jtot, c->band_marks,
                                                           words, c->edesc, bounds_of(c));
  EIF_LAUNCH_CK(c);
  k_band_lists<<<(nbands * 32 + 255) / 256, 256, 0, c->stream>>>(c->band_marks, words, c->jtot, c->band_lists,
                                                                   c->band_counts, c->band_cap, c->d_flags);
  EIF_LAUNCH_CK(c);
  c->bands_x_valid = c->boxes_x_valid;
  return EIF_OK;
}

int launch_exchange(eif_ctx *c) {
  if (c->np == 0) {
    EIF_PROF(c, "ibm_gather", 0);
    EIF_CK(c, cudaMemsetAsync(c->dux, 0, sizeof(double) * c->nfield, c->stream));
    EIF_CK(c, cudaMemsetAsync(c->duy, 0, sizeof(double) * c->nfield, c->stream));
    return EIF_OK;
  }
  int rc = launch_boxes(c, false);
  if (rc) return rc;
  rc = launch_work(c, 1, 0);
  if (rc) return rc;
  GatherArgs g;
  g.edesc = c->edesc; g.wbuf = c->wbuf;
  g.dux = c->dux; g.duy = c->duy; g.flags = c->d_flags;
  g.np = c->np; g.itot = c->itot; g.jtot = c->jtot; g.ld = c->ld;
  g.bd = bounds_of(c);
  g.lists = c->band_lists; g.counts = c->band_counts; g.cap = c->band_cap;
  if (!(c->boxes_x_valid && c->bands_x_valid) && (rc = launch_band_lists(c))) return rc;
  dim3 grid((c->itot + GTX - 1) / GTX, (c->jtot + GTY - 1) / GTY);
  EIF_PROF(c, "ibm_gather", 2);
  const int nhalo = 2 * (c->itot + 2) + 2 * c->jtot;
  if (c->cfg.precision == EIF_PREC_MIXED) {
    k_gather<float2, float><<<grid, GTHREADS, 0, c->stream>>>(g);
    EIF_LAUNCH_CK(c);
    k_ibm_halo<float><<<(nhalo + 255) / 256, 256, 0, c->stream>>>(reinterpret_cast<float *>(c->dux),
                                                                  reinterpret_cast<float *>(c->duy), c->itot,
                                                                  c->jtot, c->ld);
  } else {
    k_gather<double2, double><<<grid, GTHREADS, 0, c->stream>>>(g);
    EIF_LAUNCH_CK(c);
    k_ibm_halo<double><<<(nhalo + 255) / 256, 256, 0, c->stream>>>(c->dux, c->duy, c->itot, c->jtot, c->ld);
  }
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

}  // namespace eif

// ---------------------------------------------------------------------------
// Transposed box evaluations for the discrete adjoint (double precision).
//
// The inertia integrals I = sum_cells w_v(D) (u_c, r x u_c) dxdy / (m, I_z)
// (inertia.c:41-52) and the exchange sums F = -sum_cells w_s(D) (U_r - u_c) dxdy
// / (dt m, dt I_z) with the field response dux = sum w_s (U_r - u_c)
// (exchange.c:61-76) depend on the cell velocities u_c (face averages), on the
// particle velocities U, Omega, and on the centre and angle through the lever arm
// r = x - X and the signed distance D = d/h of the cell centre. With q = R(-az) r
// the body-frame offset and the distance computed through the normal foot
// (ellipse.c:30-65), dD/dq at the foot is minus the outward unit normal over h
// (the foot parameter is stationary, so it does not contribute), hence
//   dD/dX = -g,   dD/daz = g_x r_y - g_y r_x,   g = R(az) dD/dq.
// w_v = (1 + tanh(2D))/2 has dw_v/dD = w_s, and w_s = 1 - tanh^2(2D) has
// dw_s/dD = -4 tanh(2D) w_s.
//
// One warp per box row task as in k_ibm_work. Per cell the kernel writes the cell
// cotangent of the face-averaged velocity into the scratch buffer (gathered per
// cell afterwards in the fixed order of the forward exchange) and sums per task the
// cotangents of (X, Y, az) and (U, V, Omega). Boxes are those of the forward
// evaluation (the loop bounds are piecewise constant in the positions).
namespace {

struct AdjWorkArgs {
  const double *P;
  const double *ux, *uy, *xc, *yc, *dt;
  const int *off;
  const int4 *tdesc;
  const double *bar;        // 3 x np: inertia cotangent (mode 0) or force cotangent (mode 1)
  const double *gx, *gy;    // mode 1: cell cotangents of the field response
  double *part;             // 6 per task
  double2 *wbuf;
  double *geom;             // geo 1/2: per task slot th, gwx, gwy (3 x slots, by component)
  long long nslot;
  int geo;
  int pcap, np, ld, mode, use_increment;
  double dx, dy, ly, h;
  Bounds bd;
};

__global__ void __launch_bounds__(256) k_ibm_adj(AdjWorkArgs a) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int total = EIF_CHK(a.bd.rec, a.np, a.bd.off, 70) ? __ldg(a.off + a.np) : 0;
  const double rh = 1. / a.h;
  const double dxdy = a.dx * a.dy;
  const double kdt = a.mode == 1 ? dxdy / __ldg(a.dt) : 0.;
  const int pc = a.pcap, ld = a.ld;
  for (int c = warp; c < total; c += nwarps) {
    if (!EIF_CHK(a.bd.rec, 6LL * c + 5, 6LL * (a.bd.partial / 3), 71)) continue;
    const int4 dsc = __ldg(a.tdesc + c);
    const int n = dsc.x;
    if (!EIF_CHK(a.bd.rec, n, a.np, 72)) continue;
    RowTask t;
    const bool task = task_of(dsc, a.np, t) && EIF_CHK(a.bd.rec, t.j, a.bd.yc - 1, 73);
    const double *P = a.P;
    const double pden = __ldg(P + EIF_P_DEN * pc + n), pa = __ldg(P + EIF_P_A * pc + n), pb = __ldg(P + EIF_P_B * pc + n);
    double px = __ldg(P + EIF_P_X * pc + n), py = __ldg(P + EIF_P_Y * pc + n), paz = __ldg(P + EIF_P_AZ * pc + n);
    if (a.use_increment) {
      px = px + __ldg(P + EIF_P_DX * pc + n);
      py = py + __ldg(P + EIF_P_DY * pc + n);
      paz = paz + __ldg(P + EIF_P_DAZ * pc + n);
    }
    const double pm = pmass(pden, pa, pb), pim = pmoi(pden, pa, pb);
    const double pux = __ldg(P + EIF_P_UX * pc + n), puy = __ldg(P + EIF_P_UY * pc + n), pvz = __ldg(P + EIF_P_VZ * pc + n);
    const double b0 = __ldg(a.bar + n), b1 = __ldg(a.bar + a.np + n), b2 = __ldg(a.bar + 2 * a.np + n);
    const Ell e = make_ell(pa, pb, px, py, paz);
    const double py_ = py + a.ly * (task ? t.img : 0);
    const int j = task ? t.j : 1;
    const double y = __ldg(a.yc + j);
    const double ry = y - py_;
    const double mn = fmin(pa, pb);
    double sX = 0., sY = 0., sA = 0., sU = 0., sV = 0., sW = 0.;
#pragma unroll 1
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      bool in = task && i <= t.ie;
      if (in) {
        in = EIF_CHK(a.bd.rec, i, a.bd.xc - 1, 74) && EIF_CHK(a.bd.rec, j * ld + i, a.bd.field, 75) &&
             EIF_CHK(a.bd.rec, (j + 1) * ld + i, a.bd.field, 76) && EIF_CHK(a.bd.rec, j * ld + (i - 1), a.bd.field, 77);
      }
      double2 contrib = make_double2(0., 0.);
      if (in) {
        const double x = __ldg(a.xc + i);
        const double rx = x - px;
        const double qx = e.cz * rx - e.sz * ry, qy = e.sz * rx + e.cz * ry;
        // distance bound from the gauge of the ellipse: beyond FAR_CELLS_D cells tanh(2D)
        // is +-1 in double precision and both weights' derivatives vanish
        const double rho = sqrt((qx / pa) * (qx / pa) + (qy / pb) * (qy / pb));
        double th, gwx = 0., gwy = 0.;
        const long long slot = (long long)c * CHUNK + half * 32 + lane;
        const bool cached = a.geo == 2 && EIF_CHK(a.bd.rec, slot, a.nslot, 81);
        if (cached) {
          th = a.geom[slot];
          gwx = a.geom[a.nslot + slot];
          gwy = a.geom[2 * a.nslot + slot];
        } else if (mn * fabs(rho - 1.) * rh >= FAR_CELLS_D) {
          th = rho < 1. ? 1. : -1.;
        } else {
          const double f0 = 1. - (qx / pa) * (qx / pa) - (qy / pb) * (qy / pb);
          const double sign = f0 > 0. ? 1. : -1.;
          const double tt = normal_t(e, qx, qy);
          double st, ct;
          sincos(tt, &st, &ct);
          const double fx = pa * ct - qx, fy = pb * st - qy;
          th = tanh(BETA * (sign * sqrt(fx * fx + fy * fy) * rh));
          // outward normal at the foot (cos t / a, sin t / b); dD/dq = -n / h
          double nx = ct / pa, ny = st / pb;
          const double nn = 1. / sqrt(nx * nx + ny * ny);
          nx *= nn;
          ny *= nn;
          const double gbx = -nx * rh, gby = -ny * rh;
          // g = R(az) dD/dq with cz = cos(-az), sz = sin(-az)
          gwx = e.cz * gbx + e.sz * gby;
          gwy = -e.sz * gbx + e.cz * gby;
        }
        if (a.geo == 1 && EIF_CHK(a.bd.rec, slot, a.nslot, 82)) {
          a.geom[slot] = th;
          a.geom[a.nslot + slot] = gwx;
          a.geom[2 * a.nslot + slot] = gwy;
        }
        const double ws = 0.5 * BETA * (1. - th * th);
        const double uxf = 0.5 * (__ldg(a.ux + j * ld + (i - 1)) + __ldg(a.ux + j * ld + i));
        const double uyf = 0.5 * (__ldg(a.uy + j * ld + i) + __ldg(a.uy + (j + 1) * ld + i));
        const double dDdaz = gwx * ry - gwy * rx;
        if (a.mode == 0) {
          const double wv = 0.5 * (1. + th);
          const double cx = b0 / pm, cy = b1 / pm, cz = b2 / pim;
          contrib = make_double2(wv * dxdy * (cx - cz * ry), wv * dxdy * (cy + cz * rx));
          const double sv = dxdy * (cx * uxf + cy * uyf + cz * (-ry * uxf + rx * uyf));
          const double dw = ws * sv;
          sX += -dw * gwx - wv * dxdy * cz * uyf;
          sY += -dw * gwy + wv * dxdy * cz * uxf;
          sA += dw * dDdaz;
        } else {
          const int cc = j * ld + i;
          const double urx = pux - pvz * ry, ury = puy + pvz * rx;
          const double ex = urx - uxf, ey = ury - uyf;
          const double Cx = __ldg(a.gx + cc) - b0 * kdt / pm + b2 * ry * kdt / pim;
          const double Cy = __ldg(a.gy + cc) - b1 * kdt / pm - b2 * rx * kdt / pim;
          const double Ex = ws * Cx, Ey = ws * Cy;
          contrib = make_double2(-Ex, -Ey);
          sU += Ex;
          sV += Ey;
          sW += -ry * Ex + rx * Ey;
          const double dw = (ex * Cx + ey * Cy) * (-2. * BETA * th * ws);
          sX += -dw * gwx - pvz * Ey + b2 * ws * ey * kdt / pim;
          sY += -dw * gwy + pvz * Ex - b2 * ws * ex * kdt / pim;
          sA += dw * dDdaz;
        }
      }
      if (EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, a.bd.wbuf, 78))
        a.wbuf[(size_t)c * CHUNK + half * 32 + lane] = contrib;
    }
    sX = eifd::warp_sum(sX);
    sY = eifd::warp_sum(sY);
    sA = eifd::warp_sum(sA);
    sU = eifd::warp_sum(sU);
    sV = eifd::warp_sum(sV);
    sW = eifd::warp_sum(sW);
    if (lane == 0) {
      double *q = a.part + 6 * (size_t)c;
      q[0] = sX; q[1] = sY; q[2] = sA; q[3] = sU; q[4] = sV; q[5] = sW;
    }
  }
}

// per-particle sums of the task cotangents in task order: out[k * np + n]
__global__ void k_adj_chunk_reduce(const double *__restrict__ part, const int *__restrict__ off,
                                   double *__restrict__ out, int np, Bounds bd) {
  const int lane = threadIdx.x & 31;
  const int n = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (n >= np) return;
  if (!EIF_CHK(bd.rec, n + 1, bd.off, 79)) return;
  const int c0 = off[n], c1 = off[n + 1];
  double s[6] = {0., 0., 0., 0., 0., 0.};
  for (int c = c0 + lane; c < c1; c += 32) {
    if (!EIF_CHK(bd.rec, 6LL * c + 5, 6LL * (bd.partial / 3), 80)) break;
#pragma unroll
    for (int k = 0; k < 6; k++) s[k] += part[6 * (size_t)c + k];
  }
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const double v = eifd::warp_sum(s[k]);
    if (lane == 0) out[(size_t)k * np + n] = v;
  }
}

}  // namespace

namespace eif {

int launch_adj_pass(eif_ctx *c, const AdjPass &p) {
  if (c->np == 0) return EIF_OK;
  if (p.use_increment) c->incr_zero = false;
  int rc = launch_boxes(c, p.use_increment);
  if (rc) return rc;
  AdjWorkArgs w;
  w.P = c->P; w.ux = p.ux; w.uy = p.uy; w.xc = c->xc; w.yc = c->yc; w.dt = c->d_scal;
  w.off = c->chunk_off; w.tdesc = c->tdesc;
  w.bar = p.bar; w.gx = p.gx; w.gy = p.gy;
  w.part = p.part;
  w.wbuf = reinterpret_cast<double2 *>(c->wbuf);
  w.geom = p.geom;
  w.nslot = (long long)c->wcap;
  w.geo = p.geom ? p.geo : 0;
  w.pcap = c->pcap; w.np = c->np; w.ld = c->ld; w.mode = p.mode; w.use_increment = p.use_increment ? 1 : 0;
  w.dx = c->dx; w.dy = c->dy; w.ly = c->ly; w.h = std::min(c->dx, c->dy);
  w.bd = bounds_of(c);
  const int blocks = std::max(1, std::min(c->sms * 8, (c->chunk_cap * 32 + 255) / 256));
  k_ibm_adj<<<blocks, 256, 0, c->stream>>>(w);
  EIF_LAUNCH_CK(c);
  k_adj_chunk_reduce<<<(c->np * 32 + 255) / 256, 256, 0, c->stream>>>(p.part, c->chunk_off, p.out, c->np,
                                                                        bounds_of(c));
  EIF_LAUNCH_CK(c);
  if ((rc = band_lists_of_boxes(c))) return rc;
  GatherArgs g;
  g.edesc = c->edesc; g.wbuf = c->wbuf;
  g.dux = p.fx; g.duy = p.fy; g.flags = c->d_flags;
  g.np = c->np; g.itot = c->itot; g.jtot = c->jtot; g.ld = c->ld;
  g.bd = bounds_of(c);
  g.lists = c->band_lists; g.counts = c->band_counts; g.cap = c->band_cap;
  dim3 grid((c->itot + GTX - 1) / GTX, (c->jtot + GTY - 1) / GTY);
  k_gather<double2, double><<<grid, GTHREADS, 0, c->stream>>>(g);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

int adj_chunk_cap(const eif_ctx *c) { return c->chunk_cap; }
size_t adj_slot_cap(const eif_ctx *c) { return c->wcap; }

}  // namespace eif
