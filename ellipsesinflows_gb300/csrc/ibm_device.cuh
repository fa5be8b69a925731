// Device code of the immersed-boundary evaluations shared by the stand-alone
// kernels (ibm.cu) and the batch's per-stage sub-iteration kernel (subiter.cu):
// geometry helpers, the per-particle boxes, the task table and the per-task and
// per-particle bodies of the volume integrals and the momentum exchange.
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
// Loads through the read-only data path (__ldg) are only valid for data that no
// thread writes while the kernel runs. The bodies take a template flag NC: true in
// the stand-alone single-precision kernels, false in the persistent sub-iteration
// kernel, whose phases write the particle records, boxes, task table and parameters
// that later phases read (there those loads are ordinary, coherent after the grid
// barrier), and false in both for the double-precision task body, so that both run
// one instantiation of it.
#pragma once
#include "eif_internal.cuh"
#include <cfloat>

namespace {

// a load through the read-only path when NC, an ordinary load otherwise
template <bool NC, typename T>
__device__ __forceinline__ T ldro(const T *p) {
  if constexpr (NC) return __ldg(p);
  else return *p;
}

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

// ---------------------------------------------------------------------------
// The normal-foot iteration of ellipse.c:30-65 in single precision (the mixed form's
// indicator, and the start of the double-precision iteration below). The distance at
// the foot is stationary in t, so an angle error dt changes it by O(a dt^2): stopping
// once the step is below 1e-3 leaves distance errors near 1e-9 cells (checked against
// fully converged iterations over the aspect ratios 1-3).
constexpr float NORMAL_TOL_F = 1.e-3f;
constexpr int NORMAL_MAX_F = 24;

struct EllF {
  float a, b, cz, sz, kex, key;
};

// The reference's iteration (ellipse.c:30-65) in single precision, on the first-quadrant
// offsets (px, py) = (|x_|, |y_|); normal_t_f unfolds the angle. Its fixed point
// is the normal foot whatever the accuracy of the intermediate sin/cos, square
// roots and arcsine, so the loop uses the hardware approximations (__sincosf,
// rsqrtf) and the Taylor polynomial x + x^3/6 + 3x^5/40 of asin (odd, increasing
// and zero only at zero like asin, so the step keeps its sign and vanishes at the
// foot); the distance at the converged angle is evaluated with the accurate
// sincosf, and the distance is stationary in the angle.
__device__ __forceinline__ float normal_t_f_q1(const EllF &e, float px, float py) {
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
  return t;
}
__device__ __forceinline__ float normal_t_f(const EllF &e, float x_, float y_) {
  float t = normal_t_f_q1(e, fabsf(x_), fabsf(y_));
  if (x_ < 0.f) t = 3.14159265358979323846f - t;
  if (y_ < 0.f) t = -t;
  return t;
}


// ellipse.c:30-65 (x_, y_ in the body frame). The iteration, its stopping rule and its
// cap are the reference's; it starts from the foot that the same iteration finds in
// single precision (on the FP32 pipe, about 1e-4 or closer) instead of from pi/4. The
// fixed point is the same, and the double-precision iterations (the expensive part on
// this GPU's FP64 pipe) drop from about four to two: the first moves t by the start's
// error, the second by its square, below the 1e-8 stop. Not inlined, like
// ibm_work_tasks: compiled on its own it gives the same bits in every kernel.
__device__ __noinline__ double normal_t(const Ell &e, double x_, double y_) {
  const double px = fabs(x_), py = fabs(y_);
  EllF ef;
  ef.a = eifd::d2f(e.a); ef.b = eifd::d2f(e.b); ef.kex = eifd::d2f(e.kex); ef.key = eifd::d2f(e.key);
  ef.cz = 0.f; ef.sz = 0.f;
  double t = eifd::f2d(normal_t_f_q1(ef, eifd::d2f(px), eifd::d2f(py)));
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

using eifd::pmass;
using eifd::pmoi;

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
// the work is split into eight parts run by different warps, each over 32
// particles: parts 0-2 the boxes of images -1, 0, +1 (their task counts are added to
// nchunk, zeroed before), parts 3-7 groups of parameters (mixed form only). One
// thread: particle n, part sub.
constexpr int BOX_PARTS = 8;
__device__ __forceinline__ void box_part(const BoxArgs &a, int n, int sub) {
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

// The same table with the task offsets formed in the same kernel, for particle
// counts up to TT_MAX_NP: every block sums the task counts of the particles before
// its own (a few thousand integers from L2), then each warp writes its particle's
// offset and table entries. Replaces k_scan + k_task_table (one launch and one
// single-block pass fewer on the path of every box build). One block of TT_WARPS
// warps: particles block * TT_WARPS ...
constexpr int TT_WARPS = 8;
constexpr int TT_MAX_NP = 8192;
__device__ __forceinline__ void task_table_block(const int *box, const int *cnt, int *off, int4 *tdesc, int np,
                                                 const Bounds &bd, int cap, int block) {
  __shared__ int red[TT_WARPS], wcnt[TT_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n0 = block * TT_WARPS;
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

// The last indicator evaluation of the mixed form inside a sub-iteration loop (at the
// positions X + dX of a sub-iteration after the first): its weights, one per task slot,
// and the particles' geometry parameters (the PF_WORDS block), boxes and first task,
// with a flag set once a complete evaluation is stored. The loop stops when the
// increments have settled, so the positions X of the next stage differ from those by
// the last change of the increments (below 1e-8 dt in velocity); the single-precision
// geometry of nearly every particle is then bitwise the stored one, and so are its
// weights, which the next stage's first evaluation copies instead of recomputing.
struct WeightMemo {
  float *w;
  float *pf;
  int *box, *off;
  int *valid;
};
// geometry words of the per-particle parameter block (everything but the mass, inertia
// and velocity words PF_RPM .. PF_VZ); with the 12 box bounds, 32 words: one per lane
__device__ __forceinline__ int memo_word(int lane) { return lane < 6 ? lane : lane + 5; }

struct WorkArgs {
  const double *P;
  const double *ux, *uy, *xc, *yc, *dt;
  // mixed form: ux, uy rounded to float (eifd::d2f), kept with them by the kernels that
  // write the velocities; the single-precision bodies read these
  const float *uxf, *uyf;
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
  // normal-foot iteration, added to count[0] and count[1], and the tasks whose weights
  // come from the memo, added to count[2] (null: not counted)
  unsigned long long *count;
  // mixed form: memo_mode 1 (the stage start, ibm_memo_f_tasks) takes the weights of a
  // task from the memo when its particle's geometry and boxes are the memo's; 2
  // (ibm_work_f_tasks in the loops) stores computed weights in it
  WeightMemo memo;
  int memo_mode;
  // the stage start of the mixed form (ibm_memo_f_tasks): miss[0] counts the tasks the
  // memo did not serve, miss[1 ..] lists them; with `only` set, ibm_work_f_tasks
  // evaluates just the tasks listed there (same layout)
  int *miss;
  const int *only;
  Bounds bd;
};

// One warp per row task: indicator weights, partial sums, and (for the exchange)
// per-cell field contributions. The warp runs the tasks first, first + stride, ...
// with the weight mode wmode; slots: CHUNK entries of shared memory of its own.
// Not inlined: compiled on its own, the double-precision arithmetic (its contractions
// into fused multiply-adds) is the same in every kernel that calls it, so the batch's
// stage kernel gives the bits of the stand-alone kernel.
template <bool NC>
__device__ __noinline__ void ibm_work_tasks(const WorkArgs &a, int wmode, int first, int stride, double2 *slots) {
  const int lane = threadIdx.x & 31;
  const int total = EIF_CHK(a.bd.rec, a.np, a.bd.off, 10) ? ldro<NC>(a.off + a.np) : 0;
  const double rh = 1. / a.h;
  const double dxdy = a.dx * a.dy;
  const double dtv = a.mode == 1 ? __ldg(a.dt) : 0.;
  const double rdtv = a.mode == 1 ? 1. / dtv : 0.;
  const double md = FAR_CELLS_D * a.h;
  const int pc = a.pcap, ld = a.ld;
  double *wcache = static_cast<double *>(a.wcache);
  for (int c = first; c < total; c += stride) {
    if (!EIF_CHK(a.bd.rec, c, a.bd.partial / 3, 21)) continue;
    const int4 dsc = ldro<NC>(a.tdesc + c);
    const int n = dsc.x;
    if (!EIF_CHK(a.bd.rec, n, a.np, 11)) continue;
    if (!EIF_CHK(a.bd.rec, EIF_P_VZ * pc + n, a.bd.P, 13)) continue;
    RowTask t;
    const bool task = task_of(dsc, a.np, t) && EIF_CHK(a.bd.rec, t.j, a.bd.yc - 1, 15);
    const double *P = a.P;
    const double pden = ldro<NC>(P + EIF_P_DEN * pc + n), pa = ldro<NC>(P + EIF_P_A * pc + n),
                 pb = ldro<NC>(P + EIF_P_B * pc + n);
    double px = ldro<NC>(P + EIF_P_X * pc + n), py = ldro<NC>(P + EIF_P_Y * pc + n), paz = ldro<NC>(P + EIF_P_AZ * pc + n);
    if (a.mode == 0) {
      // inertia.c:29-31: positions at k + increment
      px = px + ldro<NC>(P + EIF_P_DX * pc + n);
      py = py + ldro<NC>(P + EIF_P_DY * pc + n);
      paz = paz + ldro<NC>(P + EIF_P_DAZ * pc + n);
    }
    // reciprocals of the mass and the moment of inertia, once per task: the per-cell
    // divisions of inertia.c and exchange.c become multiplications (a division costs
    // about ten FP64 operations; the results change by an ulp per term)
    const double rpm = 1. / pmass(pden, pa, pb);
    const double rpim = 1. / pmoi(pden, pa, pb);
    const double pux = ldro<NC>(P + EIF_P_UX * pc + n), puy = ldro<NC>(P + EIF_P_UY * pc + n),
                 pvz = ldro<NC>(P + EIF_P_VZ * pc + n);
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
          s0 += valx * rpm;
          s1 += valy * rpm;
          s2 += (-(y - py_) * valx * rpim) + ((x - px) * valy * rpim);
        } else {
          // exchange.c:61-76
          const double w = 0.5 * BETA * (1. - th * th);
          const double uxp = pux - pvz * (y - py_);
          const double uyp = puy + pvz * (x - px);
          const double fx = w * (uxp - uxf) * rdtv;
          const double fy = w * (uyp - uyf) * rdtv;
          contrib = a.weights_only ? make_double2(w, w) : make_double2(fx * dtv, fy * dtv);
          const double Fx = fx * a.dx * a.dy, Fy = fy * a.dx * a.dy;
          s0 += -(Fx * rpm);
          s1 += -(Fy * rpm);
          s2 += ((y - py_) * Fx * rpim) - ((x - px) * Fy * rpim);
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
// foot iteration is normal_t_f (above).

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

// One cell's contributions to the inertia integrals (inertia.c:9-70) in single precision,
// with every rounding explicit: the bodies that form these sums (the full evaluation, the
// memo-served stage start, the cached-weight sums) then give the same bits in whatever
// kernel they are compiled, whichever products the compiler would fuse there.
__device__ __forceinline__ void inertia_cell_f(float th, float X, float Y, float uxs, float uys, float dxdy,
                                               float rpm, float rpim, float &s0, float &s1, float &s2) {
  const float w = __fmul_rn(0.5f, __fadd_rn(1.f, th));
  const float valx = __fmul_rn(__fmul_rn(__fmul_rn(w, 0.5f), uxs), dxdy);
  const float valy = __fmul_rn(__fmul_rn(__fmul_rn(w, 0.5f), uys), dxdy);
  s0 = __fmaf_rn(valx, rpm, s0);
  s1 = __fmaf_rn(valy, rpm, s1);
  s2 = __fmaf_rn(__fmaf_rn(X, valy, __fmul_rn(-Y, valx)), rpim, s2);
}

// one warp per row task, single precision (see ibm_work_tasks)
template <bool NC>
__device__ __forceinline__ void ibm_work_f_tasks(const WorkArgs &a, int wmode, int first, int stride, float2 *slots) {
  const int lane = threadIdx.x & 31;
  // all tasks, or (with a.only) the listed ones: task number c of list entry k
  const int total = a.only ? (int)min((long long)ldro<NC>(a.only), (long long)(a.bd.partial / 3))
                           : (EIF_CHK(a.bd.rec, a.np, a.bd.off, 50) ? ldro<NC>(a.off + a.np) : 0);
  auto task_no = [&](int k) { return a.only ? ldro<NC>(a.only + 1 + k) : k; };
  const float rh = a.rh_f, dxf = a.dx_f, dyf = a.dy_f, dxdy = a.dxdy_f;
  const float rdtv = a.mode == 1 ? __ldg(a.coef + 9) : 0.f;
  const int ld = a.ld;
  float2 *wb = reinterpret_cast<float2 *>(a.wbuf);
  float *wcache = static_cast<float *>(a.wcache);
  // the next task's table entry is loaded while the current task is processed
  int4 nxt = make_int4(-1, 0, 0, 0);
  if (first < total) {
    const int cf = task_no(first);
    if (EIF_CHK(a.bd.rec, cf, a.bd.partial / 3, 51)) nxt = ldro<NC>(a.tdesc + cf);
  }
  for (int k = first; k < total; k += stride) {
    const int c = task_no(k);
    const int4 dsc = nxt;
    if (k + stride < total) {
      const int cn = task_no(k + stride);
      if (EIF_CHK(a.bd.rec, cn, a.bd.partial / 3, 51)) nxt = ldro<NC>(a.tdesc + cn);
    }
    const int n = dsc.x;
    if (!EIF_CHK(a.bd.rec, n, a.np, 52)) continue;
    RowTask t;
    const bool task = task_of(dsc, a.np, t);
    const float4 *q4 = reinterpret_cast<const float4 *>(a.pf + (size_t)PF_WORDS * n);
    const float4 qA = ldro<NC>(q4), qB = ldro<NC>(q4 + 1), qC = ldro<NC>(q4 + 2), qD = ldro<NC>(q4 + 3),
                 qE = ldro<NC>(q4 + 4);
    const float4 qF = ldro<NC>(q4 + 5), qG = ldro<NC>(q4 + 6);
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
    // the cells of the task and their field values: loaded before the geometry, so that
    // the loads are in flight while the weights are evaluated
    float fuw[2], fue[2], fvs[2], fvn[2];
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      bool in = task && i <= t.ie;
      if (in) {
        in = EIF_CHK(a.bd.rec, j * ld + i, a.bd.field, 54) && EIF_CHK(a.bd.rec, (j + 1) * ld + i, a.bd.field, 55) &&
             EIF_CHK(a.bd.rec, j * ld + (i - 1), a.bd.field, 56);
      }
      cin[half] = in;
      fuw[half] = fue[half] = fvs[half] = fvn[half] = 0.f;
      if (in) {
        fuw[half] = __ldg(a.uxf + j * ld + (i - 1));
        fue[half] = __ldg(a.uxf + j * ld + i);
        fvs[half] = __ldg(a.uyf + j * ld + i);
        fvn[half] = __ldg(a.uyf + (j + 1) * ld + i);
      }
    }
    // (the stage start's weights from the memo are taken by ibm_memo_f_tasks, which
    // leaves this body only the tasks the memo did not serve)
    if (wmode == 2) {
      // weights of the same geometry from an earlier evaluation
#pragma unroll
      for (int half = 0; half < CHUNK / 32; half++) {
        const int i = (task ? t.ib : 1) + half * 32 + lane;
        if (cin[half]) cin[half] = EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, 2 * a.bd.wbuf, 59);
        cX[half] = ((float)(i - i0) - gx) * dxf;
        th2[half] = cin[half] ? wcache[(size_t)c * CHUNK + half * 32 + lane] : 0.f;
      }
    } else {
    // far cells of this row (PF_AL .. PF_RO2: al, ka, de, so^2, si^2, ro^2)
    float olo, ohi, ilo, ihi;
    row_chords(qE.w, qF.x, qF.y, qF.z, qF.w, qG.x, Y, olo, ohi, ilo, ihi);
    // pass 1: cells of the row, far cells settled, body-frame offsets of the near ones
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      const bool in = cin[half];
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
    if (a.memo_mode == 2) {
#pragma unroll
      for (int half = 0; half < CHUNK / 32; half++)
        if (EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, a.bd.wbuf, 61))
          a.memo.w[(size_t)c * CHUNK + half * 32 + lane] = th2[half];
    }
    }
    if (wmode == 1) {
#pragma unroll
      for (int half = 0; half < CHUNK / 32; half++)
        if (EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, 2 * a.bd.wbuf, 60))
          wcache[(size_t)c * CHUNK + half * 32 + lane] = th2[half];
    }
    float sacc0 = 0.f, sacc1 = 0.f, sacc2 = 0.f;
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      float2 contrib = make_float2(0.f, 0.f);
      // cells of weight exactly zero (inertia: far outside; exchange: any far cell) are skipped
      const float th_ = th2[half];
      const bool live = a.mode == 0 ? th_ != -1.f : fabsf(th_) != 1.f;
      if (cin[half] && live) {
        const float X = cX[half], th = th_;
        const float uxs = fuw[half] + fue[half];
        const float uys = fvs[half] + fvn[half];
        if (a.mode == 0) {
          inertia_cell_f(th, X, Y, uxs, uys, dxdy, rpm, rpim, sacc0, sacc1, sacc2);
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

// The stage start of the mixed form (inertia at X with zero increments, weights stored for
// the stage: wmode 1, memo_mode 1 of ibm_work_f_tasks) without the geometry code: a task
// whose particle geometry words and boxes are bitwise those of the memo takes the memo's
// weights, stores them in wcache and forms its sums exactly as ibm_work_f_tasks does;
// any other task is appended to a.miss for k_ibm_work_f, which evaluates those in full.
// It runs with the registers of the sums kernel, so more warps hide its loads.
template <bool NC>
__device__ __forceinline__ void ibm_memo_f_tasks(const WorkArgs &a, int first, int stride) {
  const int lane = threadIdx.x & 31;
  const int total = EIF_CHK(a.bd.rec, a.np, a.bd.off, 90) ? ldro<NC>(a.off + a.np) : 0;
  const float dxf = a.dx_f, dyf = a.dy_f, dxdy = a.dxdy_f;
  const int ld = a.ld;
  float *wcache = static_cast<float *>(a.wcache);
  const bool valid = ldro<NC>(a.memo.valid) != 0;
  for (int c = first; c < total; c += stride) {
    if (!EIF_CHK(a.bd.rec, c, a.bd.partial / 3, 91)) continue;
    const int4 dsc = ldro<NC>(a.tdesc + c);
    const int n = dsc.x;
    if (!EIF_CHK(a.bd.rec, n, a.np, 92)) continue;
    bool eq = false;
    if (valid) {
      if (lane < 20) {
        const size_t q = (size_t)PF_WORDS * n + memo_word(lane);
        eq = __float_as_uint(ldro<NC>(a.pf + q)) == __float_as_uint(ldro<NC>(a.memo.pf + q));
      } else {
        const size_t q = 12 * (size_t)n + (lane - 20);
        eq = ldro<NC>(a.box + q) == ldro<NC>(a.memo.box + q);
      }
    }
    if (!__all_sync(0xffffffffu, eq)) {
      if (lane == 0) {
        const int k = atomicAdd(a.miss, 1);
        if (EIF_CHK(a.bd.rec, k, a.bd.partial / 3, 93)) a.miss[1 + k] = c;
      }
      continue;
    }
    if (a.count && lane == 0) atomicAdd(a.count + 2, 1ull);
    const long long src = (long long)c + (ldro<NC>(a.memo.off + n) - ldro<NC>(a.off + n));
    RowTask t;
    const bool task = task_of(dsc, a.np, t);
    const float4 *q4 = reinterpret_cast<const float4 *>(a.pf + (size_t)PF_WORDS * n);
    const float4 qB = ldro<NC>(q4 + 1), qC = ldro<NC>(q4 + 2), qD = ldro<NC>(q4 + 3), qE = ldro<NC>(q4 + 4);
    const float rpm = qB.z, rpim = qB.w, gx = qC.w;
    const int i0 = __float_as_int(qD.x);
    const int m = task ? t.img + 1 : 1;
    const int j0i = __float_as_int(m == 0 ? qD.y : (m == 1 ? qD.z : qD.w));
    const float gyi = m == 0 ? qE.x : (m == 1 ? qE.y : qE.z);
    const int j = task ? t.j : 1;
    const float Y = ((float)(j - j0i) - gyi) * dyf;
    bool cin[2];
    float cX[2], th2[2], fuw[2], fue[2], fvs[2], fvn[2];
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      bool in = task && i <= t.ie;
      if (in) {
        in = EIF_CHK(a.bd.rec, j * ld + i, a.bd.field, 94) && EIF_CHK(a.bd.rec, (j + 1) * ld + i, a.bd.field, 95) &&
             EIF_CHK(a.bd.rec, j * ld + (i - 1), a.bd.field, 96);
      }
      fuw[half] = fue[half] = fvs[half] = fvn[half] = 0.f;
      if (in) {
        fuw[half] = __ldg(a.uxf + j * ld + (i - 1));
        fue[half] = __ldg(a.uxf + j * ld + i);
        fvs[half] = __ldg(a.uyf + j * ld + i);
        fvn[half] = __ldg(a.uyf + (j + 1) * ld + i);
      }
      if (in) in = EIF_CHK(a.bd.rec, src * CHUNK + half * 32 + lane, a.bd.wbuf, 97);
      cin[half] = in;
      cX[half] = ((float)(i - i0) - gx) * dxf;
      th2[half] = in ? a.memo.w[(size_t)src * CHUNK + half * 32 + lane] : 0.f;
    }
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++)
      if (EIF_CHK(a.bd.rec, (long long)c * CHUNK + half * 32 + lane, 2 * a.bd.wbuf, 98))
        wcache[(size_t)c * CHUNK + half * 32 + lane] = th2[half];
    float sacc0 = 0.f, sacc1 = 0.f, sacc2 = 0.f;
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      const float th_ = th2[half];
      if (cin[half] && th_ != -1.f) {
        const float uxs = fuw[half] + fue[half];
        const float uys = fvs[half] + fvn[half];
        inertia_cell_f(th_, cX[half], Y, uxs, uys, dxdy, rpm, rpim, sacc0, sacc1, sacc2);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sacc0 += __shfl_xor_sync(0xffffffffu, sacc0, o);
      sacc1 += __shfl_xor_sync(0xffffffffu, sacc1, o);
      sacc2 += __shfl_xor_sync(0xffffffffu, sacc2, o);
    }
    if (lane == 0 && EIF_CHK(a.bd.rec, 3LL * c + 2, a.bd.partial, 99)) {
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
// The warp runs the tasks first, first + stride, ...
template <bool NC>
__device__ __forceinline__ void ibm_sum_f_tasks(const WorkArgs &a, int first, int stride) {
  const int lane = threadIdx.x & 31;
  const int warp = first, nwarps = stride;
  const int total = EIF_CHK(a.bd.rec, a.np, a.bd.off, 70) ? ldro<NC>(a.off + a.np) : 0;
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
    nxt = ldro<NC>(a.tdesc + warp);
    nth0 = wcache[(size_t)warp * CHUNK + lane];
    nth1 = wcache[(size_t)warp * CHUNK + 32 + lane];
  }
  for (int c = warp; c < total; c += nwarps) {
    const int4 dsc = nxt;
    const float th_pre[2] = {nth0, nth1};
    const int cn = c + nwarps;
    if (cn < total && EIF_CHK(a.bd.rec, cn, a.bd.partial / 3, 71) &&
        EIF_CHK(a.bd.rec, (long long)cn * CHUNK + CHUNK - 1, 2 * a.bd.wbuf, 77)) {
      nxt = ldro<NC>(a.tdesc + cn);
      nth0 = wcache[(size_t)cn * CHUNK + lane];
      nth1 = wcache[(size_t)cn * CHUNK + 32 + lane];
    }
    const int n = dsc.x;
    if (!EIF_CHK(a.bd.rec, n, a.np, 72)) continue;
    RowTask t;
    const bool task = task_of(dsc, a.np, t);
    const float4 *q4 = reinterpret_cast<const float4 *>(a.pf + (size_t)PF_WORDS * n);
    const float4 qB = ldro<NC>(q4 + 1), qC = ldro<NC>(q4 + 2), qD = ldro<NC>(q4 + 3), qE = ldro<NC>(q4 + 4);
    const float rpm = qB.z, rpim = qB.w, pux = qC.x, puy = qC.y, pvz = qC.z, gx = qC.w;
    const int i0 = __float_as_int(qD.x);
    const int m = task ? t.img + 1 : 1;
    const int j0i = __float_as_int(m == 0 ? qD.y : (m == 1 ? qD.z : qD.w));
    const float gyi = m == 0 ? qE.x : (m == 1 ? qE.y : qE.z);
    const int j = task ? t.j : 1;
    const float Y = ((float)(j - j0i) - gyi) * dyf;
    // the field values of both halves are loaded before either is used, so that the
    // warp has all eight loads of the task in flight at once
    bool live[2];
    float thv[2];
    float uw[2], ue[2], vs[2], vn[2];
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      bool in = task && i <= t.ie;
      if (in) {
        in = EIF_CHK(a.bd.rec, j * ld + i, a.bd.field, 74) && EIF_CHK(a.bd.rec, (j + 1) * ld + i, a.bd.field, 75) &&
             EIF_CHK(a.bd.rec, j * ld + (i - 1), a.bd.field, 76);
      }
      const float th = in ? th_pre[half] : 0.f;
      thv[half] = th;
      // cells of weight exactly zero (inertia: far outside; exchange: any far cell) are skipped
      live[half] = in && (a.mode == 0 ? th != -1.f : fabsf(th) != 1.f);
      uw[half] = ue[half] = vs[half] = vn[half] = 0.f;
      if (live[half]) {
        uw[half] = __ldg(a.uxf + j * ld + (i - 1));
        ue[half] = __ldg(a.uxf + j * ld + i);
        vs[half] = __ldg(a.uyf + j * ld + i);
        vn[half] = __ldg(a.uyf + (j + 1) * ld + i);
      }
    }
    float sacc0 = 0.f, sacc1 = 0.f, sacc2 = 0.f;
#pragma unroll
    for (int half = 0; half < CHUNK / 32; half++) {
      const int i = (task ? t.ib : 1) + half * 32 + lane;
      const long long slot = (long long)c * CHUNK + half * 32 + lane;
      float2 contrib = make_float2(0.f, 0.f);
      const float th = thv[half];
      if (live[half]) {
        const float X = ((float)(i - i0) - gx) * dxf;
        const float uxs = uw[half] + ue[half];
        const float uys = vs[half] + vn[half];
        if (a.mode == 0) {
          inertia_cell_f(th, X, Y, uxs, uys, dxdy, rpm, rpim, sacc0, sacc1, sacc2);
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

// per-particle sums over chunks in a fixed order (one warp: particle n)
__device__ __forceinline__ void chunk_reduce_warp(const double *partial, const int *off, double *P, int pcap, int np,
                                                  int f0, int f1, int f2, const Bounds &bd, int n) {
  const int lane = threadIdx.x & 31;
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
// With memo set (after a sub-iteration's indicator evaluation that stored its weights in
// it), the particle's geometry words, boxes and first task are copied to the memo.
__device__ __forceinline__ void chunk_reduce_f_warp(const float *partial, const int *off, double *P, int pcap, int np,
                                                    int f0, int f1, int f2, const Bounds &bd, int n,
                                                    const WeightMemo *memo = nullptr, const float *pf = nullptr,
                                                    const int *box = nullptr) {
  const int lane = threadIdx.x & 31;
  if (n >= np) return;
  if (memo) {
    if (lane < 20) {
      const size_t q = (size_t)PF_WORDS * n + memo_word(lane);
      memo->pf[q] = pf[q];
    } else {
      const size_t q = 12 * (size_t)n + (lane - 20);
      memo->box[q] = box[q];
    }
    if (lane == 0) memo->off[n] = off[n];
    if (lane == 0 && n == 0) *memo->valid = 1;
  }
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

// ---- arguments of the box, table and task bodies from a context (host) ----

inline Bounds bounds_of(const eif_ctx *c) {
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

inline WeightMemo memo_of(const eif_ctx *c) {
  WeightMemo m;
  m.w = c->memo_w;
  m.pf = c->memo_pf;
  m.box = c->memo_box;
  m.off = c->memo_off;
  m.valid = c->memo_valid;
  return m;
}

// boxes of the particles at X (+ dX with use_increment); their task counts go to
// nchunk = chunk_off + np + 1
inline BoxArgs box_args(const eif_ctx *c, bool use_increment) {
  BoxArgs b;
  b.bd = bounds_of(c);
  b.bd_off_base = c->chunk_off;
  b.P = c->P; b.pcap = c->pcap; b.np = c->np; b.itot = c->itot; b.jtot = c->jtot;
  b.use_increment = use_increment ? 1 : 0;
  b.dx = c->dx; b.dy = c->dy; b.ly = c->ly; b.yf1 = c->h_yf[0];
  b.box = c->box;
  b.pf = c->cfg.precision == EIF_PREC_MIXED ? c->pf : nullptr;
  b.iter = nullptr;
  b.nchunk = c->chunk_off + (c->np + 1);
  return b;
}

// task evaluations of mode 0 (inertia into the integrals cn) or 1 (exchange) over the
// current velocity buffers; wmode 0, no loop counter, no counts
inline WorkArgs work_args(const eif_ctx *c, int mode, int cn) {
  WorkArgs w;
  w.P = c->P; w.ux = c->ux[c->cur]; w.uy = c->uy[c->cur]; w.xc = c->xc; w.yc = c->yc; w.dt = c->d_scal;
  w.uxf = c->uxf[c->cur]; w.uyf = c->uyf[c->cur];
  w.box = c->box; w.off = c->chunk_off; w.partial = c->partial; w.wbuf = reinterpret_cast<double2 *>(c->wbuf);
  w.pcap = c->pcap; w.np = c->np; w.ld = c->ld; w.mode = mode; w.cn = cn;
  w.dx = c->dx; w.dy = c->dy; w.ly = c->ly; w.h = c->dx < c->dy ? c->dx : c->dy;
  w.bd = bounds_of(c);
  w.pf = c->pf;
  w.tdesc = c->tdesc;
  w.coef = c->d_coef;
  w.rh_f = (float)(1. / w.h);
  w.dx_f = (float)c->dx;
  w.dy_f = (float)c->dy;
  w.dxdy_f = (float)(c->dx * c->dy);
  w.wcache = c->wcache;
  w.wmode = 0;
  w.iter = nullptr;
  w.gate = 0;
  w.weights_only = c->ibm_weights_only ? 1 : 0;
  w.count = nullptr;
  w.memo = memo_of(c);
  w.memo_mode = 0;
  w.miss = nullptr;
  w.only = nullptr;
  return w;
}

}  // namespace
