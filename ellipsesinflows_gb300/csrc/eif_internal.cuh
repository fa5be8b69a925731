// Internal declarations of the GB300 implementation of include/eif.h.
//
// Device data layout (one context = one suspension on one GPU):
//  * Fields keep the reference's haloed index spaces (include/arrays/fluid.h)
//    but rows are padded to a pitch `ld` (a multiple of 32 doubles, 256 B):
//      UX(i,j) -> ux[j*ld + (i-1)]      i = 1..itot+1, j = 0..jtot+1
//      UY(i,j) -> uy[j*ld + i]          i = 0..itot+1, j = 0..jtot+1 (also p, psi, dux, duy)
//    Row 0 and row jtot+1 are the periodic halo rows; wall columns hold the
//    boundary values. Every kernel that writes a field also writes the halo
//    copies and wall/Neumann values it affects, so the device state is always
//    boundary-consistent (the reference refreshes them with separate calls,
//    src/fluid/boundary_conditions.c).
//  * The explicit RK source terms use the same index spaces as the velocity
//    they belong to (SRCUXA(i,j) at ux's index, SRCUYA(i,j) at uy's index).
//  * ux/uy are double-buffered: the predictor reads one buffer and writes the
//    other, which removes the read-after-write hazard of an in-place stencil.
//  * Particles are structure-of-arrays: field f of particle n at P[f*pcap + n],
//    f in the order of the reference's particle_t (EIF_P_* in eif.h).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include "eif.h"

#define EIF_WARP 32

// error flags raised by kernels (bit mask in ctx->d_flags)
#define EIF_FLAG_NOCONV 1u
#define EIF_FLAG_NONFINITE 2u
#define EIF_FLAG_TIMEOUT 4u   // a bounded wait (an asynchronous copy, a grid barrier) gave up

// cap of the equivalent-circle fixed point (the reference has none,
// src/suspensions/collision.c:117-133,141-152)
#define EIF_FIT_MAX_ITER 10000
// cap of the normal-foot iteration (src/ellipse.c:57-59: stop after n > 100)
#define EIF_NORMAL_MAX_ITER 101

// Interior block length of the partitioned tridiagonal solver along y.
#define EIF_TDM_M 16

#include <vector>
#include <string>

// collision candidate lists: room for EIF_CAND_CAP candidates per particle (particles.cu)
#define EIF_CAND_CAP 64

namespace eif {

// per-kernel event timing of one context
struct Profiler {
  bool enabled = false;
  struct Entry { std::string name; long long launches = 0; double ms = 0.; };
  std::vector<Entry> entries;
  struct Pending { int entry; cudaEvent_t start, stop; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
};

// Poisson solver tables, built once per context on the host in double precision.
struct PoissonPlan {
  int n;            // DCT length (itot), even
  int m;            // complex FFT length n/2
  int nfac;         // radix sequence of the m-point FFT
  int fac[16];
  double2 *tw;      // exp(-2 pi i k / m), k < m
  double2 *rot;     // exp(-i pi k / 2n), k < n
  double2 *wn;      // exp(-2 pi i k / n), k < n
  float4 *tw_f, *rot_f, *wn_f;  // the same tables as float pairs (re hi, re lo, im hi, im lo)
  // single-precision tables of the refined solve (mixed form): twiddles (re, im) and
  // the block Thomas factors and left responses, [i][k] like tdm_inv, tdm_up, tdm_g
  float2 *tw2 = nullptr, *rot2 = nullptr, *wn2 = nullptr;
  float *tdm_inv_f = nullptr, *tdm_up_f = nullptr, *tdm_g_f = nullptr;
  float2 *qdf = nullptr;   // right-hand side of the first pass as (hi, lo) pairs, jtot rows of pitch ld
  // tridiagonal solver along y (jtot rows, one system per wavenumber)
  int blk;          // interior rows per block + 1 (EIF_TDM_M), or 0: serial path
  int nblk;         // blocks per column (jtot / blk)
  double *tdm_inv;  // [k][i]  1/pivot of the interior Thomas sweep, i < blk-1
  double *tdm_up;   // [k][i]  modified upper diagonal, i < blk-1
  double *tdm_g;    // [k][i]  response of the interior block to its left neighbour
  float2 *tdm_g_df = nullptr;  // the same as (hi, lo) float pairs (mixed form)
  float2 *tdm_inv_df = nullptr, *tdm_up_df = nullptr;  // tdm_inv, tdm_up as float pairs (mixed form)
  double *red_inv;  // [k][b]  reduced cyclic system: Thomas pivots (b < nblk-1)
  double *red_up;   // [k][b]
  double *red_q1;   // [k][b]  correction vector of the reduced cyclic system
  double *red_coef; // [k][4]  A, B, den, pin flag
  // second-level partition of the reduced system (g2 values per group, q2 groups; 0: not used)
  int g2 = 0, q2 = 0;
  double *r2_inv = nullptr, *r2_up = nullptr, *r2_phi = nullptr;   // [i][k], i < g2-1
  double *r2_qinv = nullptr, *r2_qup = nullptr, *r2_q1 = nullptr;  // [q][k], q < q2-1
  double *r2_coef = nullptr;                                        // [k][4] A2, B2, den2, pin flag
  double *lam;      // [k]     eigenvalue of the DCT direction
  double *ywork;    // nblk*itot: reduced right-hand sides / interface values
  float *iface_f = nullptr;  // nblk*itot: the solved interface values rounded to float (refined solve)
};

struct Adjoint;  // adjoint.cu
struct Snapshot;  // snapshot.cu
struct Stats;     // stats.cu
}  // namespace eif

struct eif_ctx {
  eif_config_t cfg;
  int itot, jtot, ld;
  size_t nfield;                // ld * (jtot+2)
  double lx, ly, dx, dy;
  int device;
  cudaStream_t stream;
  // second stream for particle-only work that runs beside the fluid kernels; the
  // launch functions use `stream`, which side_begin/side_end point at it
  cudaStream_t side = nullptr, main_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_ibm = nullptr, ev_coll = nullptr;
  // eif_advance_pull: the step graphs record ev_fields once the last RK stage's
  // projection has written the fields; their copy to the host runs on copy_stream
  cudaEvent_t ev_fields = nullptr;
  cudaStream_t copy_stream = nullptr;
  bool bands_x_valid = false;   // band lists built for the current boxes at X
  // discrete adjoint (adjoint.cu): right-hand side that replaces the divergence in the
  // double-precision Poisson solve while set; the exchange writes the summed weights
  // instead of the forcing while ibm_weights_only is set; the adjoint state
  const double *adj_rhs = nullptr;
  bool ibm_weights_only = false;
  eif::Adjoint *adj = nullptr;
  eif::Snapshot *snap = nullptr;  // asynchronous checkpoint copies (snapshot.cu)
  eif::Stats *stats = nullptr;    // time-averaged statistics (stats.cu)
  // fields
  double *ux[2], *uy[2];
  int cur;                      // index of the current velocity buffer
  double *p, *psi;
  double *sxa[2], *sya[2];      // RK explicit terms: [scur] current stage, [1-scur] previous
  int scur;
  double *dux, *duy;
  double *qhat;                 // Poisson work field (wavenumber space)
  // grid metrics (device, indexed like the reference arrays)
  double *xc;                   // XC(0..itot+1)
  double *yc;                   // YC(1..jtot) at [j]
  double *rdxf, *rdxc;          // 1/DXF(i), 1/DXC(i) at [i]
  double *cxm, *cxp, *cym, *cyp;// stencil interpolation weights at [i]
  double *dxc;                  // DXC(i) at [i]
  double *dxf = nullptr;        // DXF(i) at [i]
  float *rdxf_f, *rdxc_f, *cxm_f, *cxp_f, *cym_f, *cyp_f;  // single-precision copies
  // the single-precision x metrics when they are uniform in the interior (the mixed
  // predictor then takes them as arguments and loads only at the wall columns)
  struct UniformX {
    bool on = false;
    float rdxf = 0.f, rdxc = 0.f, cx = 0.f, cy = 0.f;
  } uni_x;
  float2 *rdxc_df = nullptr;    // 1/dxc as double-float pairs (hi, lo)
  float *sxf[2], *syf[2];       // RK explicit terms of the mixed form
  // mixed form: ux, uy rounded to float (eifd::d2f), entry by entry, the velocities the
  // single-precision immersed-boundary kernels read; written with the doubles by the
  // predictor and the projection, and refreshed whole after the boundary conditions
  float *uxf[2] = {nullptr, nullptr}, *uyf[2] = {nullptr, nullptr};
  // host copies of the metrics
  double *h_xf, *h_xc, *h_dxf, *h_dxc, *h_yf, *h_yc;
  eif::PoissonPlan pp;
  // particles
  int np, pcap;
  double *P;                    // EIF_NFIELDS * pcap
  // particle sub-iteration: [0] residual accumulator (IEEE bits), [1] loop counter (low word)
  // and block arrivals (high word); counters reported by eif_counters: [2] sub-iterations
  // run, [3] box cells whose indicator geometry was evaluated and [4] of those the near
  // cells that ran the normal-foot iteration, [5] indicator tasks whose weights came from
  // the memo ([3] to [5] while kernel timing is on; [5] by eif_memo_count)
  unsigned long long *d_inc = nullptr;
  // step graphs (eif_advance): one per parity of the double-buffer indices at the step's start
  struct StepGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int cur0 = -1, scur0 = -1, cur1 = 0, scur1 = 0;
  } graphs[2];
  bool use_graphs = true;
  // tile shapes of the stencil and block-Thomas kernels, chosen once per grid size by the
  // tuner (tune.cu) among shapes that give the same results: predictor and projection
  // tile heights (rows per block of 32 columns), threads per block of the block Thomas
  struct Tiles {
    int pred = 8, corr = 8, tdm = 128;
    bool pred_copy = true;   // mixed predictor: tiles staged by tensor copies where available
    bool tuned = false;
  } tiles;
  unsigned buf_gen = 0;         // bumped when device buffers are reallocated (batch graphs hold them)
  bool incr_zero = false;       // the particle increments are zero (after a reset)
  // a non-finite velocity was reported: the RK explicit terms kept for the next stage may
  // hold NaN (multiplied by beta = 0 in the first stage, which still gives NaN), so the
  // next fluid push clears them, as the reference's fluid_init starts them at zero
  bool src_nonfinite = false;
  // the mixed form solves the Poisson equation in single precision with one refinement
  // whose right-hand side is the residual formed in double-float arithmetic: psi is then
  // kept as the two single-precision solutions psi1, psi2 (psi = psi1 + psi2), psi1 in
  // the first nfield floats of the psi buffer and psi2 in the next nfield, both with the
  // uy layout (pitch ld, halo rows and ghost columns)
  bool psi_pair = false;
  // the mixed predictor stages its tiles with bulk tensor copies (fluid.cu): resident
  // blocks per SM of the three tile heights (0: not available, the plain kernel runs)
  int pred_tma_ctas[3] = {0, 0, 0};
  bool boxes_x_valid = false;   // the IBM boxes hold the positions X (see launch_boxes)
  bool weights_x_valid = false; // wcache holds the indicator weights of those boxes
  void *wcache = nullptr;       // indicator weight per IBM task slot (wcap entries)
  bool in_loop = false;                      // capturing the body of a sub-iteration loop
  bool reset_in_stage_kernel = false;        // batch capture: the stage kernel resets the increments
  cudaGraphConditionalHandle loop_handle = 0;
  int ibm_ctas_per_sm[3] = {0, 0, 0};  // resident CTAs per SM of the IBM work kernels (FP64, mixed, mixed cached)
  unsigned *band_marks = nullptr;  // per band of 8 rows: bitmap over the 3*np (particle, image) boxes
  // immersed-boundary work
  int *box;                     // per particle: 3 images x {imin,imax,jmin,jmax}
  int *chunk_off;               // per particle: first chunk (exclusive scan), [np] = total
  double *partial;              // per chunk: 3 partial sums
  double *wbuf;                 // per box cell: dux, duy contribution
  size_t wcap;                  // capacity of wbuf in cells
  int chunk_cap;                // capacity of partial in chunks
  float *pf;                    // per-particle single-precision parameters (mixed form)
  int4 *tdesc;                  // task table: particle, row, columns and image of every chunk
  // weights of the last indicator evaluation in a sub-iteration loop (mixed form), with
  // the particles' geometry words, boxes and first tasks (WeightMemo in ibm_device.cuh)
  // tasks of a stage start the memo did not serve: [0] count, then their numbers
  int *memo_miss = nullptr;
  float *memo_w = nullptr, *memo_pf = nullptr;
  int *memo_box = nullptr, *memo_off = nullptr, *memo_valid = nullptr;
  bool memo_on = true;          // false: EIF_NO_MEMO set, every evaluation computes
  int *band_lists, *band_counts;// ordered (particle, image) lists per band of gather rows
  int band_cap;
  int4 *edesc = nullptr;        // per (particle, image): box, row pitch and scratch offset (gather)
  // device scalars
  double *d_scal;               // [0] dt, [1] residual, [2] scratch
  float *d_coef;                // single-precision dt products: [3*rk+0..2] alpha/beta/gamma*dt, [9] 1/dt,
                                // [12+2*rk], [13+2*rk]: 1/(gamma dt) as a float pair
                                // [20+2*rk], [21+2*rk]: gamma dt as a float pair
  unsigned *d_flags;
  double *h_scal;               // pinned mirror
  unsigned *h_flags;
  int sms;
  // host bookkeeping
  int step;
  double time;
  double dt_host;
  bool fluid_pushed;
  bool sync_debug;
  unsigned long long *d_check;  // bounds-guard record: flag, tag, index, bound
  unsigned long long *h_check;  // pinned mirror
  // per-step copies of dt, the flags and the bounds record for graph steps queued one
  // ahead (eif_advance): two pinned slots and the events that mark their copies
  struct StepSlot {
    double scal[4];
    unsigned long long check[4];
    unsigned flags;
  };
  StepSlot *h_slots = nullptr;
  cudaEvent_t ev_step[2] = {nullptr, nullptr};
  eif::Profiler prof;
  char err[512];
};

namespace eif {

// ---- kernel timing: a scope records events around the launches inside it ----
struct ProfScope {
  eif_ctx *c;
  int entry;
  cudaEvent_t stop;
  ProfScope(eif_ctx *c, const char *name, int kernels);
  ~ProfScope();
};
#define EIF_PROF(c, name, kernels) eif::ProfScope eif_prof_scope_((c), (name), (kernels))
int profile_flush(eif_ctx *c);
int check_records(eif_ctx *c);
// ---- step graphs (graph.cu) ----
int step_graph_launch(eif_ctx *c);
void graphs_free(eif_ctx *c);
int capture_step(eif_ctx *c, cudaGraph_t g, int *cur1, int *scur1);
int step_capture_begin(eif_ctx *c);
void step_capture_end(eif_ctx *c, int cur0, int scur0);
int capture_step_part(eif_ctx *c, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, int part,
                      std::vector<cudaGraphNode_t> *sinks, bool particles_in_stage_kernel = false);
int capture_subiteration_loop(eif_ctx *c, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, int rk,
                              std::vector<cudaGraphNode_t> *sinks);

// ---- sub-iterations of many suspensions in one persistent kernel per stage (subiter.cu) ----
struct SubiterPlan;
constexpr size_t SUBITER_MAX = 1024;   // suspensions per stage kernel
bool subiter_joinable(const eif_ctx *c);
int subiter_plan_create(eif_ctx *const *ctx, int n, SubiterPlan **out, std::string *err);
void subiter_plan_destroy(SubiterPlan *p);
// the descriptor of suspension j (context c) in RK stage rk, from the state of c after
// the capture of that stage's front
void subiter_describe(SubiterPlan *p, int rk, int j, const eif_ctx *c);
// the plan's memset node (arrival counters; no dependences) and the kernel node of stage rk
int subiter_add_reset(SubiterPlan *p, cudaGraph_t g, cudaGraphNode_t *node, std::string *err);
int subiter_add_stage(SubiterPlan *p, int rk, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps,
                      cudaGraphNode_t *node, std::string *err);
int subiter_upload(SubiterPlan *p, std::string *err);
int rk_stage_front(eif_ctx *c, int rk);
int ibm_prepare(eif_ctx *c);
void profile_free(eif_ctx *c);

// ---- launch helpers ----
int fail(eif_ctx *c, int code, const char *fmt, ...);
int check_flags(eif_ctx *c);   // after a synchronisation: reports and clears the kernel error flags
int check_cuda(eif_ctx *c, cudaError_t e, const char *what);
#define EIF_CK(c, call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return eif::check_cuda((c), e_, #call); } while (0)
// After a launch: report launch errors; with EIF_SYNC_DEBUG set in the
// environment, also wait for the kernel and name the launch site on failure.
int launch_check(eif_ctx *c, const char *file, int line);
#define EIF_LAUNCH_CK(c) do { int r_ = eif::launch_check((c), __FILE__, __LINE__); if (r_) return r_; } while (0)

// ---- fluid (fluid.cu) ----
int launch_boundaries(eif_ctx *c);
int launch_bc_p_like(eif_ctx *c, double *a);
int launch_predictor(eif_ctx *c, int rk);
int launch_update_momentum_field(eif_ctx *c);
int launch_correct(eif_ctx *c, int rk, bool with_ibm, bool with_pressure);
int launch_update_pressure(eif_ctx *c);
int launch_decide_dt(eif_ctx *c);
int launch_divergence(eif_ctx *c, double *divmax, double *divsum);
int launch_f2d_copy(eif_ctx *c, const float *in, double *out, size_t n);
int launch_d2f_copy(eif_ctx *c, const double *in, float *out, size_t n);
// out = eifd::d2f(in) element by element (the float copies of the mixed form's velocities)
int launch_round_to_float(eif_ctx *c, const double *in, float *out, size_t n);
int launch_coef(eif_ctx *c);
// the tensor-copy predictor's launch shapes (a host query, before any graph capture)
int predictor_prepare(eif_ctx *c);

// ---- Poisson (poisson.cu) ----
int poisson_init(eif_ctx *c);
void poisson_free(eif_ctx *c);
int launch_potential(eif_ctx *c, int rk, bool with_ibm);
// psi as doubles (psi1 + psi2 when psi_pair is set) into dst (nfield doubles)
int launch_psi_to_double(eif_ctx *c, double *dst);

// ---- immersed boundary (ibm.cu) ----
size_t ibm_tasks_needed(const eif_ctx *c, const double *rec, int n);
int ibm_reserve(eif_ctx *c, size_t chunks);
void ibm_free(eif_ctx *c);
int launch_inertia(eif_ctx *c, int cn);
int launch_exchange(eif_ctx *c);
int launch_band_lists(eif_ctx *c);
// transposed box evaluation of the discrete adjoint (ibm.cu): mode 0 the inertia
// integrals at X (+ dX with use_increment), mode 1 the momentum exchange at X; bar
// holds 3 x np cotangents of the integrals (mode 0) or of the particle forces
// (mode 1); gx, gy (mode 1) the cell cotangents of the field response. Writes
// out (6 x np: cotangents of x, y, az, ux, uy, vz) and the cell cotangents of the
// face-averaged velocity into fx, fy (interior cells).
// geo: 0 evaluates the indicator geometry of every box cell, 1 evaluates and stores it
// per task slot in geom (3 doubles per slot: tanh(2D), the x and y components of the
// gradient of D), 2 reads it back (same boxes and positions)
struct AdjPass {
  int mode = 0;
  bool use_increment = false;
  const double *ux = nullptr, *uy = nullptr, *bar = nullptr, *gx = nullptr, *gy = nullptr;
  double *part = nullptr, *out = nullptr, *fx = nullptr, *fy = nullptr;
  int geo = 0;
  double *geom = nullptr;
};
size_t adj_slot_cap(const eif_ctx *c);
int launch_adj_pass(eif_ctx *c, const AdjPass &p);
// logging.c:87-172: q[0..1] x/y momentum, q[2..3] x/y kinetic energy (synchronising)
int launch_field_sums(eif_ctx *c, double *q);
// choose c->tiles by timing the candidate shapes on scratch copies of the fields
// (once per context; results are cached per grid size and precision); not during capture
int tune_tiles(eif_ctx *c);
void snapshot_free(eif_ctx *c);
void stats_free(eif_ctx *c);
int adj_chunk_cap(const eif_ctx *c);
int sub_iteration(eif_ctx *c, int rk);
bool overlap_on(const eif_ctx *c);

// ---- particles (particles.cu) ----
int launch_collision(eif_ctx *c, int cn);
int launch_reset_increments(eif_ctx *c);
int launch_increment(eif_ctx *c, int rk);
int launch_update_particles(eif_ctx *c);

// RK3 coefficients (src/param/init.c:169-191)
struct RK { double alpha, beta, gamma; };
RK rk_coef(int rk);

}  // namespace eif

// ---- device helpers shared by the kernels ----
#define EIF_HD __host__ __device__ __forceinline__

namespace eifd {

// Bounds guards: an access outside its buffer is recorded (first one wins)
// and skipped instead of performed; the host reports the record as an error at
// its next synchronisation. The immersed-boundary kernels, whose indices come
// from particle geometry, are always built with the guards (EIF_CHECK).
#ifdef EIF_CHECK
__device__ __forceinline__ bool chk(unsigned long long *rec, long long idx, long long bound, int tag) {
  if (idx >= 0 && idx < bound) return true;
  if (atomicCAS(rec, 0ull, 1ull) == 0ull) {
    rec[1] = (unsigned long long)tag;
    rec[2] = (unsigned long long)idx;
    rec[3] = (unsigned long long)bound;
  }
  return false;
}
#define EIF_CHK(rec, idx, bound, tag) eifd::chk((rec), (long long)(idx), (long long)(bound), (tag))
#else
#define EIF_CHK(rec, idx, bound, tag) true
#endif

// mass and moment of inertia of an ellipse (src/suspensions/auxiliary.c:63-75)
__device__ __forceinline__ double pmass(double den, double a, double b) { return den * (M_PI * a * b); }
__device__ __forceinline__ double pmoi(double den, double a, double b) {
  return 0.25 * pmass(den, a, b) * (a * a + b * b);
}

__device__ __forceinline__ int ux_idx(int i, int j, int ld) { return j * ld + (i - 1); }
__device__ __forceinline__ int uy_idx(int i, int j, int ld) { return j * ld + i; }

// Conversions between double and float with integer operations on the IEEE-754
// fields. On this GPU the hardware double->float conversion runs at a small
// fraction of the FP64 rate, so the mixed-precision kernels use these instead.
// d2f: exponent rebiased from 1023 to 127, mantissa cut to 23 bits and rounded
// on the first discarded bit (ties away from zero); magnitudes below the
// smallest normal float give a signed zero, above the largest float infinity.
__device__ __forceinline__ float d2f(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u, mag = hi & 0x7fffffffu;
  unsigned f = (((mag - (896u << 20)) << 3) | (lo >> 29)) + ((lo >> 28) & 1u);
  f = mag < (897u << 20) ? 0u : f;
  f = mag >= (1151u << 20) ? 0x7f800000u : f;
  return __uint_as_float(sign | f);
}

// f2d: exact for normal floats; zero and subnormal floats give a signed zero.
__device__ __forceinline__ double f2d(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned sign = u & 0x80000000u, mag = u & 0x7fffffffu;
  unsigned hi = sign | ((mag >> 3) + (896u << 20));
  unsigned lo = mag << 29;
  hi = mag < 0x00800000u ? sign : hi;
  lo = mag < 0x00800000u ? 0u : lo;
  hi = mag >= 0x7f800000u ? (sign | 0x7ff00000u | ((mag >> 3) & 0x000fffffu)) : hi;
  return __hiloint2double((int)hi, (int)lo);
}

// f2d(hi) + f2d(lo) rounded to double, the value of that FP64 addition, with integer
// operations where the exact sum lies in the binade of hi: then |lo| is a whole number
// d of double ulps at hi's exponent (lo's exponent at most 29 below hi's), the sum is
// exact, and its bit pattern is hi's plus or minus d. The other cases (and zeros,
// subnormals, infinities) take the FP64 addition.
__device__ __forceinline__ double pair_to_double(float hi, float lo) {
  const double h = f2d(hi);
  const unsigned hb = __float_as_uint(hi), lb = __float_as_uint(lo);
  const unsigned eh = (hb >> 23) & 0xffu, el = (lb >> 23) & 0xffu;
  const bool hi_normal = eh != 0u && eh != 255u;
  if (hi_normal && el == 0u) return h;   // f2d(lo) is a signed zero
  const int k = (int)eh - (int)el;
  if (hi_normal && el != 255u && k >= 0 && k <= 29) {
    const unsigned long long d = (unsigned long long)((lb & 0x007fffffu) | 0x00800000u) << (29 - k);
    const unsigned long long bits = (unsigned long long)__double_as_longlong(h);
    const unsigned long long m = bits & 0x000fffffffffffffull;
    if (((hb ^ lb) >> 31) == 0u) {
      if (m + d < (1ull << 52)) return __longlong_as_double((long long)(bits + d));
    } else if (m >= d) {
      return __longlong_as_double((long long)(bits - d));
    }
  }
  return h + f2d(lo);
}

// a double as an unevaluated sum hi + lo of two floats, split with integer
// operations only: hi keeps the leading 24 significant bits (truncated), lo is
// the remaining 29 bits rounded to a float, so hi + lo carries about 48 bits.
// Magnitudes below 2^-74 split into (x as a float, 0) precision-wise.
__device__ __forceinline__ float2 split(double x) {
  const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
  const unsigned sign = hw & 0x80000000u, mag = hw & 0x7fffffffu;
  const unsigned e = mag >> 20;                                   // biased double exponent
  unsigned hb = ((mag - (896u << 20)) << 3) | (lw >> 29);         // truncated 24-bit significand
  hb = mag < (897u << 20) ? 0u : hb;
  // remaining bits: (lw & 0x1fffffff) * 2^(e - 1075)
  const float rest = (float)(lw & 0x1fffffffu);
  const int se = (int)e - 1075 + 127;
  const float scale = se >= 1 ? __uint_as_float((unsigned)se << 23) : 0.f;
  const float lo = mag < (897u << 20) ? 0.f : rest * scale;
  return make_float2(__uint_as_float(sign | hb), sign ? -lo : lo);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace eifd
