// Sub-iterations of the particles (src/main.c:36-50) of many suspensions in one
// persistent kernel per RK stage.
//
// A batch (batch.cu) captures each suspension's stage front as a graph branch; the
// branches join before one cooperative kernel that runs the sub-iteration loops of all
// joined suspensions, and fork again after it for the particle updates and the next
// stage. The kernel's CTAs (all resident: a cooperative launch of as many CTAs as fit
// on the GPU at once) loop over the sub-iterations; a sub-iteration has four phases
// separated by grid barriers:
//   1. the collision forces at X + dX (block units of PAIR_WARPS particles) and, after
//      the first sub-iteration, the boxes at X + dX (warp units: 32 particles, one
//      part); in the first one the increments are zero and the boxes and weights that
//      the stage front built at X are still in place;
//   2. (after the first) the task tables (block units of TT_WARPS particles);
//   3. the row tasks of the inertia integrals of all suspensions in one index space (a
//      warp per task; cached weights in the first sub-iteration); the task counts are
//      zeroed for the next boxes;
//   4. per particle (a warp) the sum over its tasks, then its increment and the
//      suspension's residual (an integer max of the IEEE bits, independent of order).
// After phase 4 every CTA evaluates the stopping rule of each suspension (main.c:40-48:
// go on while the residual is not below 1e-8 and at most 101 sub-iterations ran) from
// the same residuals, so all CTAs agree on the set still iterating; a suspension that
// stops takes no part in later sub-iterations. Every body is the one of the stand-alone
// kernels (ibm_device.cuh, particle_device.cuh) with the same decomposition per task,
// particle and block, so each suspension gets the same bits as in its own loop.
// When no suspension iterates any more, the kernel updates every suspension's particles
// (update.c) and, before stages 1 and 2, resets their increments (reset.c): the particle
// launches around the loop, which the suspensions' own branches then leave out.
//
// The units of a phase are numbered suspension by suspension (fixed offsets from the
// particle counts) and worker w (a CTA or a warp) takes units w, w + W, ... of that
// numbering; the row tasks are numbered on the device from the task counts of phase 2.
//
// The grid barrier is an arrival counter per stage, zeroed by a memset node at the
// start of every step and polled with acquire loads. A poll gives up after 2^22 tries:
// the CTA sets the plan's error word, which makes the others give up at their next
// poll, and every suspension's EIF_FLAG_TIMEOUT, and the CTAs return. Data that one
// phase writes and a later one reads is read with ordinary loads, not through the
// read-only path. For the tests of that bounded wait, EIF_TEST_HOLD_BARRIER=1 in the
// environment when a batch's graph is built keeps CTA 0 of the first stage's kernel
// from arriving at its first barrier: the other CTAs give up, and the step reports it.
#ifndef EIF_CHECK
#define EIF_CHECK 1
#endif
#include "eif_internal.cuh"
#include "ibm_device.cuh"
#include "particle_device.cuh"
#include <algorithm>
#include <cstdlib>

namespace {

// one suspension's sub-iteration loop in one RK stage
struct SubDesc {
  BoxArgs box;     // boxes at X + dX
  WorkArgs work;   // inertia integrals at X + dX (mode 0, integrals 1)
  double *P;
  int pcap, np, tcap, mixed;
  int *cnt, *off;
  int4 *tdesc;
  double ly, lx, gamma, Fr2;
  double *scal;                  // [0] dt, [1] residual
  unsigned *flags, *counter;     // error flags, the stage's sub-iteration count
  unsigned long long *total;     // sub-iterations run (eif_counters)
  int u_box, u_coll, u_tab, u_part;   // first unit of the suspension in phases 1 (boxes, collisions), 2, 4
};

struct StageArgs {
  const SubDesc *d;
  int n;
  int reset_next;               // the particles' increments are reset for a following stage
  int hold;                     // a CTA that does not arrive at the first barrier (tests), or -1
  unsigned *sync;               // [0] arrivals, [1] error
  unsigned long long *res;      // two residual words per suspension (alternating sub-iterations)
};

constexpr int SUB_THREADS = 256;
constexpr int SUB_WARPS = SUB_THREADS / 32;
constexpr int SUB_MAX = (int)eif::SUBITER_MAX;
constexpr unsigned SUB_CAP = 102;      // the stopping rule ends every loop by the 102nd sub-iteration
constexpr unsigned SPIN_MAX = 1u << 22;
constexpr int SYNC_WORDS = 32;         // per stage (arrivals and error word, padded)
static_assert(PAIR_WARPS == SUB_WARPS && TT_WARPS == SUB_WARPS, "block units of the phases");

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// grid barrier number idx (0, 1, ...) of this launch; false when it gave up. arrive:
// the CTA counts itself (false only for the tests of the bounded wait)
__device__ bool grid_barrier(unsigned *sync, unsigned idx, bool arrive) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned target = gridDim.x * (idx + 1u);
    __threadfence();
    if (arrive) atomicAdd(sync, 1u);
    int good = 0;
    for (unsigned k = 0; k < SPIN_MAX; k++) {
      if (ld_acquire(sync) >= target) {
        good = 1;
        break;
      }
      if (ld_acquire(sync + 1) != 0u) break;
      __nanosleep(64);
    }
    if (!good) atomicOr(sync + 1, 1u);
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// the first of the units u = 0, 1, ... that worker w of W takes when the units are
// numbered from `base`
__device__ __forceinline__ int first_unit(int w, int base, int W) {
  const int r = (w - base) % W;
  return r < 0 ? r + W : r;
}

// per suspension, in shared memory: the loop control of the phases, so that a worker
// walks the suspensions without loading their descriptors
enum { ST_NP, ST_UBOX, ST_UCOLL, ST_UTAB, ST_UPART, ST_MIXED, ST_TASKS, ST_WORDS = 8 };

__global__ void __launch_bounds__(SUB_THREADS, 2) k_subiterations(StageArgs s) {
  __shared__ unsigned act[SUB_MAX / 32];   // suspensions still iterating
  __shared__ float2 slot_f[SUB_WARPS][CHUNK];
  __shared__ double2 slot_d[SUB_WARPS][CHUNK];
  extern __shared__ int stab[];            // ST_WORDS per suspension
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int G = gridDim.x, W = G * SUB_WARPS, T = G * SUB_THREADS;
  const int wid = blockIdx.x * SUB_WARPS + wl, tid = blockIdx.x * SUB_THREADS + threadIdx.x;
  const int n = s.n;
  for (int q = threadIdx.x; q < SUB_MAX / 32; q += SUB_THREADS) {
    const int lo = 32 * q;
    act[q] = lo >= n ? 0u : (n - lo >= 32 ? 0xffffffffu : ((1u << (n - lo)) - 1u));
  }
  for (int j = threadIdx.x; j < n; j += SUB_THREADS) {
    const SubDesc &d = s.d[j];
    int *e = stab + ST_WORDS * j;
    e[ST_NP] = d.np;
    e[ST_UBOX] = d.u_box;
    e[ST_UCOLL] = d.u_coll;
    e[ST_UTAB] = d.u_tab;
    e[ST_UPART] = d.u_part;
    e[ST_MIXED] = d.mixed;
    e[ST_TASKS] = 0;
  }
  if (blockIdx.x == 0)
    for (int j = threadIdx.x; j < 2 * n; j += SUB_THREADS) s.res[j] = 0ull;
  __syncthreads();
  auto active = [&](int j) { return ((act[j >> 5] >> (j & 31)) & 1u) != 0u; };
  unsigned bar = 0;
  bool ok = true;
  auto barrier = [&]() {
    const bool arrive = bar != 0u || (int)blockIdx.x != s.hold;
    return grid_barrier(s.sync, bar++, arrive);
  };
  for (unsigned it = 0; it < SUB_CAP; it++) {
    // 1. collision forces; boxes after the first sub-iteration
    for (int j = 0; j < n; j++) {
      if (!active(j)) continue;
      const int *e = stab + ST_WORDS * j;
      const int units = (e[ST_NP] + PAIR_WARPS - 1) / PAIR_WARPS;
      int b = first_unit(blockIdx.x, e[ST_UCOLL], G);
      if (b >= units) continue;
      const SubDesc &d = s.d[j];
      for (; b < units; b += G) {
        collision_block(d.P, d.pcap, d.np, 1, d.ly, d.lx, d.flags, b);
        __syncthreads();
      }
    }
    if (it > 0) {
      for (int j = 0; j < n; j++) {
        if (!active(j)) continue;
        const int *e = stab + ST_WORDS * j;
        const int groups = (e[ST_NP] + 31) / 32;
        const int units = groups * (e[ST_MIXED] ? BOX_PARTS : 3);
        int u = first_unit(wid, e[ST_UBOX], W);
        if (u >= units) continue;
        const SubDesc &d = s.d[j];
        for (; u < units; u += W) box_part(d.box, (u % groups) * 32 + lane, u / groups);
      }
      if (!(ok = barrier())) break;
      // 2. task tables
      for (int j = 0; j < n; j++) {
        if (!active(j)) continue;
        const int *e = stab + ST_WORDS * j;
        const int units = (e[ST_NP] + TT_WARPS - 1) / TT_WARPS;
        int b = first_unit(blockIdx.x, e[ST_UTAB], G);
        if (b >= units) continue;
        const SubDesc &d = s.d[j];
        for (; b < units; b += G) {
          task_table_block(d.box.box, d.cnt, d.off, d.tdesc, d.np, d.box.bd, d.tcap, b);
          __syncthreads();
        }
      }
    }
    if (!(ok = barrier())) break;
    // 3. row tasks of the inertia integrals; task counts zeroed for the next boxes. The
    // task totals of phase 2 are read into shared memory first, one load per suspension.
    for (int j = threadIdx.x; j < n; j += SUB_THREADS) {
      int *e = stab + ST_WORDS * j;
      e[ST_TASKS] = active(j) && e[ST_NP] > 0 ? s.d[j].off[e[ST_NP]] : 0;
    }
    __syncthreads();
    int base = 0;
    for (int j = 0; j < n; j++) {
      if (!active(j)) continue;
      const int *e = stab + ST_WORDS * j;
      const int np = e[ST_NP], total = e[ST_TASKS];
      if (np == 0) continue;
      const int first = first_unit(wid, base, W);
      base += total;
      const bool zero_cnt = blockIdx.x * SUB_THREADS < np;
      if (first >= total && !zero_cnt) continue;
      const SubDesc &d = s.d[j];
      if (first < total) {
        if (e[ST_MIXED]) {
          if (it == 0) ibm_sum_f_tasks<false>(d.work, first, W);
          else ibm_work_f_tasks<false>(d.work, 0, first, W, slot_f[wl]);
        } else {
          ibm_work_tasks<false>(d.work, it == 0 ? 2 : 0, first, W, slot_d[wl]);
        }
      }
      for (int q = tid; q < np; q += T) d.cnt[q] = 0;
    }
    if (!(ok = barrier())) break;
    // 4. sums over the tasks, increments, residuals
    for (int j = 0; j < n; j++) {
      if (!active(j)) continue;
      const int *e = stab + ST_WORDS * j;
      int m = first_unit(wid, e[ST_UPART], W);
      if (m >= e[ST_NP]) continue;
      const SubDesc &d = s.d[j];
      const double dt = d.scal[0];
      unsigned long long *res = s.res + 2 * j + (it & 1u);
      for (; m < d.np; m += W) {
        if (d.mixed) {
          // after a sub-iteration with the indicator geometry: its weights are in the memo
          chunk_reduce_f_warp(reinterpret_cast<const float *>(d.work.partial), d.off, d.P, d.pcap, d.np,
                              EIF_P_IUX0 + 1, EIF_P_IUY0 + 1, EIF_P_IVZ0 + 1, d.box.bd, m,
                              it > 0 && d.work.memo_mode == 2 ? &d.work.memo : nullptr, d.work.pf, d.box.box);
        } else {
          chunk_reduce_warp(d.work.partial, d.off, d.P, d.pcap, d.np, EIF_P_IUX0 + 1, EIF_P_IUY0 + 1,
                            EIF_P_IVZ0 + 1, d.box.bd, m);
        }
        if (lane == 0) {
          const double r = increment_particle(d.P, d.pcap, m, d.gamma, d.Fr2, dt, 0.);
          if (r > 0.) atomicMax(res, (unsigned long long)__double_as_longlong(r));
        }
      }
    }
    if (!(ok = barrier())) break;
    // the stopping rule of every suspension, evaluated alike by all CTAs
    for (int j = threadIdx.x; j < n; j += SUB_THREADS) {
      if (!active(j)) continue;
      const double r = __longlong_as_double(
          (long long)*reinterpret_cast<volatile unsigned long long *>(s.res + 2 * j + (it & 1u)));
      const unsigned count = it + 1u;
      if (!(!(r < 1.e-8) && count <= 101u)) atomicAnd(&act[j >> 5], ~(1u << (j & 31)));
      if (blockIdx.x == 0) {
        const SubDesc &d = s.d[j];
        d.scal[1] = r;
        *d.counter = count;
        *d.total += 1ull;
        s.res[2 * j + ((it + 1u) & 1u)] = 0ull;
      }
    }
    __syncthreads();
    bool any = false;
    for (int q = 0; q < SUB_MAX / 32; q++) any |= act[q] != 0u;
    if (!any) break;
  }
  if (!ok) {
    if (threadIdx.x == 0)
      for (int j = 0; j < n; j++) atomicOr(s.d[j].flags, EIF_FLAG_TIMEOUT);
    return;
  }
  // the particle update of the stage (update.c:8-34) and, before a following stage, the
  // reset of the increments (reset.c:7-18); the last increments were written before the
  // last grid barrier
  for (int j = 0; j < n; j++) {
    const int *e = stab + ST_WORDS * j;
    int m = first_unit(tid, e[ST_UPART], T);
    if (m >= e[ST_NP]) continue;
    const SubDesc &d = s.d[j];
    for (; m < d.np; m += T) {
      update_particle(d.P, d.pcap, m, d.ly);
      if (s.reset_next) reset_particle(d.P, d.pcap, m);
    }
  }
}

}  // namespace

namespace eif {

struct SubiterPlan {
  int n = 0, grid = 0;
  std::vector<SubDesc> h;               // 3 stages x n
  SubDesc *d_desc = nullptr;
  unsigned *d_sync = nullptr;           // 3 stages x SYNC_WORDS
  unsigned long long *d_res = nullptr;  // 3 stages x 2n
  int hold = -1;                        // EIF_TEST_HOLD_BARRIER: CTA 0 of stage 0 held back
};

bool subiter_joinable(const eif_ctx *c) { return c->np <= TT_MAX_NP; }

void subiter_plan_destroy(SubiterPlan *p) {
  if (!p) return;
  if (p->d_desc) cudaFree(p->d_desc);
  if (p->d_sync) cudaFree(p->d_sync);
  if (p->d_res) cudaFree(p->d_res);
  delete p;
}

static int plan_fail(std::string *err, const char *what, cudaError_t e) {
  *err = std::string(what) + ": " + cudaGetErrorString(e);
  return EIF_ERR_CUDA;
}

int subiter_plan_create(eif_ctx *const *ctx, int n, SubiterPlan **out, std::string *err) {
  *out = nullptr;
  if (n <= 0 || n > SUB_MAX) {
    *err = "a stage kernel takes 1 to " + std::to_string(SUB_MAX) + " suspensions";
    return EIF_ERR_ARG;
  }
  int coop = 0, occ = 0;
  cudaError_t e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx[0]->device);
  if (e != cudaSuccess) return plan_fail(err, "cudaDeviceGetAttribute", e);
  if (!coop) {
    *err = "the device has no cooperative launch";
    return EIF_ERR_CUDA;
  }
  // the loop-control table in dynamic shared memory: ST_WORDS ints per suspension
  e = cudaFuncSetAttribute(k_subiterations, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(sizeof(int) * ST_WORDS * SUB_MAX));
  if (e != cudaSuccess) return plan_fail(err, "cudaFuncSetAttribute", e);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_subiterations, SUB_THREADS, sizeof(int) * ST_WORDS * n);
  if (e != cudaSuccess) return plan_fail(err, "cudaOccupancyMaxActiveBlocksPerMultiprocessor", e);
  if (occ < 1) {
    *err = "the stage kernel does not fit on an SM";
    return EIF_ERR_CUDA;
  }
  SubiterPlan *p = new (std::nothrow) SubiterPlan;
  if (!p) return EIF_ERR_NOMEM;
  p->n = n;
  p->grid = occ * ctx[0]->sms;
  const char *hold = std::getenv("EIF_TEST_HOLD_BARRIER");
  p->hold = hold && hold[0] == '1' ? 0 : -1;
  p->h.assign((size_t)3 * n, SubDesc{});
  if ((e = cudaMalloc((void **)&p->d_desc, sizeof(SubDesc) * 3 * n)) != cudaSuccess ||
      (e = cudaMalloc((void **)&p->d_sync, sizeof(unsigned) * 3 * SYNC_WORDS)) != cudaSuccess ||
      (e = cudaMalloc((void **)&p->d_res, sizeof(unsigned long long) * 3 * 2 * n)) != cudaSuccess) {
    subiter_plan_destroy(p);
    return plan_fail(err, "cudaMalloc", e);
  }
  *out = p;
  return EIF_OK;
}

void subiter_describe(SubiterPlan *p, int rk, int j, const eif_ctx *c) {
  SubDesc &d = p->h[(size_t)rk * p->n + j];
  d.box = box_args(c, true);
  d.work = work_args(c, 0, 1);
  // the evaluations with geometry (sub-iterations after the first) store their weights
  if (c->cfg.precision == EIF_PREC_MIXED) d.work.memo_mode = 2;
  d.P = c->P;
  d.pcap = c->pcap;
  d.np = c->np;
  d.tcap = c->chunk_cap;
  d.mixed = c->cfg.precision == EIF_PREC_MIXED ? 1 : 0;
  d.cnt = c->np > 0 ? c->chunk_off + (c->np + 1) : nullptr;
  d.off = c->chunk_off;
  d.tdesc = c->tdesc;
  d.ly = c->ly;
  d.lx = c->lx;
  d.gamma = rk_coef(rk).gamma;
  d.Fr2 = c->cfg.Fr * c->cfg.Fr;
  d.scal = c->d_scal;
  d.flags = c->d_flags;
  d.counter = reinterpret_cast<unsigned *>(c->d_inc + 1);
  d.total = c->d_inc + 2;
}

int subiter_add_reset(SubiterPlan *p, cudaGraph_t g, cudaGraphNode_t *node, std::string *err) {
  cudaMemsetParams m = {};
  m.dst = p->d_sync;
  m.value = 0;
  m.elementSize = sizeof(unsigned);
  m.width = 3 * SYNC_WORDS;
  m.height = 1;
  const cudaError_t e = cudaGraphAddMemsetNode(node, g, nullptr, 0, &m);
  return e == cudaSuccess ? EIF_OK : plan_fail(err, "cudaGraphAddMemsetNode", e);
}

int subiter_add_stage(SubiterPlan *p, int rk, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps,
                      cudaGraphNode_t *node, std::string *err) {
  StageArgs a;
  a.d = p->d_desc + (size_t)rk * p->n;
  a.n = p->n;
  a.sync = p->d_sync + SYNC_WORDS * rk;
  a.res = p->d_res + (size_t)2 * p->n * rk;
  a.reset_next = rk < 2 ? 1 : 0;
  a.hold = rk == 0 ? p->hold : -1;
  void *args[] = {&a};
  cudaKernelNodeParams k = {};
  k.func = reinterpret_cast<void *>(k_subiterations);
  k.gridDim = dim3(p->grid);
  k.blockDim = dim3(SUB_THREADS);
  k.sharedMemBytes = (unsigned)(sizeof(int) * ST_WORDS * p->n);
  k.kernelParams = args;
  cudaError_t e = cudaGraphAddKernelNode(node, g, deps.data(), deps.size(), &k);
  if (e != cudaSuccess) return plan_fail(err, "cudaGraphAddKernelNode", e);
  cudaKernelNodeAttrValue v = {};
  v.cooperative = 1;
  e = cudaGraphKernelNodeSetAttribute(*node, cudaKernelNodeAttributeCooperative, &v);
  return e == cudaSuccess ? EIF_OK : plan_fail(err, "cudaGraphKernelNodeSetAttribute (cooperative)", e);
}

int subiter_upload(SubiterPlan *p, std::string *err) {
  for (int rk = 0; rk < 3; rk++) {
    int u_box = 0, u_coll = 0, u_tab = 0, u_part = 0;
    for (int j = 0; j < p->n; j++) {
      SubDesc &d = p->h[(size_t)rk * p->n + j];
      d.u_box = u_box;
      d.u_coll = u_coll;
      d.u_tab = u_tab;
      d.u_part = u_part;
      u_box += ((d.np + 31) / 32) * (d.mixed ? BOX_PARTS : 3);
      u_coll += (d.np + PAIR_WARPS - 1) / PAIR_WARPS;
      u_tab += (d.np + TT_WARPS - 1) / TT_WARPS;
      u_part += d.np;
    }
  }
  const cudaError_t e = cudaMemcpy(p->d_desc, p->h.data(), sizeof(SubDesc) * p->h.size(), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? EIF_OK : plan_fail(err, "cudaMemcpy (stage descriptors)", e);
}

}  // namespace eif
