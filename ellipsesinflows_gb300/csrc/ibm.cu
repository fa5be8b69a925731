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

#include "ibm_device.cuh"

namespace {

// Stand-alone kernels over the bodies of ibm_device.cuh. Inside the sub-iteration
// loop of a step graph (iter set) the loop counter decides what runs: in the first
// sub-iteration the increments are zero, the positions are X and the boxes and the
// weights built at X before the loop are still in place.
__global__ void __launch_bounds__(32) k_boxes(BoxArgs a) {
  if (a.iter && *a.iter == 0u) return;
  box_part(a, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

__global__ void __launch_bounds__(TT_WARPS * 32) k_task_table_scan(const int *__restrict__ box, const int *__restrict__ cnt,
                                                                  int *__restrict__ off, int4 *__restrict__ tdesc, int np,
                                                                  Bounds bd, int cap, const unsigned *__restrict__ iter) {
  if (iter && *iter == 0u) return;
  task_table_block(box, cnt, off, tdesc, np, bd, cap, blockIdx.x);
}

// The double-precision body is the batch stage kernel's instantiation (ordinary loads):
// one function, compiled alike in both translation units, gives both kernels the same
// bits.
__global__ void __launch_bounds__(256) k_ibm_work(WorkArgs a) {
  // per warp: body-frame offsets of its near cells, overwritten by their weights
  __shared__ double2 slot_buf[8][CHUNK];
  const int wmode = a.iter ? (*a.iter == 0u ? 2 : 0) : a.wmode;
  ibm_work_tasks<false>(a, wmode, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, (gridDim.x * blockDim.x) >> 5,
                        slot_buf[threadIdx.x >> 5]);
}

__global__ void __launch_bounds__(256, 3) k_ibm_work_f(WorkArgs a) {
  if (a.gate && ((a.gate == 1) != (*a.iter == 0u))) return;
  __shared__ float2 slot_buf[8][CHUNK];
  ibm_work_f_tasks<true>(a, a.wmode, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, (gridDim.x * blockDim.x) >> 5,
                         slot_buf[threadIdx.x >> 5]);
}

// the stage start's evaluation at X (mixed form): memo-served tasks, the rest listed
__global__ void __launch_bounds__(256, 4) k_ibm_memo_f(WorkArgs a) {
  ibm_memo_f_tasks<true>(a, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, (gridDim.x * blockDim.x) >> 5);
}

__global__ void __launch_bounds__(256, 4) k_ibm_sum_f(WorkArgs a) {
  if (a.gate && ((a.gate == 1) != (*a.iter == 0u))) return;
  ibm_sum_f_tasks<true>(a, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, (gridDim.x * blockDim.x) >> 5);
}

__global__ void k_chunk_reduce(const double *__restrict__ partial, const int *__restrict__ off, double *__restrict__ P,
                               int pcap, int np, int f0, int f1, int f2, Bounds bd) {
  chunk_reduce_warp(partial, off, P, pcap, np, f0, f1, f2, bd, (blockIdx.x * blockDim.x + threadIdx.x) >> 5);
}

// save: after an indicator evaluation that stored its weights in the memo (with iter:
// only in the sub-iterations after the first, which evaluate the geometry)
__global__ void k_chunk_reduce_f(const float *__restrict__ partial, const int *__restrict__ off, double *__restrict__ P,
                                 int pcap, int np, int f0, int f1, int f2, Bounds bd, WeightMemo memo, int save,
                                 const unsigned *__restrict__ iter, const float *__restrict__ pf,
                                 const int *__restrict__ box) {
  const bool s = save && (!iter || *iter != 0u);
  chunk_reduce_f_warp(partial, off, P, pcap, np, f0, f1, f2, bd, (blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                      s ? &memo : nullptr, pf, box);
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
  if (c->cfg.precision == EIF_PREC_MIXED) {
    EIF_CK(c, cudaMalloc((void **)&c->memo_w, sizeof(float) * c->wcap));
    EIF_CK(c, cudaMalloc((void **)&c->memo_pf, sizeof(float) * PF_WORDS * c->np));
    EIF_CK(c, cudaMalloc((void **)&c->memo_box, sizeof(int) * 12 * c->np));
    EIF_CK(c, cudaMalloc((void **)&c->memo_off, sizeof(int) * c->np));
    EIF_CK(c, cudaMalloc((void **)&c->memo_valid, sizeof(int)));
    EIF_CK(c, cudaMemset(c->memo_valid, 0, sizeof(int)));
    EIF_CK(c, cudaMalloc((void **)&c->memo_miss, sizeof(int) * ((size_t)chunks + 1)));
  }
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
  for (void *m : {(void *)c->memo_w, (void *)c->memo_pf, (void *)c->memo_box, (void *)c->memo_off, (void *)c->memo_valid,
                  (void *)c->memo_miss})
    if (m) cudaFree(m);
  c->memo_w = nullptr; c->memo_pf = nullptr; c->memo_box = nullptr; c->memo_off = nullptr; c->memo_valid = nullptr;
  c->memo_miss = nullptr;
  c->band_lists = nullptr; c->band_counts = nullptr; c->band_marks = nullptr; c->edesc = nullptr;
  c->box = nullptr; c->chunk_off = nullptr; c->partial = nullptr; c->wbuf = nullptr; c->wcache = nullptr;
  c->weights_x_valid = false;
  c->pf = nullptr; c->tdesc = nullptr;
  c->chunk_cap = 0; c->wcap = 0;
}

static int launch_boxes(eif_ctx *c, bool use_increment) {
  // boxes at the positions X (no increment, or increments known to be zero) are
  // reused until the positions or the particle set change
  const bool x_only = !use_increment || c->incr_zero;
  if (x_only && c->boxes_x_valid) return EIF_OK;
  c->boxes_x_valid = false;
  c->weights_x_valid = false;
  c->bands_x_valid = false;
  BoxArgs b = box_args(c, use_increment);
  b.iter = c->in_loop ? reinterpret_cast<const unsigned *>(c->d_inc + 1) : nullptr;
  int *cnt = b.nchunk;
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
  WorkArgs w = work_args(c, mode, cn);
  const bool mixed = c->cfg.precision == EIF_PREC_MIXED;
  // weights at the positions X (inertia with zero increments, or the exchange)
  // are stored once and reused while the boxes at X stay valid
  const bool x_only = mode == 1 || c->incr_zero;
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
  // the weight memo (mixed form): the loop's evaluations with geometry (integrals 1)
  // store their weights in it; the first evaluation at X of a stage (integrals 0,
  // weights stored for the stage) takes them where the geometry is the memo's
  const bool memo_store = mixed && mode == 0 && cn == 1 && (c->in_loop || w.wmode == 0);
  if (mixed && mode == 0 && cn == 0 && w.wmode == 1 && c->memo_on) w.memo_mode = 1;
  {
    // launches that evaluate the indicator geometry are timed as ibm_indicator, those
    // with stored weights (sums and field contributions only) as inertia or exchange,
    // the stage start's evaluation that takes its weights from the memo as
    // ibm_stage_start
    const bool geometry = w.wmode != 2 && !(mixed && c->in_loop);
    EIF_PROF(c, w.memo_mode == 1 ? "ibm_stage_start" :
                (geometry ? "ibm_indicator" : (mode == 0 ? "ibm_inertia" : "ibm_exchange")),
             (mixed && c->in_loop) || w.memo_mode == 1 ? 2 : 1);
    if (w.memo_mode == 1) {
      // the stage start: the memo-served tasks in the light kernel (sums-kernel
      // registers), then the full evaluation of the tasks it listed as not served
      EIF_CK(c, cudaMemsetAsync(c->memo_miss, 0, sizeof(int), c->stream));
      WorkArgs wm = w, wf = w;
      wm.miss = c->memo_miss;
      wf.only = c->memo_miss;
      wf.memo_mode = 0;
      k_ibm_memo_f<<<c->sms * c->ibm_ctas_per_sm[2], 256, 0, c->stream>>>(wm);
      EIF_LAUNCH_CK(c);
      k_ibm_work_f<<<blocks, 256, 0, c->stream>>>(wf);
    } else if (mixed && c->in_loop) {
      // first sub-iteration: cached weights; later ones: full evaluation (decided on the device)
      WorkArgs w1 = w, w2 = w;
      w1.wmode = 2; w1.gate = 1;
      w2.wmode = 0; w2.gate = 2; w2.memo_mode = 2;
      k_ibm_sum_f<<<c->sms * c->ibm_ctas_per_sm[2], 256, 0, c->stream>>>(w1);
      EIF_LAUNCH_CK(c);
      k_ibm_work_f<<<blocks, 256, 0, c->stream>>>(w2);
    } else if (mixed && w.wmode == 2) {
      k_ibm_sum_f<<<c->sms * c->ibm_ctas_per_sm[2], 256, 0, c->stream>>>(w);
    } else if (mixed) {
      if (memo_store) w.memo_mode = 2;
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
  if (mixed) {
    k_chunk_reduce_f<<<(c->np * 32 + 255) / 256, 256, 0, c->stream>>>(
        reinterpret_cast<const float *>(c->partial), c->chunk_off, c->P, c->pcap, c->np, f0, f1, f2, bounds_of(c),
        memo_of(c), memo_store ? 1 : 0, c->in_loop ? w.iter : nullptr, c->pf, c->box);
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
