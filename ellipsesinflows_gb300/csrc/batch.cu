// Batches of independent suspensions advanced by one CUDA graph per step.
//
// A batch groups existing contexts (any grid sizes, particle counts and both
// precisions). Its step graph holds one branch per context for the context's own
// kernels (capture_step_part in graph.cu: dt, the fronts of the three RK stages, the
// particle updates); the branches have no dependences on one another, so the kernels
// of small suspensions run side by side and fill the GPU. The particle sub-iteration
// loops of all suspensions with up to TT_MAX_NP particles run in one persistent kernel
// per stage (subiter.cu): the branches join before it and fork after it. A suspension
// with more particles keeps its own loop (a conditional node) in its branch, which then
// runs its whole step independently; so do all suspensions when the environment
// variable EIF_BATCH_SUBITER is "branches". One graph launch advances every suspension
// by one step. The kernel bodies, their order within a suspension and the data they
// touch are those of eif_advance, so every suspension gets the same bits as when
// advanced alone.
//
// The branches swap double buffers, so a batch graph is tied to the buffer indices
// of all its contexts at the start of a step; two graphs are kept (the indices
// alternate with period one or two steps). A context whose buffers are
// reallocated (a push with another particle count) makes the batch rebuild.
#include "eif_internal.cuh"
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

struct eif_batch {
  std::vector<eif_ctx *> ctx;
  struct Graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<int> cur0, scur0, cur1, scur1;
    std::vector<unsigned> gen;
    std::vector<eif::SubiterPlan *> plans;   // stage kernels of the joined suspensions
  } graphs[2];
  bool stage_kernels = true;   // joined sub-iteration loops (false: a loop per branch)
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  cudaEvent_t ev_step[2] = {nullptr, nullptr};
  // per suspension: device addresses of dt (scal), flags and bounds record, gathered
  // after every step into one packed buffer and copied to the host in one transfer
  const void **d_src = nullptr;
  unsigned long long *d_pack = nullptr, *h_pack[2] = {nullptr, nullptr};
  std::string err;
};

// words per suspension in the packed scalars: scal[4], check[4], flags
constexpr int PACK_WORDS = 9;

namespace {

__global__ void k_pack_scalars(const void *const *__restrict__ src, unsigned long long *__restrict__ pack, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long *scal = static_cast<const unsigned long long *>(src[3 * i]);
  const unsigned long long *check = static_cast<const unsigned long long *>(src[3 * i + 2]);
  const unsigned *flags = static_cast<const unsigned *>(src[3 * i + 1]);
  unsigned long long *o = pack + (size_t)PACK_WORDS * i;
  for (int k = 0; k < 4; k++) o[k] = scal[k];
  for (int k = 0; k < 4; k++) o[4 + k] = check ? check[k] : 0ull;
  o[8] = *flags;
}

int batch_fail(eif_batch *b, int code, const std::string &msg) {
  b->err = msg;
  return code;
}

void free_graph(eif_batch::Graph &g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  for (eif::SubiterPlan *p : g.plans) eif::subiter_plan_destroy(p);
  g = eif_batch::Graph{};
}

bool matches(const eif_batch *b, const eif_batch::Graph &g) {
  if (!g.exec) return false;
  for (size_t i = 0; i < b->ctx.size(); i++) {
    const eif_ctx *c = b->ctx[i];
    if (g.cur0[i] != c->cur || g.scur0[i] != c->scur || g.gen[i] != c->buf_gen) return false;
  }
  return true;
}

// Suspensions `idx` (at most one stage kernel's worth) with their sub-iteration loops
// in one kernel per stage: the branches of the stage fronts join before the stage's
// kernel, which also follows the same stage's kernel of the previous group (`prev`:
// cooperative kernels run one at a time).
int build_joined(eif_batch *b, eif_batch::Graph &g, const std::vector<size_t> &idx, std::vector<cudaGraphNode_t> &prev) {
  std::vector<eif_ctx *> cs;
  for (size_t i : idx) cs.push_back(b->ctx[i]);
  const int m = (int)cs.size();
  eif::SubiterPlan *plan = nullptr;
  std::string err;
  int rc = eif::subiter_plan_create(cs.data(), m, &plan, &err);
  if (rc) return batch_fail(b, rc, "stage kernel: " + err);
  g.plans.push_back(plan);
  cudaGraphNode_t reset = nullptr;
  if ((rc = eif::subiter_add_reset(plan, g.graph, &reset, &err))) return batch_fail(b, rc, "stage kernel: " + err);
  for (int k = 0; k < m; k++) {
    if ((rc = eif::step_capture_begin(cs[k])))
      return batch_fail(b, rc, "suspension " + std::to_string(idx[k]) + ": " + eif_last_error(cs[k]));
  }
  std::vector<std::vector<cudaGraphNode_t>> tails(m);
  std::vector<cudaGraphNode_t> kernel;
  auto restore = [&]() {
    for (int k = 0; k < m; k++) eif::step_capture_end(cs[k], g.cur0[idx[k]], g.scur0[idx[k]]);
  };
  for (int part = 0; part < 4; part++) {
    for (int k = 0; k < m; k++) {
      if ((rc = eif::capture_step_part(cs[k], g.graph, kernel, part, &tails[k], true))) {
        restore();
        return batch_fail(b, rc, "suspension " + std::to_string(idx[k]) + ": " + eif_last_error(cs[k]));
      }
    }
    if (part == 3) break;
    std::vector<cudaGraphNode_t> deps{reset};
    for (int k = 0; k < m; k++) {
      eif::subiter_describe(plan, part, k, cs[k]);
      deps.insert(deps.end(), tails[k].begin(), tails[k].end());
    }
    if (prev.size() == 3) deps.push_back(prev[part]);
    cudaGraphNode_t node = nullptr;
    if ((rc = eif::subiter_add_stage(plan, part, g.graph, deps, &node, &err))) {
      restore();
      return batch_fail(b, rc, "stage kernel: " + err);
    }
    kernel.assign(1, node);
    if (prev.size() == 3) prev[part] = node;
    else if (part == (int)prev.size()) prev.push_back(node);
  }
  for (int k = 0; k < m; k++) {
    g.cur1[idx[k]] = cs[k]->cur;
    g.scur1[idx[k]] = cs[k]->scur;
  }
  restore();
  if ((rc = eif::subiter_upload(plan, &err))) return batch_fail(b, rc, "stage kernel: " + err);
  return EIF_OK;
}

int build(eif_batch *b, eif_batch::Graph &out) {
  eif_batch::Graph g;
  cudaError_t e = cudaGraphCreate(&g.graph, 0);
  if (e != cudaSuccess) return batch_fail(b, EIF_ERR_CUDA, std::string("cudaGraphCreate: ") + cudaGetErrorString(e));
  const size_t n = b->ctx.size();
  g.cur1.assign(n, 0);
  g.scur1.assign(n, 0);
  std::vector<size_t> joined;
  for (size_t i = 0; i < n; i++) {
    eif_ctx *c = b->ctx[i];
    g.cur0.push_back(c->cur);
    g.scur0.push_back(c->scur);
    g.gen.push_back(c->buf_gen);
    if (b->stage_kernels && eif::subiter_joinable(c)) {
      joined.push_back(i);
      continue;
    }
    int cur1 = 0, scur1 = 0;
    const int rc = eif::capture_step(c, g.graph, &cur1, &scur1);
    if (rc) {
      free_graph(g);
      return batch_fail(b, rc, "suspension " + std::to_string(i) + ": " + eif_last_error(c));
    }
    g.cur1[i] = cur1;
    g.scur1[i] = scur1;
  }
  std::vector<cudaGraphNode_t> prev;
  for (size_t k0 = 0; k0 < joined.size(); k0 += eif::SUBITER_MAX) {
    const std::vector<size_t> group(joined.begin() + k0, joined.begin() + std::min(joined.size(), k0 + eif::SUBITER_MAX));
    const int rc = build_joined(b, g, group, prev);
    if (rc) {
      free_graph(g);
      return rc;
    }
  }
  e = cudaGraphInstantiate(&g.exec, g.graph, 0);
  if (e != cudaSuccess) {
    free_graph(g);
    return batch_fail(b, EIF_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  }
  free_graph(out);
  out = g;
  return EIF_OK;
}

// reads dt, the flags and the bounds record of every suspension after step s
int finish_step(eif_batch *b, int s) {
  cudaError_t e = cudaEventSynchronize(b->ev_step[s & 1]);
  if (e != cudaSuccess) return batch_fail(b, EIF_ERR_CUDA, std::string("batch step: ") + cudaGetErrorString(e));
  const unsigned long long *pk = b->h_pack[s & 1];
  int first_rc = EIF_OK;
  for (size_t i = 0; i < b->ctx.size(); i++) {
    eif_ctx *c = b->ctx[i];
    const unsigned long long *w = pk + (size_t)PACK_WORDS * i;
    std::memcpy(c->h_scal, w, sizeof(double) * 4);
    c->dt_host = c->h_scal[0];
    c->step += 1;
    c->time += c->dt_host;
    int rc = EIF_OK;
    if (w[4] != 0ull) {
      cudaStreamSynchronize(b->stream);
      cudaMemset(c->d_check, 0, sizeof(unsigned long long) * 4);
      rc = eif::fail(c, EIF_ERR_CUDA, "bounds guard %llu: index %llu outside [0, %llu)", w[5], w[6], w[7]);
    } else if (w[8] != 0ull) {
      cudaStreamSynchronize(b->stream);
      *c->h_flags = (unsigned)w[8];
      rc = eif::check_flags(c);
    }
    if (rc && first_rc == EIF_OK) {
      first_rc = batch_fail(b, rc, "suspension " + std::to_string(i) + ": " + eif_last_error(c));
    }
  }
  return first_rc;
}

}  // namespace

extern "C" {

int eif_batch_create(eif_ctx *const *ctxs, int n, eif_batch **out) {
  if (!ctxs || n <= 0 || !out) return EIF_ERR_ARG;
  for (int i = 0; i < n; i++) {
    if (!ctxs[i]) return EIF_ERR_ARG;
    if (ctxs[i]->device != ctxs[0]->device) return EIF_ERR_ARG;
    for (int k = 0; k < i; k++)
      if (ctxs[k] == ctxs[i]) return EIF_ERR_ARG;
  }
  eif_batch *b = new (std::nothrow) eif_batch;
  if (!b) return EIF_ERR_NOMEM;
  b->ctx.assign(ctxs, ctxs + n);
  const char *mode = std::getenv("EIF_BATCH_SUBITER");
  b->stage_kernels = !(mode && std::strcmp(mode, "branches") == 0);
  std::vector<const void *> src;
  for (int i = 0; i < n; i++) {
    src.push_back(ctxs[i]->d_scal);
    src.push_back(ctxs[i]->d_flags);
    src.push_back(ctxs[i]->d_check);
  }
  bool ok = cudaSetDevice(ctxs[0]->device) == cudaSuccess &&
            cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->ev_step[0], cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->ev_step[1], cudaEventDisableTiming) == cudaSuccess &&
            cudaMalloc((void **)&b->d_src, sizeof(void *) * src.size()) == cudaSuccess &&
            cudaMemcpy(b->d_src, src.data(), sizeof(void *) * src.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMalloc((void **)&b->d_pack, sizeof(unsigned long long) * PACK_WORDS * n) == cudaSuccess &&
            cudaMallocHost((void **)&b->h_pack[0], sizeof(unsigned long long) * PACK_WORDS * n) == cudaSuccess &&
            cudaMallocHost((void **)&b->h_pack[1], sizeof(unsigned long long) * PACK_WORDS * n) == cudaSuccess;
  if (!ok) {
    eif_batch_destroy(b);
    return EIF_ERR_CUDA;
  }
  // tile shapes of every suspension before the step graphs capture their launches
  for (int i = 0; i < n; i++) {
    if (ctxs[i]->fluid_pushed && eif::tune_tiles(ctxs[i]) != EIF_OK) {
      eif_batch_destroy(b);
      return EIF_ERR_CUDA;
    }
  }
  *out = b;
  return EIF_OK;
}

int eif_batch_destroy(eif_batch *b) {
  if (!b) return EIF_ERR_ARG;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto &g : b->graphs) free_graph(g);
  if (b->ev) cudaEventDestroy(b->ev);
  for (auto &e : b->ev_step)
    if (e) cudaEventDestroy(e);
  if (b->d_src) cudaFree(b->d_src);
  if (b->d_pack) cudaFree(b->d_pack);
  for (auto &h : b->h_pack)
    if (h) cudaFreeHost(h);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return EIF_OK;
}

const char *eif_batch_last_error(const eif_batch *b) { return b ? b->err.c_str() : "null batch"; }

int eif_batch_size(const eif_batch *b) { return b ? (int)b->ctx.size() : 0; }

void *eif_batch_stream(eif_batch *b) { return b ? (void *)b->stream : nullptr; }

int eif_batch_advance(eif_batch *b, int nsteps) {
  if (!b || nsteps < 0) return EIF_ERR_ARG;
  for (size_t i = 0; i < b->ctx.size(); i++) {
    eif_ctx *c = b->ctx[i];
    if (!c->fluid_pushed) return batch_fail(b, EIF_ERR_STATE, "suspension " + std::to_string(i) + ": push the fluid state first");
  }
  if (cudaSetDevice(b->ctx[0]->device) != cudaSuccess) return batch_fail(b, EIF_ERR_CUDA, "cudaSetDevice");
  // steps are queued one ahead of the host's read of the previous step's scalars
  for (int s = 0; s < nsteps; s++) {
    eif_batch::Graph *g = nullptr;
    for (auto &cand : b->graphs)
      if (matches(b, cand)) g = &cand;
    if (!g) {
      // a rebuild captures every suspension again: let the queued step finish first
      cudaError_t e = cudaStreamSynchronize(b->stream);
      if (e != cudaSuccess) return batch_fail(b, EIF_ERR_CUDA, std::string("batch step: ") + cudaGetErrorString(e));
      eif_batch::Graph *slot = !b->graphs[0].exec ? &b->graphs[0] : (!b->graphs[1].exec ? &b->graphs[1] : &b->graphs[0]);
      if (b->graphs[0].exec && b->graphs[1].exec) {
        free_graph(b->graphs[0]);
        free_graph(b->graphs[1]);
      }
      const int rc = build(b, *slot);
      if (rc) return rc;
      g = slot;
    }
    // the step follows whatever the suspensions' own streams hold (pushes, stage calls)
    for (eif_ctx *c : b->ctx) {
      if (cudaEventRecord(b->ev, c->stream) != cudaSuccess || cudaStreamWaitEvent(b->stream, b->ev, 0) != cudaSuccess)
        return batch_fail(b, EIF_ERR_CUDA, "ordering after the suspensions' streams");
    }
    cudaError_t e = cudaGraphLaunch(g->exec, b->stream);
    if (e != cudaSuccess) return batch_fail(b, EIF_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
    for (size_t i = 0; i < b->ctx.size(); i++) {
      b->ctx[i]->cur = g->cur1[i];
      b->ctx[i]->scur = g->scur1[i];
    }
    const int n = (int)b->ctx.size();
    k_pack_scalars<<<(n + 63) / 64, 64, 0, b->stream>>>(b->d_src, b->d_pack, n);
    e = cudaMemcpyAsync(b->h_pack[s & 1], b->d_pack, sizeof(unsigned long long) * PACK_WORDS * n,
                        cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev_step[s & 1], b->stream);
    if (e != cudaSuccess) return batch_fail(b, EIF_ERR_CUDA, std::string("batch scalars: ") + cudaGetErrorString(e));
    if (s > 0) {
      const int rc = finish_step(b, s - 1);
      if (rc) return rc;
    }
  }
  if (nsteps > 0) {
    const int rc = finish_step(b, nsteps - 1);
    if (rc) return rc;
  }
  const cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return batch_fail(b, EIF_ERR_CUDA, std::string("batch step: ") + cudaGetErrorString(e));
  return EIF_OK;
}

}  // extern "C"
