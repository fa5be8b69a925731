// Step graphs: one time step of eif_advance as a single CUDA graph.
//
// The graph holds, in launch order, the dt decision and for each RK stage the
// stage kernels, a conditional WHILE node whose body is one particle
// sub-iteration (inertia at the increment, collisions, increments), and the
// particle update (src/main.c:13-53). Work that the stage driver puts on the side
// stream is captured as a parallel branch of the same graph. The last block of
// k_increment sets the loop condition on the device from the residual and the
// sub-iteration count, so a step needs
// no host round trip; the host synchronises once per step to read dt and the
// error flags. The kernels and their order are those of the host-driven path
// (rk_stage), so both paths give bit-identical results.
//
// The stage kernels swap the double-buffered velocity and source arrays, so the
// buffers a step touches depend on the buffer indices at its start; one graph
// is kept per starting pair of indices (at most two occur). Graphs are rebuilt
// after the particle buffers are reallocated.
#include "eif_internal.cuh"
#include <vector>

namespace eif {

namespace {

int end_capture(eif_ctx *c, std::vector<cudaGraphNode_t> *sinks) {
  if (sinks) {
    cudaStreamCaptureStatus st;
    const cudaGraphNode_t *deps = nullptr;
    size_t n = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(c->stream, &st, nullptr, nullptr, &deps, nullptr, &n);
    if (e == cudaSuccess) sinks->assign(deps, deps + n);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) return check_cuda(c, e, "cudaStreamGetCaptureInfo");
    if (e2 != cudaSuccess) return check_cuda(c, e2, "cudaStreamEndCapture");
    return EIF_OK;
  }
  cudaGraph_t g = nullptr;
  EIF_CK(c, cudaStreamEndCapture(c->stream, &g));
  return EIF_OK;
}

// abandon a capture after an error, leaving the streams usable
void abort_capture(eif_ctx *c) {
  for (cudaStream_t s : {c->stream, c->side}) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (s && cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
    }
  }
  cudaGetLastError();
  c->in_loop = false;
}

}  // namespace

// Host state of c before the capture of a step: the graph must not depend on boxes
// computed before it, so it starts without them.
int step_capture_begin(eif_ctx *c) {
  int rc = ibm_prepare(c);
  if (rc) return rc;
  c->boxes_x_valid = false;
  c->weights_x_valid = false;
  c->incr_zero = false;
  return EIF_OK;
}

// Host state of c after the capture of a step (or after a failed capture): nothing
// has run yet, so the step starts from the buffers (cur0, scur0); the step ends with
// new positions, so no boxes are valid after it.
void step_capture_end(eif_ctx *c, int cur0, int scur0) {
  abort_capture(c);
  c->cur = cur0;
  c->scur = scur0;
  c->boxes_x_valid = false;
  c->weights_x_valid = false;
}

// Captures part `part` of one time step of c into g after the nodes deps (none: an
// independent branch) and returns its last nodes in sinks. Part 0 is the dt decision
// and the front of RK stage 0 (src/main.c:14-35), parts 1 and 2 the particle update
// of the stage before (main.c:51-53) and the front of the next stage, part 3 the
// particle update of stage 2. The sub-iteration loops (main.c:36-50) go between the
// parts: a conditional node per context (capture_subiteration_loop), or one kernel for
// all the suspensions of a batch, which then also updates the particles at the end of the
// stage and resets the increments for the next (particles_in_stage_kernel: those launches
// are left out of parts 1-3).
int capture_step_part(eif_ctx *c, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, int part,
                      std::vector<cudaGraphNode_t> *sinks, bool particles_in_stage_kernel) {
  cudaError_t e = cudaStreamBeginCaptureToGraph(c->stream, g, deps.data(), nullptr, deps.size(),
                                                cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return check_cuda(c, e, "cudaStreamBeginCaptureToGraph");
  int rc;
  if (part == 0) {
    if ((rc = launch_decide_dt(c))) return rc;
  } else {
    // after a sub-iteration loop: the increments are not zero and the boxes of the
    // loop's last positions are not those at X
    c->incr_zero = false;
    c->boxes_x_valid = false;
    c->weights_x_valid = false;
    c->bands_x_valid = false;
    if (!particles_in_stage_kernel && (rc = launch_update_particles(c))) return rc;
  }
  if (part < 3) {
    c->reset_in_stage_kernel = particles_in_stage_kernel && part > 0;
    rc = rk_stage_front(c, part);
    c->reset_in_stage_kernel = false;
    if (rc) return rc;
  }
  if (part == 2 && !particles_in_stage_kernel && c->ev_fields) {
    // the last stage's projection is done: the fields are final for this step
    // (eif_advance_pull copies them to the host beside the particle work that follows)
    const cudaError_t e = cudaEventRecordWithFlags(c->ev_fields, c->stream, cudaEventRecordExternal);
    if (e != cudaSuccess) return check_cuda(c, e, "cudaEventRecordWithFlags (fields)");
  }
  return end_capture(c, sinks);
}

// The sub-iteration loop of RK stage rk of c as a conditional WHILE node after the
// nodes deps (its counter reset before it); sinks = {the loop node}. The last block
// of k_increment sets the loop condition on the device.
int capture_subiteration_loop(eif_ctx *c, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, int rk,
                              std::vector<cudaGraphNode_t> *sinks) {
  std::vector<cudaGraphNode_t> tail;
  cudaError_t e = cudaStreamBeginCaptureToGraph(c->stream, g, deps.data(), nullptr, deps.size(),
                                                cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return check_cuda(c, e, "cudaStreamBeginCaptureToGraph");
  // the sub-iteration counter starts at zero for every stage
  e = cudaMemsetAsync(reinterpret_cast<unsigned *>(c->d_inc + 1), 0, sizeof(unsigned), c->stream);
  if (e != cudaSuccess) return check_cuda(c, e, "cudaMemsetAsync");
  int rc = end_capture(c, &tail);
  if (rc) return rc;
  cudaGraphConditionalHandle h;
  e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return check_cuda(c, e, "cudaGraphConditionalHandleCreate");
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t loop = nullptr;
  e = cudaGraphAddNode(&loop, g, tail.data(), nullptr, tail.size(), &p);
  if (e != cudaSuccess) return check_cuda(c, e, "cudaGraphAddNode (while)");
  cudaGraph_t body = p.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return check_cuda(c, e, "cudaStreamBeginCaptureToGraph (body)");
  c->in_loop = true;
  c->loop_handle = h;
  // the body runs repeatedly with changing increments: it always computes its boxes
  c->incr_zero = false;
  c->boxes_x_valid = false;
  if ((rc = sub_iteration(c, rk))) return rc;
  c->in_loop = false;
  if ((rc = end_capture(c, nullptr))) return rc;
  sinks->assign(1, loop);
  return EIF_OK;
}

// Captures one time step of c into g (appended as an independent branch: its first
// nodes have no dependences) and returns the buffer indices the step ends with. The
// host state of c is left as before the capture; on failure g may hold a partial
// branch and should be discarded.
int capture_step(eif_ctx *c, cudaGraph_t g, int *cur1, int *scur1) {
  int rc = step_capture_begin(c);
  if (rc) return rc;
  const int cur0 = c->cur, scur0 = c->scur;
  std::vector<cudaGraphNode_t> tail;
  for (int part = 0; part < 4; part++) {
    if ((rc = capture_step_part(c, g, tail, part, &tail)) ||
        (part < 3 && (rc = capture_subiteration_loop(c, g, tail, part, &tail)))) {
      step_capture_end(c, cur0, scur0);
      return rc;
    }
  }
  *cur1 = c->cur;
  *scur1 = c->scur;
  step_capture_end(c, cur0, scur0);
  return EIF_OK;
}

namespace {

int build(eif_ctx *c, eif_ctx::StepGraph &sg) {
  cudaGraph_t g = nullptr;
  EIF_CK(c, cudaGraphCreate(&g, 0));
  int cur1 = 0, scur1 = 0;
  int rc = capture_step(c, g, &cur1, &scur1);
  if (rc) {
    cudaGraphDestroy(g);
    return rc;
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return check_cuda(c, e, "cudaGraphInstantiate");
  }
  sg.graph = g;
  sg.exec = exec;
  sg.cur0 = c->cur;
  sg.scur0 = c->scur;
  sg.cur1 = cur1;
  sg.scur1 = scur1;
  return EIF_OK;
}

}  // namespace

void graphs_free(eif_ctx *c) {
  for (auto &sg : c->graphs) {
    if (sg.exec) cudaGraphExecDestroy(sg.exec);
    if (sg.graph) cudaGraphDestroy(sg.graph);
    sg = eif_ctx::StepGraph{};
  }
}

int step_graph_launch(eif_ctx *c) {
  eif_ctx::StepGraph *sg = nullptr;
  for (auto &g : c->graphs) {
    if (g.exec && g.cur0 == c->cur && g.scur0 == c->scur) sg = &g;
  }
  if (!sg) {
    for (auto &g : c->graphs) {
      if (!g.exec) { sg = &g; break; }
    }
    if (!sg) {
      graphs_free(c);
      sg = &c->graphs[0];
    }
    int rc = build(c, *sg);
    if (rc) return rc;
  }
  EIF_CK(c, cudaGraphLaunch(sg->exec, c->stream));
  c->cur = sg->cur1;
  c->scur = sg->scur1;
  return EIF_OK;
}

}  // namespace eif
