// Asynchronous state snapshots for checkpoints (save.c:109-122 writes ux, uy, p and the
// particle state at a step). eif_snapshot_take copies the state on the device (on the
// context's stream, so in order with the steps) into a snapshot buffer and starts the
// copy of that buffer to page-locked host memory on a stream of its own; the steps the
// caller launches next overlap with that transfer. eif_snapshot_wait waits for it and
// converts to the reference layouts.
#include "eif_internal.cuh"
#include <cstring>

namespace eif {

struct Snapshot {
  double *dev = nullptr, *host = nullptr;
  size_t cap = 0;               // doubles
  cudaStream_t stream = nullptr;
  cudaEvent_t taken = nullptr, copied = nullptr;
  size_t nfield = 0;
  int ld = 0, np = 0, pcap = 0, step = 0;
  double time = 0.;
  bool pending = false;
};

void snapshot_free(eif_ctx *c) {
  Snapshot *s = c->snap;
  if (!s) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->dev) cudaFree(s->dev);
  if (s->host) cudaFreeHost(s->host);
  if (s->taken) cudaEventDestroy(s->taken);
  if (s->copied) cudaEventDestroy(s->copied);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  c->snap = nullptr;
}

}  // namespace eif

using namespace eif;

extern "C" {

int eif_snapshot_take(eif_ctx *c) {
  if (!c) return EIF_ERR_ARG;
  if (!c->fluid_pushed) return fail(c, EIF_ERR_STATE, "push the fluid state before taking a snapshot");
  if (!c->snap) {
    c->snap = new Snapshot;
    EIF_CK(c, cudaStreamCreateWithFlags(&c->snap->stream, cudaStreamNonBlocking));
    EIF_CK(c, cudaEventCreateWithFlags(&c->snap->taken, cudaEventDisableTiming));
    EIF_CK(c, cudaEventCreateWithFlags(&c->snap->copied, cudaEventDisableTiming));
  }
  Snapshot *s = c->snap;
  // an earlier snapshot's transfer must finish before its buffers are reused
  EIF_CK(c, cudaEventSynchronize(s->copied));
  const size_t need = 3 * c->nfield + (size_t)EIF_NFIELDS * c->pcap;
  if (need > s->cap) {
    if (s->dev) cudaFree(s->dev);
    if (s->host) cudaFreeHost(s->host);
    s->dev = nullptr;
    s->host = nullptr;
    s->cap = 0;
    EIF_CK(c, cudaMalloc((void **)&s->dev, sizeof(double) * need));
    EIF_CK(c, cudaMallocHost((void **)&s->host, sizeof(double) * need));
    s->cap = need;
  }
  const size_t fb = sizeof(double) * c->nfield;
  EIF_CK(c, cudaMemcpyAsync(s->dev, c->ux[c->cur], fb, cudaMemcpyDeviceToDevice, c->stream));
  EIF_CK(c, cudaMemcpyAsync(s->dev + c->nfield, c->uy[c->cur], fb, cudaMemcpyDeviceToDevice, c->stream));
  EIF_CK(c, cudaMemcpyAsync(s->dev + 2 * c->nfield, c->p, fb, cudaMemcpyDeviceToDevice, c->stream));
  if (c->np > 0)
    EIF_CK(c, cudaMemcpyAsync(s->dev + 3 * c->nfield, c->P, sizeof(double) * EIF_NFIELDS * c->pcap,
                              cudaMemcpyDeviceToDevice, c->stream));
  EIF_CK(c, cudaEventRecord(s->taken, c->stream));
  EIF_CK(c, cudaStreamWaitEvent(s->stream, s->taken, 0));
  EIF_CK(c, cudaMemcpyAsync(s->host, s->dev, sizeof(double) * need, cudaMemcpyDeviceToHost, s->stream));
  EIF_CK(c, cudaEventRecord(s->copied, s->stream));
  s->nfield = c->nfield;
  s->ld = c->ld;
  s->np = c->np;
  s->pcap = c->pcap;
  s->step = c->step;
  s->time = c->time;
  s->pending = true;
  return EIF_OK;
}

// the snapshot in the eif_push_fluid layouts (any pointer may be NULL) and n particle
// records (n must be the particle count at the snapshot); step and time of the snapshot
int eif_snapshot_wait(eif_ctx *c, double *ux, double *uy, double *p, int n, double *records, int *step,
                      double *time) {
  if (!c) return EIF_ERR_ARG;
  Snapshot *s = c->snap;
  if (!s || !s->pending) return fail(c, EIF_ERR_STATE, "no snapshot taken");
  if (records && n != s->np) return fail(c, EIF_ERR_ARG, "the snapshot holds %d particles", s->np);
  EIF_CK(c, cudaEventSynchronize(s->copied));
  const int rows = c->jtot + 2;
  auto out = [&](double *dst, const double *src, int w) {
    for (int j = 0; j < rows; j++) std::memcpy(dst + (size_t)j * w, src + (size_t)j * s->ld, sizeof(double) * w);
  };
  if (ux) out(ux, s->host, c->itot + 1);
  if (uy) out(uy, s->host + s->nfield, c->itot + 2);
  if (p) out(p, s->host + 2 * s->nfield, c->itot + 2);
  if (records) {
    const double *P = s->host + 3 * s->nfield;
    for (int f = 0; f < EIF_NFIELDS; f++)
      for (int k = 0; k < s->np; k++) records[(size_t)k * EIF_NFIELDS + f] = P[(size_t)f * s->pcap + k];
  }
  if (step) *step = s->step;
  if (time) *time = s->time;
  return EIF_OK;
}

}  // extern "C"
