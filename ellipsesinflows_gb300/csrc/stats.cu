// Time-averaged statistics (src/statistics/collect.c:10-95) accumulated on the device:
// ux and ux^2 over the faces i = 1..itot+1, uy and uy^2 over i = 0..itot+1, and the
// sharp particle indicator phi (the number of particle images whose ellipse contains
// the cell centre) over the cells, for every collect; num counts the collects.
//
// The reference tests every cell against every particle (collect.c:66-81). A cell
// centre can only be inside an ellipse within its circumscribed circle, so here each
// (particle, image) visits the cells of its bounding box only (one block per box), with
// the reference's inside test in the same operations (no contraction into fused
// multiply-adds), and adds 1 to an integer count per cell; the counts are added to
// phi afterwards. Integer additions commute, so the result does not depend on the
// order of the boxes and equals the reference's sum of 1.0s.
#include "eif_internal.cuh"

namespace eif {

struct Stats {
  double *ux1 = nullptr, *ux2 = nullptr, *uy1 = nullptr, *uy2 = nullptr, *phi = nullptr;
  unsigned *cnt = nullptr;
  int num = 0;
  size_t nfield = 0;
};

void stats_free(eif_ctx *c) {
  Stats *s = c->stats;
  if (!s) return;
  for (double *p : {s->ux1, s->ux2, s->uy1, s->uy2, s->phi})
    if (p) cudaFree(p);
  if (s->cnt) cudaFree(s->cnt);
  delete s;
  c->stats = nullptr;
}

}  // namespace eif

namespace {

using eifd::ux_idx;
using eifd::uy_idx;

// collect.c:20-25, 37-42
__global__ void k_stats_fields(const double *__restrict__ ux, const double *__restrict__ uy, double *__restrict__ ux1,
                               double *__restrict__ ux2, double *__restrict__ uy1, double *__restrict__ uy2, int itot,
                               int jtot, int ld) {
  const long long n = (long long)(itot + 2) * jtot;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % (itot + 2)), j = 1 + (int)(t / (itot + 2));
    const int cy = uy_idx(i, j, ld);
    // the square rounded before the addition, as the reference computes it (no fused
    // multiply-add)
    const double v = uy[cy];
    uy1[cy] += v;
    uy2[cy] = __dadd_rn(uy2[cy], __dmul_rn(v, v));
    if (i >= 1) {
      const int cx = ux_idx(i, j, ld);
      const double u = ux[cx];
      ux1[cx] += u;
      ux2[cx] = __dadd_rn(ux2[cx], __dmul_rn(u, u));
    }
  }
}

// collect.c:66-81 restricted to the bounding box of each (particle, image)
__global__ void k_stats_phi(const double *__restrict__ P, int pcap, const double *__restrict__ xc,
                            const double *__restrict__ yc, double dx, double dy, double ly, int itot, int jtot, int ld,
                            unsigned *__restrict__ cnt) {
  const int n = blockIdx.x / 3, img = (int)(blockIdx.x % 3) - 1;
  const double pa = P[EIF_P_A * pcap + n], pb = P[EIF_P_B * pcap + n];
  const double px = P[EIF_P_X * pcap + n], py_ = P[EIF_P_Y * pcap + n] + ly * img, paz = P[EIF_P_AZ * pcap + n];
  const double r = fmax(pa, pb);
  // cells whose centre XC(i) = (i - 1/2) dx lies within r of the centre, with a cell to spare
  const int i0 = max(1, (int)floor((px - r) / dx) - 1), i1 = min(itot, (int)ceil((px + r) / dx) + 2);
  const int j0 = max(1, (int)floor((py_ - r) / dy) - 1), j1 = min(jtot, (int)ceil((py_ + r) / dy) + 2);
  if (i1 < i0 || j1 < j0) return;
  double s, c;
  sincos(-paz, &s, &c);
  const int w = i1 - i0 + 1;
  const int total = w * (j1 - j0 + 1);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int i = i0 + t % w, j = j0 + t / w;
    const double ddx = __dsub_rn(xc[i], px), ddy = __dsub_rn(yc[j], py_);
    const double x_ = __dsub_rn(__dmul_rn(c, ddx), __dmul_rn(s, ddy));
    const double y_ = __dadd_rn(__dmul_rn(s, ddx), __dmul_rn(c, ddy));
    const double qx = __ddiv_rn(x_, pa), qy = __ddiv_rn(y_, pb);
    if (__dsub_rn(__dsub_rn(1., __dmul_rn(qx, qx)), __dmul_rn(qy, qy)) > 0.) atomicAdd(cnt + uy_idx(i, j, ld), 1u);
  }
}

__global__ void k_stats_phi_add(unsigned *__restrict__ cnt, double *__restrict__ phi, int itot, int jtot, int ld) {
  const long long n = (long long)itot * jtot;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int c = uy_idx(1 + (int)(t % itot), 1 + (int)(t / itot), ld);
    const unsigned k = cnt[c];
    if (k) {
      phi[c] += (double)k;
      cnt[c] = 0u;
    }
  }
}

}  // namespace

using namespace eif;

extern "C" {

int eif_stats_reset(eif_ctx *c) {
  if (!c) return EIF_ERR_ARG;
  if (!c->stats) c->stats = new Stats;
  Stats *s = c->stats;
  const size_t bytes = sizeof(double) * c->nfield;
  if (s->nfield != c->nfield) {
    for (double **p : {&s->ux1, &s->ux2, &s->uy1, &s->uy2, &s->phi}) {
      if (*p) cudaFree(*p);
      *p = nullptr;
      EIF_CK(c, cudaMalloc((void **)p, bytes));
    }
    if (s->cnt) cudaFree(s->cnt);
    s->cnt = nullptr;
    EIF_CK(c, cudaMalloc((void **)&s->cnt, sizeof(unsigned) * c->nfield));
    s->nfield = c->nfield;
  }
  for (double *p : {s->ux1, s->ux2, s->uy1, s->uy2, s->phi}) EIF_CK(c, cudaMemsetAsync(p, 0, bytes, c->stream));
  EIF_CK(c, cudaMemsetAsync(s->cnt, 0, sizeof(unsigned) * c->nfield, c->stream));
  s->num = 0;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return EIF_OK;
}

// statistics_collect (collect.c:84-95) on the current state; asynchronous
int eif_stats_collect(eif_ctx *c) {
  if (!c) return EIF_ERR_ARG;
  if (!c->fluid_pushed) return fail(c, EIF_ERR_STATE, "push the fluid state before collecting statistics");
  if (!c->stats || c->stats->nfield != c->nfield) {
    int rc = eif_stats_reset(c);
    if (rc) return rc;
  }
  Stats *s = c->stats;
  EIF_PROF(c, "statistics", 3);
  k_stats_fields<<<c->sms * 4, 256, 0, c->stream>>>(c->ux[c->cur], c->uy[c->cur], s->ux1, s->ux2, s->uy1, s->uy2,
                                                     c->itot, c->jtot, c->ld);
  EIF_LAUNCH_CK(c);
  if (c->np > 0) {
    k_stats_phi<<<3 * c->np, 256, 0, c->stream>>>(c->P, c->pcap, c->xc, c->yc, c->dx, c->dy, c->ly, c->itot, c->jtot,
                                                   c->ld, s->cnt);
    EIF_LAUNCH_CK(c);
    k_stats_phi_add<<<c->sms * 4, 256, 0, c->stream>>>(s->cnt, s->phi, c->itot, c->jtot, c->ld);
    EIF_LAUNCH_CK(c);
  }
  s->num += 1;
  return EIF_OK;
}

// the accumulated sums in the reference's layouts (include/arrays/statistics.h): ux1, ux2
// (jtot+2) rows of itot+1, uy1, uy2, phi (jtot+2) rows of itot+2 (halo rows and the
// entries the reference does not accumulate are zero); any pointer may be NULL
int eif_stats_pull(eif_ctx *c, double *ux1, double *ux2, double *uy1, double *uy2, double *phi, int *num) {
  if (!c) return EIF_ERR_ARG;
  if (!c->stats) return fail(c, EIF_ERR_STATE, "no statistics collected");
  Stats *s = c->stats;
  const size_t dp = sizeof(double) * c->ld;
  const int rows = c->jtot + 2;
  const size_t wx = sizeof(double) * (c->itot + 1), wy = sizeof(double) * (c->itot + 2);
  auto pull = [&](double *dst, const double *src, size_t w) -> int {
    if (dst) EIF_CK(c, cudaMemcpy2DAsync(dst, w, src, dp, w, rows, cudaMemcpyDeviceToHost, c->stream));
    return EIF_OK;
  };
  int rc;
  if ((rc = pull(ux1, s->ux1, wx)) || (rc = pull(ux2, s->ux2, wx)) || (rc = pull(uy1, s->uy1, wy)) ||
      (rc = pull(uy2, s->uy2, wy)) || (rc = pull(phi, s->phi, wy)))
    return rc;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  if (num) *num = s->num;
  return EIF_OK;
}

}  // extern "C"
