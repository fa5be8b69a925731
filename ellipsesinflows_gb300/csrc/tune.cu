// Tile-shape tuner. The stencil kernels (predictor, projection) process tiles of 32
// columns by TY rows, and the block-Thomas kernel one wavenumber column per thread;
// none of these shapes changes a result, only the speed (occupancy, the halo overhead
// of the staged mixed-precision predictor, the L2 reuse of neighbouring rows). For a
// grid size and precision the tuner times every candidate on scratch copies of the
// fields the kernels write and keeps the fastest; the choice is cached for the
// process, so contexts of the same size (a batch of suspensions) are timed once.
// Set EIF_TUNE=0 in the environment to keep the default shapes, or EIF_TILES=p,c,t to
// fix them.
#include "eif_internal.cuh"
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace {

std::mutex g_mu;
std::map<std::tuple<int, int, int>, eif_ctx::Tiles> g_cache;

constexpr int REPS = 5;

// best of REPS timed launches (after one untimed), in ms
template <typename F>
int best_ms(eif_ctx *c, cudaEvent_t e0, cudaEvent_t e1, F launch, float *out) {
  int rc = launch();
  if (rc) return rc;
  float best = 1e30f;
  for (int r = 0; r < REPS; r++) {
    EIF_CK(c, cudaEventRecord(e0, c->stream));
    if ((rc = launch())) return rc;
    EIF_CK(c, cudaEventRecord(e1, c->stream));
    EIF_CK(c, cudaEventSynchronize(e1));
    float ms = 0.f;
    EIF_CK(c, cudaEventElapsedTime(&ms, e0, e1));
    best = std::min(best, ms);
  }
  *out = best;
  return EIF_OK;
}

}  // namespace

namespace eif {

int tune_tiles(eif_ctx *c) {
  if (c->tiles.tuned) return EIF_OK;
  c->tiles.tuned = true;
  const char *env = std::getenv("EIF_TUNE");
  if (env && env[0] == '0') return EIF_OK;
  // fixed shapes "pred,corr,tdm" (rows 4|8|16, rows 4|8|16, threads 64|128|256)
  if (const char *fx = std::getenv("EIF_TILES")) {
    int a = 0, b = 0, t = 0;
    auto rows_ok = [](int v) { return v == 4 || v == 8 || v == 16; };
    if (std::sscanf(fx, "%d,%d,%d", &a, &b, &t) != 3 || !rows_ok(a) || !rows_ok(b) || (t != 64 && t != 128 && t != 256))
      return fail(c, EIF_ERR_ARG, "EIF_TILES must be rows,rows,threads with rows 4|8|16 and threads 64|128|256");
    c->tiles.pred = a;
    c->tiles.corr = b;
    c->tiles.tdm = t;
    return EIF_OK;
  }
  const auto key = std::make_tuple(c->itot, c->jtot, c->cfg.precision);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      c->tiles = it->second;
      return EIF_OK;
    }
  }
  const bool mixed = c->cfg.precision == EIF_PREC_MIXED;
  // the fields the timed kernels write, swapped for scratch copies
  std::vector<double **> dfields = {&c->ux[0], &c->ux[1], &c->uy[0], &c->uy[1], &c->p, &c->psi,
                                    &c->sxa[0], &c->sxa[1], &c->sya[0], &c->sya[1]};
  std::vector<float **> ffields;
  if (mixed) ffields = {&c->sxf[0], &c->sxf[1], &c->syf[0], &c->syf[1], &c->uxf[0], &c->uxf[1], &c->uyf[0], &c->uyf[1]};
  std::vector<double *> dkeep, dscr;
  std::vector<float *> fkeep, fscr;
  const int cur = c->cur, scur = c->scur;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto cleanup = [&]() {
    for (size_t k = 0; k < dscr.size(); k++) {
      *dfields[k] = dkeep[k];
      cudaFree(dscr[k]);
    }
    for (size_t k = 0; k < fscr.size(); k++) {
      *ffields[k] = fkeep[k];
      cudaFree(fscr[k]);
    }
    c->cur = cur;
    c->scur = scur;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  };
  auto run = [&]() -> int {
    EIF_CK(c, cudaEventCreate(&e0));
    EIF_CK(c, cudaEventCreate(&e1));
    for (double **f : dfields) {
      double *q = nullptr;
      EIF_CK(c, cudaMalloc((void **)&q, sizeof(double) * c->nfield));
      EIF_CK(c, cudaMemcpyAsync(q, *f, sizeof(double) * c->nfield, cudaMemcpyDeviceToDevice, c->stream));
      dkeep.push_back(*f);
      dscr.push_back(q);
      *f = q;
    }
    for (float **f : ffields) {
      float *q = nullptr;
      EIF_CK(c, cudaMalloc((void **)&q, sizeof(float) * c->nfield));
      EIF_CK(c, cudaMemcpyAsync(q, *f, sizeof(float) * c->nfield, cudaMemcpyDeviceToDevice, c->stream));
      fkeep.push_back(*f);
      fscr.push_back(q);
      *f = q;
    }
    const bool ibm = c->np > 0;
    const int tys[3] = {4, 8, 16};
    float best = 1e30f;
    int pick = c->tiles.pred;
    bool pick_copy = c->tiles.pred_copy;
    // the mixed predictor with tensor-copy staging and the plain one, each tile height
    for (int copy = 0; copy < (mixed ? 2 : 1); copy++) {
      for (int ty : tys) {
        c->tiles.pred = ty;
        c->tiles.pred_copy = copy == 1;
        float ms = 0.f;
        int rc = best_ms(c, e0, e1, [&]() { return launch_predictor(c, 0); }, &ms);
        if (rc) return rc;
        if (ms < best) { best = ms; pick = ty; pick_copy = copy == 1; }
      }
    }
    c->tiles.pred = pick;
    c->tiles.pred_copy = pick_copy;
    best = 1e30f;
    pick = c->tiles.corr;
    for (int ty : tys) {
      c->tiles.corr = ty;
      float ms = 0.f;
      int rc = best_ms(c, e0, e1, [&]() { return launch_correct(c, 0, ibm, true); }, &ms);
      if (rc) return rc;
      if (ms < best) { best = ms; pick = ty; }
    }
    c->tiles.corr = pick;
    if (c->pp.blk > 0) {
      const int tts[3] = {64, 128, 256};
      best = 1e30f;
      pick = c->tiles.tdm;
      for (int tt : tts) {
        c->tiles.tdm = tt;
        float ms = 0.f;
        int rc = best_ms(c, e0, e1, [&]() { return launch_potential(c, 0, false); }, &ms);
        if (rc) return rc;
        if (ms < best) { best = ms; pick = tt; }
      }
      c->tiles.tdm = pick;
    }
    EIF_CK(c, cudaStreamSynchronize(c->stream));
    return EIF_OK;
  };
  const int rc = run();
  cleanup();
  if (rc) {
    c->tiles = eif_ctx::Tiles();
    c->tiles.tuned = true;
    return rc;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  g_cache[key] = c->tiles;
  return EIF_OK;
}

}  // namespace eif

extern "C" int eif_tiles(eif_ctx *c, int *tiles) {
  if (!c || !tiles) return EIF_ERR_ARG;
  tiles[0] = c->tiles.pred;
  tiles[1] = c->tiles.corr;
  tiles[2] = c->tiles.tdm;
  tiles[3] = (c->tiles.tuned ? 1 : 0) | (c->tiles.pred_copy && c->pred_tma_ctas[1] > 0 ? 2 : 0) |
             (c->cfg.precision == EIF_PREC_MIXED && c->uni_x.on ? 4 : 0);
  return EIF_OK;
}
