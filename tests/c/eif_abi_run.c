/* A plain C host of the C ABI (include/eif.h) on the GPU: reads a case (configuration,
 * fluid state, particle records, number of steps) from a binary file, advances it with
 * eif_create, eif_push_fluid, eif_push_particles and eif_advance, and writes the state
 * after the steps (step counter, time, ux, uy, p, records) to a binary file. The test
 * tests/test_gpu_c_host.py builds it with gcc against libeif_gb300.so and compares the
 * result bit for bit with the same case advanced through the Python binding.
 *
 *   eif_abi_run <input> <output>
 *
 * input:  int32 itot, jtot, precision, nsteps, n; float64 ly, Re, Fr, extfrcy,
 *         safefactors[3], uy_wall[2]; then ux, uy, p in the reference layouts and
 *         n * EIF_NFIELDS records (float64)
 * output: int32 step; float64 time; ux, uy, p, records */
#include <stdio.h>
#include <stdlib.h>
#include "eif.h"

static int read_all(FILE *f, void *p, size_t size, size_t n) { return fread(p, size, n, f) == n; }
static int write_all(FILE *f, const void *p, size_t size, size_t n) { return fwrite(p, size, n, f) == n; }

static int fail(const char *what, int rc, eif_ctx *ctx) {
  fprintf(stderr, "%s failed: %d %s\n", what, rc, ctx ? eif_last_error(ctx) : "");
  return 1;
}

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s <input> <output>\n", argv[0]);
    return 2;
  }
  FILE *in = fopen(argv[1], "rb");
  if (!in) return fail("open input", -1, NULL);
  int hdr[5];
  double par[9];
  if (!read_all(in, hdr, sizeof(int), 5) || !read_all(in, par, sizeof(double), 9)) return fail("read header", -1, NULL);
  const int itot = hdr[0], jtot = hdr[1], nsteps = hdr[3], n = hdr[4];
  eif_config_t cfg;
  cfg.itot = itot;
  cfg.jtot = jtot;
  cfg.precision = hdr[2];
  cfg.device = 0;
  cfg.ly = par[0];
  cfg.Re = par[1];
  cfg.Fr = par[2];
  cfg.extfrcy = par[3];
  cfg.safefactors[0] = par[4];
  cfg.safefactors[1] = par[5];
  cfg.safefactors[2] = par[6];
  cfg.uy_wall[0] = par[7];
  cfg.uy_wall[1] = par[8];
  const size_t nux = (size_t)(jtot + 2) * (itot + 1), nuy = (size_t)(jtot + 2) * (itot + 2);
  const size_t nrec = (size_t)n * EIF_NFIELDS;
  double *ux = malloc(sizeof(double) * nux), *uy = malloc(sizeof(double) * nuy), *p = malloc(sizeof(double) * nuy);
  double *rec = malloc(sizeof(double) * (nrec ? nrec : 1));
  if (!ux || !uy || !p || !rec) return fail("malloc", -1, NULL);
  if (!read_all(in, ux, sizeof(double), nux) || !read_all(in, uy, sizeof(double), nuy) ||
      !read_all(in, p, sizeof(double), nuy) || !read_all(in, rec, sizeof(double), nrec))
    return fail("read state", -1, NULL);
  fclose(in);

  eif_ctx *ctx = NULL;
  int rc = eif_create(&cfg, &ctx);
  if (rc) return fail("eif_create", rc, ctx);
  if ((rc = eif_push_fluid(ctx, ux, uy, p))) return fail("eif_push_fluid", rc, ctx);
  if ((rc = eif_push_particles(ctx, n, rec))) return fail("eif_push_particles", rc, ctx);
  if ((rc = eif_advance(ctx, nsteps))) return fail("eif_advance", rc, ctx);
  int step = 0;
  double time = 0.;
  if ((rc = eif_get_time(ctx, &step, &time))) return fail("eif_get_time", rc, ctx);
  if ((rc = eif_pull_fluid(ctx, ux, uy, p, NULL))) return fail("eif_pull_fluid", rc, ctx);
  if ((rc = eif_pull_particles(ctx, n, rec))) return fail("eif_pull_particles", rc, ctx);
  if ((rc = eif_destroy(ctx))) return fail("eif_destroy", rc, NULL);

  FILE *out = fopen(argv[2], "wb");
  if (!out) return fail("open output", -1, NULL);
  if (!write_all(out, &step, sizeof(int), 1) || !write_all(out, &time, sizeof(double), 1) ||
      !write_all(out, ux, sizeof(double), nux) || !write_all(out, uy, sizeof(double), nuy) ||
      !write_all(out, p, sizeof(double), nuy) || !write_all(out, rec, sizeof(double), nrec))
    return fail("write output", -1, NULL);
  fclose(out);
  free(ux);
  free(uy);
  free(p);
  free(rec);
  printf("advanced %d steps to t = %.17g\n", step, time);
  return 0;
}
