/*
 * Drop-in driver: the reference's main program (src/main.c:56-112) with the time step
 * on the GPU. Everything else is the reference's own code, linked from its sources:
 * the environment-variable parameters (param_init, src/param/init.c:215), the initial
 * and restart fields from .npy files (fluid_init, suspensions_init), logging, save and
 * statistics. The step itself -- param_decide_dt + integrate + the counters
 * (src/main.c:69-74) -- is eif_advance(ctx, 1); the fields and the particles are
 * copied back into the reference's structures just before each log, save or
 * statistics event, the only places where the reference reads them between steps.
 *
 * Environment (besides the reference's): EIF_PRECISION = fp64 (default) or mixed;
 * EIF_UY_WALL = "lo,hi" wall velocities when the build uses the reference's Couette
 * boundary variant (the reference selects it by swapping a source file).
 *
 * Build: Makefile in this directory (REF = the reference checkout).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>
#include "param.h"
#include "parallel.h"
#include "fluid.h"
#include "suspensions.h"
#include "statistics.h"
#include "save.h"
#include "logging.h"
#include "eif.h"

static void check(eif_ctx *ctx, int rc, const char *what) {
  if (rc != EIF_OK) {
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, ctx ? eif_last_error(ctx) : "no context");
    exit(1);
  }
}

/* the particle_t records are EIF_NFIELDS doubles each (include/suspensions.h:8-31) */
static double *pack_particles(const suspensions_t *s) {
  const int n = s->n_particles;
  double *rec = calloc((size_t)(n > 0 ? n : 1) * EIF_NFIELDS, sizeof(double));
  for (int k = 0; k < n; k++) memcpy(rec + (size_t)k * EIF_NFIELDS, s->particles[k], sizeof(double) * EIF_NFIELDS);
  return rec;
}

static void pull_state(eif_ctx *ctx, param_t *param, fluid_t *fluid, suspensions_t *s, double *rec) {
  check(ctx, eif_pull_fluid(ctx, fluid->ux, fluid->uy, fluid->p, fluid->psi), "eif_pull_fluid");
  check(ctx, eif_pull_particles(ctx, s->n_particles, rec), "eif_pull_particles");
  for (int k = 0; k < s->n_particles; k++) memcpy(s->particles[k], rec + (size_t)k * EIF_NFIELDS, sizeof(double) * EIF_NFIELDS);
  check(ctx, eif_get_time(ctx, &param->step, &param->time), "eif_get_time");
  check(ctx, eif_get_dt(ctx, &param->dt), "eif_get_dt");
}

int main(void) {
  MPI_Init(NULL, NULL);
  double wtimes[2] = {0.};
  wtimes[0] = parallel_get_wtime(MPI_MIN);
  param_t *param = param_init();
  parallel_t *parallel = parallel_init();
  fluid_t *fluid = fluid_init(param, parallel);
  suspensions_t *suspensions = suspensions_init(param, parallel);
  statistics_t *statistics = statistics_init(param, parallel);
  if (parallel->mpisize != 1) {
    fprintf(stderr, "the GPU step runs on one rank\n");
    MPI_Abort(MPI_COMM_WORLD, 1);
  }
  /* the context: param_t's scalars (include/param.h:24-48) */
  eif_config_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.itot = param->itot;
  cfg.jtot = param->jtot;
  cfg.ly = param->ly;
  cfg.Re = param->Re;
  cfg.Fr = param->Fr;
  cfg.extfrcy = param->extfrcy;
  for (int k = 0; k < 3; k++) cfg.safefactors[k] = param->safefactors[k];
  const char *w = getenv("EIF_UY_WALL");
  if (w && sscanf(w, "%lf,%lf", &cfg.uy_wall[0], &cfg.uy_wall[1]) != 2) {
    fprintf(stderr, "EIF_UY_WALL must be lo,hi\n");
    return 1;
  }
  const char *prec = getenv("EIF_PRECISION");
  cfg.precision = (prec && strcmp(prec, "mixed") == 0) ? EIF_PREC_MIXED : EIF_PREC_FP64;
  cfg.device = 0;
  eif_ctx *ctx = NULL;
  check(ctx, eif_create(&cfg, &ctx), "eif_create");
  double *rec = pack_particles(suspensions);
  check(ctx, eif_push_fluid(ctx, fluid->ux, fluid->uy, fluid->p), "eif_push_fluid");
  check(ctx, eif_push_particles(ctx, suspensions->n_particles, rec), "eif_push_particles");
  check(ctx, eif_set_time(ctx, param->step, param->time), "eif_set_time");
  /* main loop (src/main.c:68-96) */
  for (;;) {
    check(ctx, eif_advance(ctx, 1), "eif_advance");   /* decide_dt, integrate, step += 1, time += dt */
    check(ctx, eif_get_time(ctx, &param->step, &param->time), "eif_get_time");
    const int log_due = param->log.next < param->time;
    const int save_due = param->save.next < param->time;
    const int stat_due = param->stat.next < param->time;
    if (log_due || save_due || stat_due) pull_state(ctx, param, fluid, suspensions, rec);
    if (log_due) {
      logging(param, parallel, fluid, suspensions);
      param->log.next += param->log.rate;
    }
    if (save_due) {
      save(param, parallel, fluid, suspensions);
      param->save.next += param->save.rate;
    }
    if (stat_due) {
      statistics_collect(param, parallel, fluid, suspensions, statistics);
      param->stat.next += param->stat.rate;
    }
    if (param->time > param->timemax) break;
    wtimes[1] = parallel_get_wtime(MPI_MAX);
    if (wtimes[1] - wtimes[0] > param->wtimemax) break;
  }
  if (parallel->mpirank == 0) printf("elapsed: %.2f [s]\n", wtimes[1] - wtimes[0]);
  /* final save and statistics (src/main.c:101-103) */
  pull_state(ctx, param, fluid, suspensions, rec);
  save(param, parallel, fluid, suspensions);
  statistics_output(param, parallel, statistics);
  eif_destroy(ctx);
  free(rec);
  statistics_finalise(statistics);
  suspensions_finalise(suspensions);
  fluid_finalise(fluid);
  parallel_finalise(parallel);
  param_finalise(param);
  MPI_Finalize();
  return 0;
}
