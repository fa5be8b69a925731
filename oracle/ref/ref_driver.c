/*
 * Step-driven driver around the reference solver's own, unmodified sources.
 *
 * TEST INFRASTRUCTURE ONLY. Built by oracle/ref/Makefile into oracle/_ref/
 * together with the reference's src/ files and the single-rank MPI/FFTW shims.
 * Python tests load it with ctypes to obtain reference outputs for the same
 * inputs that are given to the GPU library.
 *
 * The reference's src/main.c is compiled into this translation unit (with its
 * main() renamed) so that its file-static integrate() (src/main.c:13-55) is
 * callable. Everything else is called through the reference's public headers:
 *   param_init             src/param/init.c:215     (reads the environment)
 *   parallel_init          src/parallel/init.c:29
 *   fluid_init             src/fluid/init.c:87
 *   param_decide_dt        src/param/decide_dt.c:11
 *   and the per-stage functions declared in include/fluid.h and include/suspensions.h.
 * The particle container is allocated here with the layout of
 * src/suspensions/init.c:10-21 (dux, duy, particles, buf) so that particles can
 * be handed in from memory instead of npy files.
 */
#define main eif_reference_program_main
#include EIF_REFERENCE_MAIN
#undef main

#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include "ellipse.h"

#define REF_NFIELDS 30

typedef struct {
  param_t *param;
  parallel_t *parallel;
  fluid_t *fluid;
  suspensions_t *suspensions;
} ref_ctx;

static void set_env_double(const char *name, double v){
  char buf[64];
  snprintf(buf, sizeof(buf), "%.17g", v);
  setenv(name, buf, 1);
}

static void set_env_int(const char *name, int v){
  char buf[64];
  snprintf(buf, sizeof(buf), "%d", v);
  setenv(name, buf, 1);
}

/* create a solver state: zero fluid, no particles; parameters go through the environment */
ref_ctx *ref_create(int itot, int jtot, double ly, double Re, double Fr, double extfrcy,
                    double sf_adv, double sf_dif, double sf_par){
  unsetenv("dirname_restart");
  set_env_int("itot", itot);
  set_env_int("jtot", jtot);
  set_env_double("ly", ly);
  set_env_double("Re", Re);
  set_env_double("Fr", Fr);
  set_env_double("extfrcy", extfrcy);
  set_env_double("safefactor_adv", sf_adv);
  set_env_double("safefactor_dif", sf_dif);
  set_env_double("safefactor_par", sf_par);
  /* param_init prints every parameter: keep the oracle quiet */
  fflush(stdout);
  FILE *saved = stdout;
  FILE *devnull = fopen("/dev/null", "w");
  if(devnull) stdout = devnull;
  ref_ctx *c = calloc(1, sizeof(ref_ctx));
  c->param = param_init();
  if(devnull){ stdout = saved; fclose(devnull); }
  c->parallel = parallel_init();
  c->fluid = fluid_init(c->param, c->parallel);
  c->suspensions = calloc(1, sizeof(suspensions_t));
  {
    /* DUX_MEMSIZE / DUY_MEMSIZE (include/arrays/suspensions.h) are written in terms of itot, jsize */
    const int itot = c->param->itot;
    const int jsize = c->param->jtot;
    c->suspensions->dux = calloc(1, DUX_MEMSIZE);
    c->suspensions->duy = calloc(1, DUY_MEMSIZE);
  }
  c->suspensions->n_particles = 0;
  c->suspensions->particles = NULL;
  c->suspensions->buf = calloc(1, sizeof(double));
  return c;
}

void ref_destroy(ref_ctx *c){
  if(c == NULL) return;
  suspensions_t *s = c->suspensions;
  for(int n = 0; n < s->n_particles; n++) free(s->particles[n]);
  free(s->particles);
  free(s->dux);
  free(s->duy);
  free(s->buf);
  free(s);
  fluid_finalise(c->fluid);
  parallel_finalise(c->parallel);
  param_finalise(c->param);
  free(c);
}

/* sizes (in doubles) of the haloed host arrays, reference layouts include/arrays/fluid.h */
int ref_sizes(const ref_ctx *c, long long *n_ux, long long *n_uy){
  const int itot = c->param->itot;
  const int jtot = c->param->jtot;
  *n_ux = (long long)(itot+1)*(jtot+2);
  *n_uy = (long long)(itot+2)*(jtot+2);
  return 0;
}

/* copy full haloed arrays in, then refresh halos/walls with the reference's BC routines */
int ref_set_fluid(ref_ctx *c, const double *ux, const double *uy, const double *p){
  long long nux, nuy;
  ref_sizes(c, &nux, &nuy);
  memcpy(c->fluid->ux, ux, sizeof(double)*nux);
  memcpy(c->fluid->uy, uy, sizeof(double)*nuy);
  memcpy(c->fluid->p, p, sizeof(double)*nuy);
  fluid_update_boundaries_ux(c->param, c->parallel, c->fluid->ux);
  fluid_update_boundaries_uy(c->param, c->parallel, c->fluid->uy);
  fluid_update_boundaries_p(c->param, c->parallel, c->fluid->p);
  return 0;
}

int ref_get_fluid(const ref_ctx *c, double *ux, double *uy, double *p, double *psi){
  long long nux, nuy;
  ref_sizes(c, &nux, &nuy);
  if(ux) memcpy(ux, c->fluid->ux, sizeof(double)*nux);
  if(uy) memcpy(uy, c->fluid->uy, sizeof(double)*nuy);
  if(p) memcpy(p, c->fluid->p, sizeof(double)*nuy);
  if(psi) memcpy(psi, c->fluid->psi, sizeof(double)*nuy);
  return 0;
}

/* source-term arrays: srcuxa/b/g (itot-1)*jtot, srcuya/b/g itot*jtot */
int ref_get_src(const ref_ctx *c, double *uxa, double *uxb, double *uxg, double *uya, double *uyb, double *uyg){
  const int itot = c->param->itot;
  const int jtot = c->param->jtot;
  size_t nx = sizeof(double)*(size_t)(itot-1)*jtot;
  size_t ny = sizeof(double)*(size_t)itot*jtot;
  if(uxa) memcpy(uxa, c->fluid->srcuxa, nx);
  if(uxb) memcpy(uxb, c->fluid->srcuxb, nx);
  if(uxg) memcpy(uxg, c->fluid->srcuxg, nx);
  if(uya) memcpy(uya, c->fluid->srcuya, ny);
  if(uyb) memcpy(uyb, c->fluid->srcuyb, ny);
  if(uyg) memcpy(uyg, c->fluid->srcuyg, ny);
  return 0;
}

int ref_set_src(ref_ctx *c, const double *uxa, const double *uya){
  const int itot = c->param->itot;
  const int jtot = c->param->jtot;
  memcpy(c->fluid->srcuxa, uxa, sizeof(double)*(size_t)(itot-1)*jtot);
  memcpy(c->fluid->srcuya, uya, sizeof(double)*(size_t)itot*jtot);
  return 0;
}

int ref_get_ibm_fields(const ref_ctx *c, double *dux, double *duy){
  long long nux, nuy;
  ref_sizes(c, &nux, &nuy);
  memcpy(dux, c->suspensions->dux, sizeof(double)*nuy);
  memcpy(duy, c->suspensions->duy, sizeof(double)*nuy);
  return 0;
}

/* particles as n records of REF_NFIELDS doubles in particle_t order (include/suspensions.h:8-31) */
int ref_set_particles(ref_ctx *c, int n, const double *records){
  suspensions_t *s = c->suspensions;
  for(int k = 0; k < s->n_particles; k++) free(s->particles[k]);
  free(s->particles);
  free(s->buf);
  s->n_particles = n;
  s->particles = calloc(n > 0 ? n : 1, sizeof(particle_t *));
  for(int k = 0; k < n; k++){
    s->particles[k] = calloc(1, sizeof(particle_t));
    memcpy(s->particles[k], records+(size_t)k*REF_NFIELDS, sizeof(particle_t));
  }
  s->buf = calloc(3*(n > 0 ? n : 1), sizeof(double));
  return sizeof(particle_t) == REF_NFIELDS*sizeof(double) ? 0 : -1;
}

int ref_get_particles(const ref_ctx *c, double *records){
  const suspensions_t *s = c->suspensions;
  for(int k = 0; k < s->n_particles; k++){
    memcpy(records+(size_t)k*REF_NFIELDS, s->particles[k], sizeof(particle_t));
  }
  return s->n_particles;
}

double ref_get_dt(const ref_ctx *c){ return c->param->dt; }
void ref_set_dt(ref_ctx *c, double dt){ c->param->dt = dt; }
double ref_get_time(const ref_ctx *c){ return c->param->time; }
int ref_get_step(const ref_ctx *c){ return c->param->step; }

/* grid metrics as produced by the reference's set_coordinate (src/param/init.c:105-167) */
int ref_get_grid(const ref_ctx *c, double *xf, double *xc, double *dxf, double *dxc, double *yf, double *yc){
  const int itot = c->param->itot;
  const int jtot = c->param->jtot;
  memcpy(xf, c->param->xf, sizeof(double)*(itot+1));
  memcpy(xc, c->param->xc, sizeof(double)*(itot+2));
  memcpy(dxf, c->param->dxf, sizeof(double)*itot);
  memcpy(dxc, c->param->dxc, sizeof(double)*(itot+1));
  memcpy(yf, c->param->yf, sizeof(double)*(jtot+1));
  memcpy(yc, c->param->yc, sizeof(double)*jtot);
  return 0;
}

/* the reference's own logging() (src/logging.c:197-208): writes output/log/*.dat under
 * the current directory for the given step, time and log rate */
int ref_logging(ref_ctx *c, int step, double time, double log_rate){
  c->param->step = step;
  c->param->time = time;
  c->param->log.rate = log_rate;
  return logging(c->param, c->parallel, c->fluid, c->suspensions);
}

/* the reference's own save() (src/save.c:109-122): writes output/save/step%010d/*.npy
 * under the current directory for the given step and time */
int ref_save(ref_ctx *c, int step, double time){
  c->param->step = step;
  c->param->time = time;
  return save(c->param, c->parallel, c->fluid, c->suspensions);
}

/* the reference's statistics (src/statistics/): statistics_init on first use,
 * statistics_collect on the current state, statistics_output (writes
 * output/stat/step%010d/ under the current directory) for the given step and time */
static statistics_t *ref_stats = NULL;
int ref_stats_collect(ref_ctx *c){
  if(!ref_stats) ref_stats = statistics_init(c->param, c->parallel);
  return statistics_collect(c->param, c->parallel, c->fluid, c->suspensions, ref_stats);
}
int ref_stats_output(ref_ctx *c, int step, double time){
  if(!ref_stats) return 1;
  c->param->step = step;
  c->param->time = time;
  int rc = statistics_output(c->param, c->parallel, ref_stats);
  statistics_finalise(ref_stats);
  ref_stats = NULL;
  return rc;
}

double ref_decide_dt(ref_ctx *c){
  param_decide_dt(c->param, c->parallel, c->fluid, c->suspensions);
  return c->param->dt;
}

/* the reference's own integrate() (src/main.c:13-55), unmodified */
int ref_integrate(ref_ctx *c){
  return integrate(c->param, c->parallel, c->fluid, c->suspensions);
}

/*
 * The same call sequence as integrate() (src/main.c:13-55) with the number of
 * particle sub-iterations of each RK stage recorded in substeps[0..2]. Tests
 * check that it is bit-identical to ref_integrate.
 */
int ref_integrate_counted(ref_ctx *c, int *substeps){
  const param_t *param = c->param;
  const parallel_t *parallel = c->parallel;
  fluid_t *fluid = c->fluid;
  suspensions_t *suspensions = c->suspensions;
  for(int rkstep = 0; rkstep < RKSTEPMAX; rkstep++){
    suspensions_reset_particle_increments(suspensions);
    fluid_update_boundaries_ux(param, parallel, fluid->ux);
    fluid_update_boundaries_uy(param, parallel, fluid->uy);
    fluid_update_boundaries_p(param, parallel, fluid->p);
    suspensions_compute_inertia(param, parallel, 0, fluid, suspensions);
    fluid_update_velocity(param, parallel, rkstep, fluid);
    suspensions_exchange_momentum(param, parallel, fluid, suspensions);
    suspensions_update_momentum_fleid(param, parallel, fluid, suspensions);
    fluid_compute_potential(param, parallel, rkstep, fluid);
    fluid_correct_velocity(param, parallel, rkstep, fluid);
    fluid_update_pressure(param, parallel, fluid);
    suspensions_compute_collision_force(param, parallel, 0, suspensions);
    int substep;
    for(substep = 0; ; substep++){
      suspensions_compute_inertia(param, parallel, 1, fluid, suspensions);
      suspensions_compute_collision_force(param, parallel, 1, suspensions);
      double residual;
      suspensions_increment_particles(param, rkstep, suspensions, &residual);
      if(residual < 1.e-8) break;
      if(substep > 100) break;
    }
    if(substeps) substeps[rkstep] = substep+1;
    suspensions_update_particles(param, suspensions);
  }
  return 0;
}

/* one time step as the reference main loop does it (src/main.c:71-77) */
int ref_step(ref_ctx *c, int count_substeps, int *substeps){
  param_decide_dt(c->param, c->parallel, c->fluid, c->suspensions);
  if(count_substeps){
    ref_integrate_counted(c, substeps);
  }else{
    integrate(c->param, c->parallel, c->fluid, c->suspensions);
  }
  c->param->step += 1;
  c->param->time += c->param->dt;
  return 0;
}

/* individual stages, for kernel-level comparisons */
int ref_update_boundaries(ref_ctx *c){
  fluid_update_boundaries_ux(c->param, c->parallel, c->fluid->ux);
  fluid_update_boundaries_uy(c->param, c->parallel, c->fluid->uy);
  fluid_update_boundaries_p(c->param, c->parallel, c->fluid->p);
  return 0;
}
int ref_reset_increments(ref_ctx *c){ return suspensions_reset_particle_increments(c->suspensions); }
int ref_compute_inertia(ref_ctx *c, int cnstep){ return suspensions_compute_inertia(c->param, c->parallel, cnstep, c->fluid, c->suspensions); }
int ref_update_velocity(ref_ctx *c, int rkstep){ return fluid_update_velocity(c->param, c->parallel, rkstep, c->fluid); }
int ref_exchange_momentum(ref_ctx *c){ return suspensions_exchange_momentum(c->param, c->parallel, c->fluid, c->suspensions); }
int ref_update_momentum_field(ref_ctx *c){ return suspensions_update_momentum_fleid(c->param, c->parallel, c->fluid, c->suspensions); }
int ref_compute_potential(ref_ctx *c, int rkstep){ return fluid_compute_potential(c->param, c->parallel, rkstep, c->fluid); }
int ref_correct_velocity(ref_ctx *c, int rkstep){ return fluid_correct_velocity(c->param, c->parallel, rkstep, c->fluid); }
int ref_update_pressure(ref_ctx *c){ return fluid_update_pressure(c->param, c->parallel, c->fluid); }
int ref_collision(ref_ctx *c, int cnstep){ return suspensions_compute_collision_force(c->param, c->parallel, cnstep, c->suspensions); }
double ref_increment(ref_ctx *c, int rkstep){
  double residual = 0.;
  suspensions_increment_particles(c->param, rkstep, c->suspensions, &residual);
  return residual;
}
int ref_update_particles(ref_ctx *c){ return suspensions_update_particles(c->param, c->suspensions); }

/* ellipse geometry helpers (src/ellipse.c, src/suspensions/auxiliary.c) */
double ref_find_normal_t(double a, double b, double x, double y){ return find_normal_t(a, b, x, y); }
double ref_s_weight(double h, double a, double b, double px, double py, double paz, double x, double y){
  return suspensions_s_weight(h, a, b, px, py, paz, x, y);
}
double ref_v_weight(double h, double a, double b, double px, double py, double paz, double x, double y){
  return suspensions_v_weight(h, a, b, px, py, paz, x, y);
}
