/*
 * EllipsesInFlows-GB300: C ABI of the time-step hot path.
 *
 * The reference solver (NaokiHori/EllipsesInFlows) advances its state with
 *     param_decide_dt(param, parallel, fluid, suspensions);   src/param/decide_dt.c:11
 *     integrate(param, parallel, fluid, suspensions);         src/main.c:13-55
 * inside its main loop (src/main.c:69-101). This library replaces those two calls.
 * The caller keeps its own host arrays in the reference's haloed layouts
 * (include/arrays/fluid.h:13-43) and its particle_t records
 * (include/suspensions.h:8-31); it pushes them once, steps on the GPU, and
 * pulls them back before logging / saving / statistics.
 *
 * Every function returns EIF_OK (0) or a negative error code; eif_last_error()
 * gives the message. A context owns one CUDA stream on one device and is not
 * thread-safe. All functions that take host arrays are synchronous with respect
 * to those arrays.
 */
#ifndef EIF_H
#define EIF_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ---- */
#define EIF_OK 0
#define EIF_ERR_ARG (-1)      /* invalid argument (sizes, null pointers, stage index) */
#define EIF_ERR_CUDA (-2)     /* a CUDA runtime call failed */
#define EIF_ERR_NOCONV (-3)   /* an iteration cap was hit on the device (circle fit) */
#define EIF_ERR_NOMEM (-4)    /* device or host allocation failed */
#define EIF_ERR_STATE (-5)    /* call out of order (e.g. step before push) */
#define EIF_ERR_NONFINITE (-6)/* a NaN/Inf was found in the velocity field */
#define EIF_ERR_TOO_LARGE (-7)/* size beyond the fixed scratch of eif_decide_dt_noalloc */

/* ---- arithmetic of the step ---- */
#define EIF_PREC_FP64 0       /* every operation in double precision */
#define EIF_PREC_MIXED 1      /* stencils / indicator / IBM forcing in float; storage,
                                 Poisson tridiagonal solves and particle dynamics in double */

/*
 * Particle record: 30 doubles in the field order of the reference's particle_t
 * (include/suspensions.h:8-31), so that a particle_t* can be passed as a double*.
 */
#define EIF_NFIELDS 30
enum eif_particle_field {
  EIF_P_DEN = 0, EIF_P_A = 1, EIF_P_B = 2,
  EIF_P_X = 3, EIF_P_Y = 4, EIF_P_AZ = 5,
  EIF_P_DX = 6, EIF_P_DY = 7, EIF_P_DAZ = 8,
  EIF_P_UX = 9, EIF_P_UY = 10, EIF_P_VZ = 11,
  EIF_P_DUX = 12, EIF_P_DUY = 13, EIF_P_DVZ = 14,
  EIF_P_FUX = 15, EIF_P_FUY = 16, EIF_P_TVZ = 17,
  EIF_P_IUX0 = 18, EIF_P_IUX1 = 19, EIF_P_IUY0 = 20, EIF_P_IUY1 = 21,
  EIF_P_IVZ0 = 22, EIF_P_IVZ1 = 23,
  EIF_P_CFX0 = 24, EIF_P_CFX1 = 25, EIF_P_CFY0 = 26, EIF_P_CFY1 = 27,
  EIF_P_CTZ0 = 28, EIF_P_CTZ1 = 29
};

/*
 * Run configuration. Mirrors the scalar members of the reference's param_t
 * (include/param.h:24-48) that the step reads, as loaded from the environment
 * by load_config (src/param/init.c:67-103). lx is fixed to 1 (include/param.h:14).
 * uy_wall is new: the reference selects moving walls by swapping
 * src/fluid/boundary_conditions.c for the Couette variant
 * (docs/source/examples/case1/config/src_fluid_boundary_conditions.c:39-40).
 */
typedef struct {
  int itot, jtot;            /* cells in x (wall-normal, walls at x=0,1) and y (periodic) */
  double ly;                 /* domain length in y */
  double Re, Fr;             /* Reynolds and Froude numbers (Fr = DBL_MAX: no buoyancy) */
  double extfrcy;            /* uniform body force in y (pressure-gradient driving) */
  double safefactors[3];     /* advective, diffusive, particle dt safety factors */
  double uy_wall[2];         /* y-velocity of the walls at x=0 and x=1 */
  int precision;             /* EIF_PREC_FP64 or EIF_PREC_MIXED */
  int device;                /* CUDA device ordinal */
} eif_config_t;

typedef struct eif_ctx eif_ctx;

/* ---- lifetime ---- */
int eif_create(const eif_config_t *cfg, eif_ctx **ctx);
int eif_destroy(eif_ctx *ctx);
const char *eif_last_error(const eif_ctx *ctx);
int eif_synchronize(eif_ctx *ctx);
/* the context's CUDA stream (a cudaStream_t), for callers that enqueue around it */
void *eif_stream(eif_ctx *ctx);

/* ---- state transfer (host arrays in the reference layouts) ----
 * ux:  (jtot+2) rows of (itot+1) doubles, UX(i,j) = ux[j*(itot+1)+(i-1)]
 * uy, p, psi: (jtot+2) rows of (itot+2) doubles, UY(i,j) = uy[j*(itot+2)+i]
 * Halo rows and wall columns are recomputed on push, as fluid_init does
 * (src/fluid/init.c:51,69,83). */
int eif_push_fluid(eif_ctx *ctx, const double *ux, const double *uy, const double *p);
int eif_pull_fluid(eif_ctx *ctx, double *ux, double *uy, double *p, double *psi);
/* records: n * EIF_NFIELDS doubles; n may change between pushes */
int eif_push_particles(eif_ctx *ctx, int n, const double *records);
int eif_pull_particles(eif_ctx *ctx, int n, double *records);
/* RK source terms: explicit part of the current (a) and previous (b) stage,
 * ux-like arrays of (itot-1)*jtot, uy-like of itot*jtot (include/arrays/fluid.h:53-103) */
int eif_pull_src(eif_ctx *ctx, double *srcuxa, double *srcuxb, double *srcuya, double *srcuyb);
int eif_push_src(eif_ctx *ctx, const double *srcuxa, const double *srcuya);
/* IBM response fields dux, duy (include/arrays/suspensions.h:13-23), uy-like layout */
int eif_pull_ibm_fields(eif_ctx *ctx, double *dux, double *duy);

/* ---- time stepping ---- */
/* param_decide_dt (src/param/decide_dt.c:11-81); the result stays on the device
 * for the following integrate and is also returned in *dt (synchronising) if dt != NULL */
int eif_decide_dt(eif_ctx *ctx, double *dt);
int eif_set_dt(eif_ctx *ctx, double dt);
int eif_get_dt(eif_ctx *ctx, double *dt);
/* integrate (src/main.c:13-55): three RK stages with the particle fixed point;
 * substeps[3] (may be NULL) receives the sub-iteration count of each stage */
int eif_integrate(eif_ctx *ctx, int *substeps);
/* nsteps times { decide_dt; integrate; step += 1; time += dt } without host
 * synchronisation between steps (src/main.c:71-77). Each step's error flags are
 * read while the next step already runs: after an error the device state, the
 * step counter and the time include the step that followed the failing one
 * (at most one), and the counters always match the device state. */
int eif_advance(eif_ctx *ctx, int nsteps);
/* eif_advance(nsteps), then the state after the last step copied into host arrays in
 * the layouts of eif_pull_fluid and eif_pull_particles (any pointer may be NULL; n must
 * be the particle count). With the step graphs the fields are final once the last RK
 * stage's projection is done, so their copy to the host (page-locked arrays: one
 * streaming pass over the interconnect) runs beside that stage's particle
 * sub-iterations and update; the records follow when the step has ended. After an error
 * the arrays' contents are unspecified. No counterpart in the reference. */
int eif_advance_pull(eif_ctx *ctx, int nsteps, double *ux, double *uy, double *p, int n, double *records);
/* step counter and simulated time accumulated by eif_advance */
int eif_get_time(eif_ctx *ctx, int *step, double *time);
int eif_set_time(eif_ctx *ctx, int step, double time);

/* ---- batches of independent suspensions (no counterpart in the reference,
 * which runs one suspension per process) ----
 * A batch groups n existing contexts on one device (any grid sizes, particle
 * counts and precisions, each pushed as usual). eif_batch_advance moves every
 * suspension nsteps steps with one CUDA graph launch per step; each suspension
 * gets the same bits as with eif_advance on its own context, and its step
 * counter and time advance likewise. The batch does not own the contexts:
 * destroy it before them. On an error the message names the suspension
 * (eif_batch_last_error); that context's eif_last_error has the detail. */
typedef struct eif_batch eif_batch;
int eif_batch_create(eif_ctx *const *ctxs, int n, eif_batch **batch);
int eif_batch_advance(eif_batch *batch, int nsteps);
int eif_batch_size(const eif_batch *batch);
/* the stream the batch's step graphs are launched on (a cudaStream_t) */
void *eif_batch_stream(eif_batch *batch);
const char *eif_batch_last_error(const eif_batch *batch);
int eif_batch_destroy(eif_batch *batch);

/* ---- time-averaged statistics (src/statistics/collect.c:10-95) on the device ----
 * collect adds ux, ux^2 (faces 1..itot+1), uy, uy^2 (i = 0..itot+1) and the sharp
 * particle indicator phi (cells) of the current state to device accumulators and
 * counts the collect (asynchronous); reset zeroes them; pull copies them out in the
 * reference's layouts (include/arrays/statistics.h; ux-like (jtot+2) x (itot+1),
 * uy-like and phi (jtot+2) x (itot+2), halo rows zero) with the number of collects. */
int eif_stats_reset(eif_ctx *ctx);
int eif_stats_collect(eif_ctx *ctx);
int eif_stats_pull(eif_ctx *ctx, double *ux1, double *ux2, double *uy1, double *uy2, double *phi, int *num);

/* ---- asynchronous snapshots for checkpoints (the state save() writes,
 * src/save.c:109-122) ----
 * take: copies ux, uy, p and the particle records on the device, in order with the
 * steps, and starts their transfer to page-locked host memory on a stream of its own:
 * steps launched afterwards overlap with the transfer.
 * wait: waits for the transfer and writes the snapshot in the eif_push_fluid layouts
 * (any pointer may be NULL) and n records (n = the particle count at take), with the
 * step and time at take. A new take waits for the previous transfer. */
int eif_snapshot_take(eif_ctx *ctx);
int eif_snapshot_wait(eif_ctx *ctx, double *ux, double *uy, double *p, int n, double *records, int *step,
                      double *time);

/* Tile shapes of the stencil and block-Thomas kernels: the tuner times the
 * candidates (tiles of 32 columns by 4, 8 or 16 rows for the predictor and the
 * projection; 64, 128 or 256 threads per block of the block Thomas) once per grid
 * size and precision, before the first eif_integrate / eif_advance / batch capture,
 * and keeps the fastest. The shapes do not change any result. EIF_TUNE=0 in the
 * environment keeps the defaults (8, 8, 128). In the mixed form the predictor runs either
 * with its tiles staged by bulk tensor copies (double-buffered, TMA) or with plain loads,
 * whichever the tuner timed faster (EIF_NO_TMA=1 at context creation: plain loads only).
 * tiles[4]: predictor rows, projection rows, Thomas threads, flags (bit 0: tuned, bit 1:
 * predictor tiles staged by tensor copies, bit 2: the mixed predictor with plain loads
 * takes the x metrics as uniform values away from the wall cells, which it does when
 * their single-precision values are bitwise uniform there; EIF_NO_UNIFORM_X=1 at context
 * creation: always from the arrays). No counterpart in the reference. */
int eif_tiles(eif_ctx *ctx, int *tiles);

/* ---- discrete adjoint of the step (no counterpart in the reference) ----
 * Transposed linearisation of integrate (src/main.c:13-55) in the double-precision
 * form with dt held at the value eif_set_dt / eif_decide_dt left on the device.
 * EIF_ADJOINT_COUPLED: the whole step, particles moving: predictor, immersed-boundary
 * exchange (src/suspensions/exchange.c:13-88) and field update (update.c:36-59),
 * Poisson solve and projection, inertia integrals (inertia.c:9-70), Newton-Euler
 * increments and the recorded sub-iterations of the particle fixed point
 * (increment.c, main.c:32-52). Collision forces enter as constants: the adjoint is
 * that of contact-free motion, and backward fails (EIF_ERR_STATE) for a recorded step
 * in which a collision force was non-zero.
 * EIF_ADJOINT_FROZEN: the particle records are parameters of the step (no inertia,
 * collision, increment or update runs; the forcing acts with their rigid-body
 * velocities).
 *   begin(max_steps, mode)  allocates a tape of max_steps steps
 *   forward(record)    one step, recorded for backward when record != 0; step and
 *                      time advance as in eif_advance (coupled mode: the same bits as
 *                      eif_integrate)
 *   seed(ub, vb, pb)   cotangents of the fluid state after the last recorded step
 *                      (host arrays in the eif_push_fluid layouts; pb may be NULL).
 *                      The cotangents of halo rows and of the pressure's wall
 *                      columns are added to the entries they copy; the velocity
 *                      wall columns are no state (those of vb start the wall-velocity
 *                      gradient); the mean of pb over the cells is removed (the
 *                      pressure is determined up to a constant). Resets the
 *                      particle cotangents.
 *   seed_particles(n, rb)  particle cotangents (n records of EIF_NFIELDS doubles;
 *                      x, y, az, ux, uy, vz are read)
 *   backward()         transposed step of the last recorded step, which leaves the tape
 *   pull(ub, vb, pb)   current fluid cotangents, zero on halo rows and wall columns (the
 *                      pushed state's are recomputed on push); any pointer may be NULL
 *   pull_particles(n, rb)  current particle cotangents (other fields zero)
 *   wall_gradient(g)   d/d uy_wall[0..1] accumulated over the steps gone back through
 *   substeps(s, k)     sub-iteration counts of the three stages of recorded step s
 * FP64 form only (EIF_ERR_ARG otherwise). */
#define EIF_ADJOINT_COUPLED 0
#define EIF_ADJOINT_FROZEN 1
int eif_adjoint_begin(eif_ctx *ctx, int max_steps, int mode);
int eif_adjoint_forward(eif_ctx *ctx, int record);
int eif_adjoint_seed(eif_ctx *ctx, const double *ux_bar, const double *uy_bar, const double *p_bar);
int eif_adjoint_seed_particles(eif_ctx *ctx, int n, const double *records_bar);
int eif_adjoint_backward(eif_ctx *ctx);
int eif_adjoint_pull(eif_ctx *ctx, double *ux_bar, double *uy_bar, double *p_bar);
int eif_adjoint_pull_particles(eif_ctx *ctx, int n, double *records_bar);
int eif_adjoint_wall_gradient(eif_ctx *ctx, double *d_uy_wall);
int eif_adjoint_substeps(eif_ctx *ctx, int step, int *substeps);
int eif_adjoint_recorded(eif_ctx *ctx);
int eif_adjoint_end(eif_ctx *ctx);

/* ---- stage-level entry points, one per reference function ---- */
int eif_update_boundaries(eif_ctx *ctx);                              /* src/fluid/boundary_conditions.c:7-62 */
int eif_reset_particle_increments(eif_ctx *ctx);                      /* src/suspensions/reset.c:7-18 */
int eif_compute_inertia(eif_ctx *ctx, int cnstep);                    /* src/suspensions/inertia.c:96-102 */
int eif_update_velocity(eif_ctx *ctx, int rkstep);                    /* src/fluid/update_velocity.c:229-237 */
int eif_exchange_momentum(eif_ctx *ctx);                              /* src/suspensions/exchange.c:114-120 */
int eif_update_momentum_field(eif_ctx *ctx);                          /* src/suspensions/update.c:36-59 */
int eif_compute_potential(eif_ctx *ctx, int rkstep);                  /* src/fluid/compute_potential.c:48-138 */
int eif_correct_velocity(eif_ctx *ctx, int rkstep);                   /* src/fluid/correct_velocity.c:6-42 */
int eif_update_pressure(eif_ctx *ctx);                                /* src/fluid/update_pressure.c:7-24 */
int eif_compute_collision_force(eif_ctx *ctx, int cnstep);            /* src/suspensions/collision.c:306-367 */
int eif_increment_particles(eif_ctx *ctx, int rkstep, double *residual); /* src/suspensions/increment.c:66-72 */
int eif_update_particles(eif_ctx *ctx);                               /* src/suspensions/update.c:61-65 */

/* ---- time-step size without device allocation ----
 * No counterpart in the reference. Computes the same dt as eif_decide_dt
 * (param_decide_dt) directly from the caller's device arrays, for callers that
 * cannot let a library allocate device memory: applications that own all
 * device memory through their own pool, and time-critical loops in which a
 * cudaMalloc/cudaFree would synchronise the device. It allocates nothing; its
 * scratch is a fixed array in the library's static device memory (about
 * 128 KiB per GPU, held until the process exits), which limits itot to
 * EIF_NOALLOC_MAX_ITOT (larger grids return EIF_ERR_TOO_LARGE).
 *   ux, uy:     device arrays in the reference layouts (rows 0..jtot+1) with row
 *               pitches ux_pitch >= itot+1 and uy_pitch >= itot+2 (in doubles)
 *   safefactors: host array of 3 (advective, diffusive, particle)
 *   particles:  device array of n_particles * EIF_NFIELDS doubles (may be NULL if 0)
 *   dt:         device pointer that receives the result, written on `stream`
 *   stream:     a cudaStream_t (NULL: the legacy default stream)
 * A NaN or an infinity in the velocities read gives *dt = NaN (eif_decide_dt
 * returns EIF_ERR_NONFINITE for the same state; this entry point has no flag
 * output, and a NaN step fails every comparison a caller makes with it).
 * The first call on a device looks up the scratch address (do it before any
 * stream capture). All calls share the scratch array: calls that overlap on
 * the GPU race and must be serialised by the caller. */
#define EIF_NOALLOC_MAX_ITOT 16384
int eif_decide_dt_noalloc(const double *ux, int ux_pitch, const double *uy, int uy_pitch, int itot, int jtot,
                          double ly, double Re, const double *safefactors, const double *particles,
                          int n_particles, double *dt, void *stream);

/* ---- self-test of the integer-pipe double<->float conversions used by the
 * mixed-precision kernels (no counterpart in the reference) ----
 * Converts n values spread over the normal range (plus zeros and the range
 * limits) with both the library's conversions and the hardware ones and
 * returns how many results differ by more than the rounding of a tie (d2f) or
 * at all (f2d; the count includes the float pairs whose integer conversion to
 * double differs from the FP64 sum of the two parts). */
int eif_selftest_conversions(int device, int n, long long *d2f_mismatch, long long *f2d_mismatch);

/* ---- diagnostics: the reductions of the reference's logging (src/logging.c:40-172),
 * on the device, so that a log event needs no field pull ----
 * divergence: max |div u| and the sum of div u over the cells (check_divergence, :40-85)
 * momentum:   moms[0] = sum UX(i,j) DXC(i) dy over i = 1..itot+1, moms[1] = sum UY DXF dy
 *             over i = 1..itot (check_momentum, :87-128)
 * energy:     the same sums of UX^2/2 and UY^2/2 (check_energy, :130-172)
 * log_quantities: q[6] = {divmax, divsum, mom_x, mom_y, energy_x, energy_y}
 * Sums are accumulated in a fixed order (deterministic), not in the reference's loop
 * order: they agree with it to rounding (relative 1e-14 at 2048 x 4096). */
int eif_divergence(eif_ctx *ctx, double *divmax, double *divsum);
int eif_momentum(eif_ctx *ctx, double *moms);
int eif_energy(eif_ctx *ctx, double *energy);
int eif_log_quantities(eif_ctx *ctx, double *q);

/* ---- kernel timing (no counterpart in the reference, which only times the
 * whole run with MPI_Wtime, src/main.c:60-61,97-105) ----
 * When enabled, every kernel launch of the context is bracketed by CUDA events
 * on the context's stream and accumulated per kernel name. */
int eif_profile_enable(eif_ctx *ctx, int enable);
int eif_profile_reset(eif_ctx *ctx);
/* number of kernel names recorded so far (synchronises the stream) */
int eif_profile_count(eif_ctx *ctx, int *count);
/* name, launch count and total device time (ms) of entry k */
int eif_profile_get(eif_ctx *ctx, int k, char *name, int name_len, long long *launches, double *ms);
/* work counters of the context (synchronises the stream): counts[0] = particle
 * sub-iterations run since eif_create (every stage of every step, src/main.c:36-50);
 * counts[1] = box cells whose indicator geometry was evaluated and counts[2] = those
 * of them that ran the normal-foot iteration (src/ellipse.c:30-65), both counted
 * only while kernel timing is enabled. No counterpart in the reference. */
int eif_counters(eif_ctx *ctx, long long *counts);
/* indicator tasks (box rows) of the mixed form whose weights the first evaluation of an
 * RK stage took from the last evaluation of the previous sub-iteration loop instead of
 * computing them (the particle's single-precision geometry and boxes bitwise equal to
 * that evaluation's, so the weights are too); counted while kernel timing is enabled.
 * EIF_NO_MEMO=1 in the environment at eif_create turns the reuse off. No counterpart in
 * the reference. */
int eif_memo_count(eif_ctx *ctx, long long *tasks);

#ifdef __cplusplus
}
#endif

#endif /* EIF_H */
