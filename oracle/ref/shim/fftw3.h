/*
 * Stand-in for the part of FFTW3 the reference solver calls: 1-D real-to-real
 * plans of kind REDFT10 (DCT-II) and REDFT01 (DCT-III), executed in place.
 * (src/fluid/compute_potential.c:31-35, 84-92, 120-128.)
 *
 * TEST INFRASTRUCTURE ONLY: used to compile the reference's own sources into
 * the CPU oracle library. Definitions (unnormalised, as in FFTW):
 *   REDFT10: Y_k = 2 sum_{n=0}^{N-1} x_n cos(pi (n+1/2) k / N)
 *   REDFT01: Y_k = x_0 + 2 sum_{n=1}^{N-1} x_n cos(pi n (k+1/2) / N)
 */
#if !defined(EIF_SHIM_FFTW3_H)
#define EIF_SHIM_FFTW3_H

typedef double _Complex fftw_complex;
typedef struct eif_fftw_plan_ *fftw_plan;
typedef int fftw_r2r_kind;

#define FFTW_REDFT10 ((fftw_r2r_kind)4)
#define FFTW_REDFT01 ((fftw_r2r_kind)5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_MEASURE (0U)
#define FFTW_PATIENT (1U << 5)

fftw_plan fftw_plan_r2r_1d(int n, double *in, double *out, fftw_r2r_kind kind, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);
void fftw_cleanup(void);

#endif
