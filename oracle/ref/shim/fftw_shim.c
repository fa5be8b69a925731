/*
 * DCT-II / DCT-III stand-in for FFTW's REDFT10 / REDFT01 (see fftw3.h).
 * TEST INFRASTRUCTURE ONLY.
 *
 * Method (Makhoul 1980, "A fast cosine transform in one and two dimensions"):
 *   DCT-II:  v_m = x_{2m}, v_{N-1-m} = x_{2m+1};  V = DFT(v);
 *            Y_k = 2 Re( exp(-i pi k / 2N) V_k ).
 *   DCT-III: W_n = exp(i pi n / 2N) (x_n - i x_{N-n})  (x_N = 0);  w = IDFT(W) (unscaled);
 *            Y_{2m} = Re w_m,  Y_{2m+1} = Re w_{N-1-m}.
 * The DFT is a recursive mixed-radix Cooley-Tukey transform over the prime
 * factors of N, with twiddles evaluated directly from cos/sin.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <complex.h>
#include "fftw3.h"

#if !defined(M_PI)
#define M_PI 3.14159265358979323846
#endif

struct eif_fftw_plan_ {
  int n;
  fftw_r2r_kind kind;
  double *in, *out;
  double _Complex *tw;    /* exp(-2 pi i k / n), k = 0..n-1 */
  double _Complex *rot;   /* exp(-i pi k / 2n), k = 0..n-1 */
  double _Complex *a, *b, *scratch;
};

static int smallest_factor(int n){
  for(int p = 2; p*p <= n; p++){
    if(n%p == 0) return p;
  }
  return n;
}

/* out[k] = sum_m in[m*stride] exp(sign 2 pi i m k / n), n divides N; tw is for N */
static void dft_rec(int n, const double _Complex *in, int stride, double _Complex *out,
                    const double _Complex *tw, int N, int sign, double _Complex *scratch){
  if(n == 1){
    out[0] = in[0];
    return;
  }
  const int p = smallest_factor(n);
  const int m = n/p;
  /* sub-transforms of the p decimated sequences, stored consecutively in out */
  for(int r = 0; r < p; r++){
    dft_rec(m, in+r*stride, stride*p, out+r*m, tw, N, sign, scratch+n);
  }
  const int step = N/n;
  for(int k = 0; k < n; k++){
    double _Complex acc = 0.;
    for(int r = 0; r < p; r++){
      int e = (int)(((long long)r*k)%n)*step;
      double _Complex w = sign < 0 ? tw[e] : conj(tw[e]);
      acc += out[r*m+(k%m)]*w;
    }
    scratch[k] = acc;
  }
  memcpy(out, scratch, sizeof(double _Complex)*(size_t)n);
}

fftw_plan fftw_plan_r2r_1d(int n, double *in, double *out, fftw_r2r_kind kind, unsigned flags){
  (void)flags;
  struct eif_fftw_plan_ *p = calloc(1, sizeof(*p));
  p->n = n;
  p->kind = kind;
  p->in = in;
  p->out = out;
  p->tw = malloc(sizeof(double _Complex)*(size_t)n);
  p->rot = malloc(sizeof(double _Complex)*(size_t)n);
  p->a = malloc(sizeof(double _Complex)*(size_t)n);
  p->b = malloc(sizeof(double _Complex)*(size_t)n);
  p->scratch = malloc(sizeof(double _Complex)*(size_t)(2*n+2));
  for(int k = 0; k < n; k++){
    double t = 2.*M_PI*(double)k/(double)n;
    p->tw[k] = cos(t)-I*sin(t);
    double h = M_PI*(double)k/(2.*(double)n);
    p->rot[k] = cos(h)-I*sin(h);
  }
  return p;
}

void fftw_execute(const fftw_plan p){
  const int n = p->n;
  double *x = p->in;
  double *y = p->out;
  if(p->kind == FFTW_REDFT10){
    for(int m = 0; 2*m < n; m++) p->a[m] = x[2*m];
    for(int m = 0; 2*m+1 < n; m++) p->a[n-1-m] = x[2*m+1];
    dft_rec(n, p->a, 1, p->b, p->tw, n, -1, p->scratch);
    for(int k = 0; k < n; k++) y[k] = 2.*creal(p->rot[k]*p->b[k]);
  }else{
    for(int k = 0; k < n; k++){
      double xr = x[k];
      double xi = k == 0 ? 0. : x[n-k];
      p->a[k] = conj(p->rot[k])*(xr-I*xi);
    }
    dft_rec(n, p->a, 1, p->b, p->tw, n, +1, p->scratch);
    for(int m = 0; 2*m < n; m++) y[2*m] = creal(p->b[m]);
    for(int m = 0; 2*m+1 < n; m++) y[2*m+1] = creal(p->b[n-1-m]);
  }
}

void fftw_destroy_plan(fftw_plan p){
  if(p == NULL) return;
  free(p->tw); free(p->rot); free(p->a); free(p->b); free(p->scratch);
  free(p);
}

void fftw_cleanup(void){}
