/*
 * CPU restatement of the EllipsesInFlows time-step hot path ("port" oracle).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library and the CPU
 * baseline of the benchmark. Never linked into the product.
 *
 * It exposes the same entry points as include/eif.h with the prefix eifo_
 * instead of eif_, operating on host memory. Every function states the
 * reference function it follows (file:line in NaokiHori/EllipsesInFlows). The
 * arithmetic is written in the same order as the reference so that, with the
 * DCT of oracle/ref/shim/fftw_shim.c and FMA contraction disabled, results are
 * bit-identical to the reference built in oracle/_ref/; tests pin this.
 *
 * Threads: loops without cross-iteration reductions run under OpenMP when the
 * library is built with -fopenmp (eifo_set_threads). Every per-particle sum is
 * still accumulated serially in the reference's order, so results do not
 * depend on the thread count.
 */
#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "eif.h"
#include "fftw3.h"

#ifndef M_PI
#define M_PI 3.1415926535897932
#endif

#define NEXTRA 3      /* src/suspensions/auxiliary.c:8 */
#define BETA 2.       /* src/suspensions/auxiliary.c:49 */

typedef struct eifo_ctx {
  eif_config_t cfg;
  int itot, jtot;
  double lx, ly, dx, dy;
  double *xf, *xc, *dxf, *dxc, *yf, *yc;  /* 0-based copies of XF(1..), XC(0..), DXF(1..), DXC(1..), YF(1..), YC(1..) */
  double alpha[3], beta[3], gamma[3];
  double dt, time;
  int step;
  double *ux, *uy, *p, *psi;
  double *sxa, *sxb, *sxg, *sya, *syb, *syg;
  double *dux, *duy;
  double *q;                               /* Poisson work array, x-contiguous rows */
  int np;
  double *P[EIF_NFIELDS];                  /* SoA particle fields */
  double **wbox;                           /* exchange: per-particle box weights (scratch) */
  int nthreads;
  char err[256];
} eifo_ctx;

/* ---- index helpers: the reference layouts of include/arrays/fluid.h ---- */
#define UX(I, J) (c->ux[(size_t)(J)*(c->itot+1)+((I)-1)])
#define UY(I, J) (c->uy[(size_t)(J)*(c->itot+2)+(I)])
#define PP(I, J) (c->p[(size_t)(J)*(c->itot+2)+(I)])
#define PSI(I, J) (c->psi[(size_t)(J)*(c->itot+2)+(I)])
#define DUX(I, J) (c->dux[(size_t)(J)*(c->itot+2)+(I)])
#define DUY(I, J) (c->duy[(size_t)(J)*(c->itot+2)+(I)])
#define SXA(I, J) (c->sxa[(size_t)((J)-1)*(c->itot-1)+((I)-2)])
#define SXB(I, J) (c->sxb[(size_t)((J)-1)*(c->itot-1)+((I)-2)])
#define SXG(I, J) (c->sxg[(size_t)((J)-1)*(c->itot-1)+((I)-2)])
#define SYA(I, J) (c->sya[(size_t)((J)-1)*(c->itot)+((I)-1)])
#define SYB(I, J) (c->syb[(size_t)((J)-1)*(c->itot)+((I)-1)])
#define SYG(I, J) (c->syg[(size_t)((J)-1)*(c->itot)+((I)-1)])
#define XF(I) (c->xf[(I)-1])
#define XC(I) (c->xc[(I)])
#define DXF(I) (c->dxf[(I)-1])
#define DXC(I) (c->dxc[(I)-1])
#define YF(J) (c->yf[(J)-1])
#define YC(J) (c->yc[(J)-1])
#define PF(F, N) (c->P[EIF_P_##F][(N)])

static int nthreads_of(const eifo_ctx *c){ return c->nthreads > 0 ? c->nthreads : 1; }

/* ------------------------------------------------------------------------- */
/* grid and coefficients: set_coordinate, set_rk_coefs (src/param/init.c:105-191) */
static void setup_grid(eifo_ctx *c){
  const int itot = c->itot, jtot = c->jtot;
  c->xf = calloc(itot+1, sizeof(double));
  c->xc = calloc(itot+2, sizeof(double));
  c->dxf = calloc(itot, sizeof(double));
  c->dxc = calloc(itot+1, sizeof(double));
  c->yf = calloc(jtot+1, sizeof(double));
  c->yc = calloc(jtot, sizeof(double));
  const double dx = c->lx/itot;
  c->dx = dx;
  for(int i = 1; i <= itot+1; i++) XF(i) = 1.*(i-1)*dx;
  XF(1) = 0.;
  XF(itot+1) = c->lx;
  for(int i = 1; i <= itot; i++) DXF(i) = XF(i+1)-XF(i);
  XC(0) = XF(1);
  for(int i = 1; i <= itot; i++) XC(i) = 0.5*(XF(i)+XF(i+1));
  XC(itot+1) = XF(itot+1);
  for(int i = 1; i <= itot+1; i++) DXC(i) = XC(i)-XC(i-1);
  const double dy = c->ly/jtot;
  c->dy = dy;
  for(int j = 1; j <= jtot+1; j++) YF(j) = 0.+1.*(j-1)*dy;
  for(int j = 1; j <= jtot; j++) YC(j) = 0.+0.5*(2*j-1)*dy;
  const double al[3] = {32./60., 25./60., 45./60.};
  const double be[3] = {0./60., -17./60., -25./60.};
  for(int k = 0; k < 3; k++){
    c->alpha[k] = al[k];
    c->beta[k] = be[k];
    c->gamma[k] = al[k]+be[k];
  }
}

/* ------------------------------------------------------------------------- */
/* boundary and halo values (src/fluid/boundary_conditions.c:7-62) */
static void bc_ux(eifo_ctx *c, double *ux_){
  const int itot = c->itot, jtot = c->jtot;
  double *save = c->ux;
  c->ux = ux_;
  for(int i = 2; i <= itot; i++){
    UX(i, 0) = UX(i, jtot);
    UX(i, jtot+1) = UX(i, 1);
  }
  for(int j = 0; j <= jtot+1; j++){
    UX(1, j) = 0.;
    UX(itot+1, j) = 0.;
  }
  c->ux = save;
}

static void bc_uy(eifo_ctx *c, double *uy_){
  const int itot = c->itot, jtot = c->jtot;
  double *save = c->uy;
  c->uy = uy_;
  for(int i = 1; i <= itot; i++){
    UY(i, 0) = UY(i, jtot);
    UY(i, jtot+1) = UY(i, 1);
  }
  for(int j = 0; j <= jtot+1; j++){
    UY(0, j) = c->cfg.uy_wall[0];
    UY(itot+1, j) = c->cfg.uy_wall[1];
  }
  c->uy = save;
}

/* p-like arrays: p, psi, dux, duy share the layout */
static void bc_p(eifo_ctx *c, double *a){
  const int itot = c->itot, jtot = c->jtot;
  const size_t ld = (size_t)itot+2;
  for(int i = 1; i <= itot; i++){
    a[0*ld+i] = a[(size_t)jtot*ld+i];
    a[(size_t)(jtot+1)*ld+i] = a[1*ld+i];
  }
  for(int j = 0; j <= jtot+1; j++){
    a[(size_t)j*ld+0] = a[(size_t)j*ld+1];
    a[(size_t)j*ld+itot+1] = a[(size_t)j*ld+itot];
  }
}

int eifo_update_boundaries(eifo_ctx *c){
  bc_ux(c, c->ux);
  bc_uy(c, c->uy);
  bc_p(c, c->p);
  return EIF_OK;
}

/* ------------------------------------------------------------------------- */
/* predictor (src/fluid/update_velocity.c:9-237) */
static void src_ux(eifo_ctx *c){
  const int itot = c->itot, jtot = c->jtot;
  const double dy = c->dy, Re = c->cfg.Re;
  memcpy(c->sxb, c->sxa, sizeof(double)*(size_t)(itot-1)*jtot);
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int i = 2; i <= itot; i++){
      const double duxdx_xm = (-UX(i-1, j)+UX(i, j))/DXF(i-1);
      const double duxdx_xp = (-UX(i, j)+UX(i+1, j))/DXF(i);
      const double duxdy_ym = (-UX(i, j-1)+UX(i, j))/dy;
      const double duxdy_yp = (-UX(i, j)+UX(i, j+1))/dy;
      const double c_xm = DXF(i-1)/(2.*DXC(i));
      const double c_xp = DXF(i)/(2.*DXC(i));
      /* advection by ux, by uy; diffusion in x, y; pressure gradient */
      const double ux_xm = 0.5*UX(i-1, j)+0.5*UX(i, j);
      const double ux_xp = 0.5*UX(i, j)+0.5*UX(i+1, j);
      const double adv1 = -c_xm*ux_xm*duxdx_xm-c_xp*ux_xp*duxdx_xp;
      const double uy_ym = c_xm*UY(i-1, j)+c_xp*UY(i, j);
      const double uy_yp = c_xm*UY(i-1, j+1)+c_xp*UY(i, j+1);
      const double adv2 = -0.5*uy_ym*duxdy_ym-0.5*uy_yp*duxdy_yp;
      const double dif1 = 1./Re*(duxdx_xp-duxdx_xm)/DXC(i);
      const double dif2 = 1./Re*(duxdy_yp-duxdy_ym)/dy;
      const double pre = -(PP(i, j)-PP(i-1, j))/DXC(i);
      SXA(i, j) = +(adv1+adv2)+(dif1+dif2);
      SXG(i, j) = pre;
    }
  }
}

static void src_uy(eifo_ctx *c){
  const int itot = c->itot, jtot = c->jtot;
  const double dy = c->dy, Re = c->cfg.Re, ext = c->cfg.extfrcy;
  memcpy(c->syb, c->sya, sizeof(double)*(size_t)itot*jtot);
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int i = 1; i <= itot; i++){
      const double duydx_xm = (-UY(i-1, j)+UY(i, j))/DXC(i);
      const double duydx_xp = (-UY(i, j)+UY(i+1, j))/DXC(i+1);
      const double duydy_ym = (-UY(i, j-1)+UY(i, j))/dy;
      const double duydy_yp = (-UY(i, j)+UY(i, j+1))/dy;
      const double c_xm = DXC(i)/(2.*DXF(i));
      const double c_xp = DXC(i+1)/(2.*DXF(i));
      const double ux_xm = 0.5*UX(i, j-1)+0.5*UX(i, j);
      const double ux_xp = 0.5*UX(i+1, j-1)+0.5*UX(i+1, j);
      const double adv1 = -c_xm*ux_xm*duydx_xm-c_xp*ux_xp*duydx_xp;
      const double uy_ym = 0.5*UY(i, j-1)+0.5*UY(i, j);
      const double uy_yp = 0.5*UY(i, j)+0.5*UY(i, j+1);
      const double adv2 = -0.5*uy_ym*duydy_ym-0.5*uy_yp*duydy_yp;
      const double dif1 = 1./Re*(duydx_xp-duydx_xm)/DXF(i);
      const double dif2 = 1./Re*(duydy_yp-duydy_ym)/dy;
      const double pre = -(PP(i, j)-PP(i, j-1))/dy;
      SYA(i, j) = +(adv1+adv2)+(dif1+dif2)+ext;
      SYG(i, j) = pre;
    }
  }
}

int eifo_update_velocity(eifo_ctx *c, int rk){
  if(rk < 0 || rk > 2) return EIF_ERR_ARG;
  const int itot = c->itot, jtot = c->jtot;
  const double a = c->alpha[rk], b = c->beta[rk], g = c->gamma[rk], dt = c->dt;
  src_ux(c);
  src_uy(c);
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int i = 2; i <= itot; i++){
      UX(i, j) += +a*dt*SXA(i, j)+b*dt*SXB(i, j)+g*dt*SXG(i, j);
    }
  }
  bc_ux(c, c->ux);
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int i = 1; i <= itot; i++){
      UY(i, j) += +a*dt*SYA(i, j)+b*dt*SYB(i, j)+g*dt*SYG(i, j);
    }
  }
  bc_uy(c, c->uy);
  return EIF_OK;
}

/* ------------------------------------------------------------------------- */
/* tridiagonal solvers (src/tdm.c:37-108) */

/* Thomas sweep on n rows with constant sub/centre diagonals l, cc; overwrites
 * u and q (src/tdm.c:37-59, where l[i] and c[i] hold these constants) */
static void thomas(int n, double l, double cc, double *u, double *q){
  u[0] = u[0]/cc;
  q[0] = q[0]/cc;
  for(int i = 1; i <= n-1; i++){
    double val = cc-l*u[i-1];
    if(fabs(val) < DBL_EPSILON){
      u[i] = 0.;
      q[i] = 0.;
    }else{
      val = 1./val;
      u[i] = val*u[i];
      q[i] = val*(q[i]-l*q[i-1]);
    }
  }
  for(int i = n-2; i >= 0; i--) q[i] -= u[i]*q[i+1];
}

/*
 * Cyclic system with constant diagonals (l, cc, u) of size n, solved as in
 * src/tdm.c:64-108: two Thomas solves on the leading n-1 rows (data and
 * correction vector), then the last unknown from the last row.
 * work: 3*(n-1) doubles.
 */
static void cyclic_constant(int n, double l, double cc, double u, double *q, double *work){
  double *u0 = work, *u1 = work+(n-1), *q1 = work+2*(n-1);
  for(int i = 0; i < n-1; i++){
    u0[i] = u;
    u1[i] = u;
    q1[i] = i == 0 ? -l : i == n-2 ? -u : 0.;
  }
  thomas(n-1, l, cc, u0, q);
  thomas(n-1, l, cc, u1, q1);
  const double num = q[n-1]-u*q[0]-l*q[n-2];
  const double den = cc+u*q1[0]+l*q1[n-2];
  q[n-1] = fabs(den) < DBL_EPSILON ? 0. : num/den;
  for(int i = 0; i <= n-2; i++) q[i] = q[i]+q[n-1]*q1[i];
}

/* ------------------------------------------------------------------------- */
/* scalar potential (src/fluid/compute_potential.c:48-138), one rank: the
 * x-aligned buffer QX(i,j) is transposed to y-aligned columns in memory */
int eifo_compute_potential(eifo_ctx *c, int rk){
  if(rk < 0 || rk > 2) return EIF_ERR_ARG;
  const int itot = c->itot, jtot = c->jtot;
  const double dx = c->dx, dy = c->dy;
  const double g = c->gamma[rk], dt = c->dt;
  double *q = c->q;
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int i = 1; i <= itot; i++){
      q[(size_t)(j-1)*itot+(i-1)] = 1./(g*dt)*(+(UX(i+1, j)-UX(i, j))/dx+(UY(i, j+1)-UY(i, j))/dy);
    }
  }
  /* DCT-II along x, row by row */
  #pragma omp parallel num_threads(nthreads_of(c))
  {
    double *r = malloc(sizeof(double)*(size_t)itot);
    fftw_plan plan = fftw_plan_r2r_1d(itot, r, r, FFTW_REDFT10, FFTW_PATIENT);
    #pragma omp for schedule(static)
    for(int j = 0; j < jtot; j++){
      memcpy(r, q+(size_t)j*itot, sizeof(double)*(size_t)itot);
      fftw_execute(plan);
      memcpy(q+(size_t)j*itot, r, sizeof(double)*(size_t)itot);
    }
    fftw_destroy_plan(plan);
    free(r);
  }
  /* per wavenumber: cyclic tridiagonal solve along y */
  const double l = 1./dy/dy;
  #pragma omp parallel num_threads(nthreads_of(c))
  {
    double *col = malloc(sizeof(double)*(size_t)jtot);
    double *work = malloc(sizeof(double)*(size_t)3*jtot);
    #pragma omp for schedule(static)
    for(int i = 1; i <= itot; i++){
      const double s = sin(M_PI*(i-1)/(2.*itot));
      const double eigenvalue = -4./(dx*dx)*(s*s);
      const double cc = -l-l+eigenvalue;
      for(int j = 0; j < jtot; j++) col[j] = q[(size_t)j*itot+(i-1)];
      cyclic_constant(jtot, l, cc, l, col, work);
      for(int j = 0; j < jtot; j++) q[(size_t)j*itot+(i-1)] = col[j];
    }
    free(col);
    free(work);
  }
  /* DCT-III along x and normalisation */
  #pragma omp parallel num_threads(nthreads_of(c))
  {
    double *r = malloc(sizeof(double)*(size_t)itot);
    fftw_plan plan = fftw_plan_r2r_1d(itot, r, r, FFTW_REDFT01, FFTW_PATIENT);
    #pragma omp for schedule(static)
    for(int j = 1; j <= jtot; j++){
      memcpy(r, q+(size_t)(j-1)*itot, sizeof(double)*(size_t)itot);
      fftw_execute(plan);
      for(int i = 1; i <= itot; i++) PSI(i, j) = r[i-1]/(2.*itot);
    }
    fftw_destroy_plan(plan);
    free(r);
  }
  bc_p(c, c->psi);
  return EIF_OK;
}

/* projection (src/fluid/correct_velocity.c:6-42) */
int eifo_correct_velocity(eifo_ctx *c, int rk){
  if(rk < 0 || rk > 2) return EIF_ERR_ARG;
  const int itot = c->itot, jtot = c->jtot;
  const double g = c->gamma[rk], dt = c->dt, dy = c->dy;
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int i = 2; i <= itot; i++){
      const double dxi = 1./DXC(i);
      UX(i, j) -= g*dt*(PSI(i, j)-PSI(i-1, j))*dxi;
    }
  }
  bc_ux(c, c->ux);
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int i = 1; i <= itot; i++){
      UY(i, j) -= g*dt*(PSI(i, j)-PSI(i, j-1))/dy;
    }
  }
  bc_uy(c, c->uy);
  return EIF_OK;
}

/* src/fluid/update_pressure.c:7-24 */
int eifo_update_pressure(eifo_ctx *c){
  const int itot = c->itot, jtot = c->jtot;
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int i = 1; i <= itot; i++) PP(i, j) += PSI(i, j);
  }
  bc_p(c, c->p);
  return EIF_OK;
}

/* ------------------------------------------------------------------------- */
/* ellipse geometry (src/ellipse.c:7-65, src/suspensions/auxiliary.c:11-75) */
static double ell_ex(double a, double b, double t){ return a*(1.-pow(b/a, 2.))*pow(cos(t), 3.); }
static double ell_ey(double a, double b, double t){ return b*(1.-pow(a/b, 2.))*pow(sin(t), 3.); }

static double ell_curvature(double a, double b, double t){
  const double ct = cos(t), st = sin(t);
  const double ct2 = pow(ct, 2.), st2 = pow(st, 2.);
  const double a2 = pow(a, 2.), b2 = pow(b, 2.);
  return a*b*(ct2+st2)/pow(+a2*st2+b2*ct2, 1.5);
}

/* parameter t of the foot of the normal from (x_, y_) (src/ellipse.c:30-65) */
double eifo_find_normal_t(double a, double b, double x_, double y_){
  const double px = fabs(x_), py = fabs(y_);
  double t = 0.25*M_PI;
  for(int n = 0; ; n++){
    const double x = a*cos(t);
    const double y = b*sin(t);
    const double ex = ell_ex(a, b, t);
    const double ey = ell_ey(a, b, t);
    const double rx = x-ex, ry = y-ey;
    const double qx = px-ex, qy = py-ey;
    const double r = sqrt(pow(ry, 2.)+pow(rx, 2.));
    const double q = sqrt(pow(qy, 2.)+pow(qx, 2.));
    const double dc = r*asin((rx*qy-ry*qx)/(r*q));
    const double dt = dc/sqrt(a*a+b*b-x*x-y*y);
    t += dt;
    t = fmin(0.5*M_PI, t);
    t = fmax(0., t);
    if(fabs(dt) < 1.e-8) break;
    if(n > 100) break;
  }
  if(x_ < 0.) t = M_PI-t;
  if(y_ < 0.) t = -t;
  return t;
}

/* signed distance in units of the grid size, positive inside (auxiliary.c:19-47) */
static double signed_dist(double h, double pa, double pb, double px, double py, double paz, double x, double y){
  const double ddx = x-px, ddy = y-py;
  const double cz = cos(-paz), sz = sin(-paz);
  const double x_ = cz*ddx-sz*ddy;
  const double y_ = sz*ddx+cz*ddy;
  const double f0 = 1.-(x_/pa)*(x_/pa)-(y_/pb)*(y_/pb);
  const double sign = f0 > 0. ? +1. : -1.;
  const double t = eifo_find_normal_t(pa, pb, x_, y_);
  const double ex = pa*cos(t)-x_, ey = pb*sin(t)-y_;
  return sign*sqrt(ex*ex+ey*ey)/h;
}

double eifo_s_weight(double h, double pa, double pb, double px, double py, double paz, double x, double y){
  const double d = signed_dist(h, pa, pb, px, py, paz, x, y);
  const double th = tanh(BETA*d);
  return 0.5*BETA*(1.-th*th);
}

double eifo_v_weight(double h, double pa, double pb, double px, double py, double paz, double x, double y){
  const double d = signed_dist(h, pa, pb, px, py, paz, x, y);
  return 0.5*(1.+tanh(BETA*d));
}

/* loop bounds of a particle box (auxiliary.c:11-17) */
static void loop_size(int lb, int ub, double h, double r, double gc, int *mn, int *mx){
  *mn = (int)(floor((gc-r)/h)-NEXTRA);
  *mx = (int)(ceil((gc+r)/h)+NEXTRA);
  if(*mn < lb) *mn = lb;
  if(*mx > ub) *mx = ub;
}

static double mass_of(double den, double a, double b){ return den*(M_PI*a*b); }
static double moi_of(double den, double a, double b){ return 0.25*mass_of(den, a, b)*(pow(a, 2.)+pow(b, 2.)); }

/* ------------------------------------------------------------------------- */
/* volume-weighted integrals (src/suspensions/inertia.c:9-102) */
int eifo_compute_inertia(eifo_ctx *c, int cn){
  if(cn < 0 || cn > 1) return EIF_ERR_ARG;
  const int itot = c->itot, jtot = c->jtot;
  const double ly = c->ly, dx = c->dx, dy = c->dy;
  const double h = fmin(dx, dy);
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(dynamic, 1)
  for(int n = 0; n < c->np; n++){
    const double pden = PF(DEN, n), pa = PF(A, n), pb = PF(B, n);
    const double px = PF(X, n)+PF(DX, n);
    const double py = PF(Y, n)+PF(DY, n);
    const double paz = PF(AZ, n)+PF(DAZ, n);
    const double pm = mass_of(pden, pa, pb);
    const double pim = moi_of(pden, pa, pb);
    double iux = 0., iuy = 0., ivz = 0.;
    for(int per = -1; per <= 1; per++){
      const double py_ = py+ly*per;
      int imin, imax, jmin, jmax;
      loop_size(1, itot, dx, fmax(pa, pb), px, &imin, &imax);
      loop_size(1, jtot, dy, fmax(pa, pb), py_-YF(1), &jmin, &jmax);
      for(int j = jmin; j <= jmax; j++){
        const double y = YC(j);
        for(int i = imin; i <= imax; i++){
          const double x = XC(i);
          const double w = eifo_v_weight(h, pa, pb, px, py_, paz, x, y);
          const double valx = w*0.5*(UX(i, j)+UX(i+1, j))*(dx*dy);
          const double valy = w*0.5*(UY(i, j)+UY(i, j+1))*(dx*dy);
          iux += valx/pm;
          ivz += -(y-py_)*valx/pim;
          iuy += valy/pm;
          ivz += +(x-px)*valy/pim;
        }
      }
    }
    c->P[EIF_P_IUX0+cn][n] = iux;
    c->P[EIF_P_IUY0+cn][n] = iuy;
    c->P[EIF_P_IVZ0+cn][n] = ivz;
  }
  return EIF_OK;
}

/* ------------------------------------------------------------------------- */
/* momentum exchange (src/suspensions/exchange.c:13-120) in two passes:
 * (1) per particle, in parallel: weights and force/torque sums, each in the
 *     reference's cell order; (2) per row, in parallel: the field response,
 *     accumulated per cell in particle order. */
int eifo_exchange_momentum(eifo_ctx *c){
  const int itot = c->itot, jtot = c->jtot;
  const double ly = c->ly, dx = c->dx, dy = c->dy, dt = c->dt;
  const double h = fmin(dx, dy);
  const size_t nfield = (size_t)(itot+2)*(jtot+2);
  memset(c->dux, 0, sizeof(double)*nfield);
  memset(c->duy, 0, sizeof(double)*nfield);
  int (*box)[3][4] = calloc(c->np > 0 ? c->np : 1, sizeof(*box));
  c->wbox = calloc(c->np > 0 ? c->np : 1, sizeof(double *));
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(dynamic, 1)
  for(int n = 0; n < c->np; n++){
    const double pden = PF(DEN, n), pa = PF(A, n), pb = PF(B, n);
    const double pm = mass_of(pden, pa, pb);
    const double pim = moi_of(pden, pa, pb);
    const double px = PF(X, n), py = PF(Y, n), paz = PF(AZ, n);
    const double pux = PF(UX, n), puy = PF(UY, n), pvz = PF(VZ, n);
    double fux = 0., fuy = 0., tvz = 0.;
    size_t total = 0;
    for(int per = -1; per <= 1; per++){
      int *bx = box[n][per+1];
      loop_size(1, itot, dx, fmax(pa, pb), px, &bx[0], &bx[1]);
      loop_size(1, jtot, dy, fmax(pa, pb), py+ly*per-YF(1), &bx[2], &bx[3]);
      if(bx[1] >= bx[0] && bx[3] >= bx[2]) total += (size_t)(bx[1]-bx[0]+1)*(bx[3]-bx[2]+1);
    }
    double *wb = malloc(sizeof(double)*2*(total > 0 ? total : 1));
    c->wbox[n] = wb;
    size_t k = 0;
    for(int per = -1; per <= 1; per++){
      const double py_ = py+ly*per;
      const int *bx = box[n][per+1];
      for(int j = bx[2]; j <= bx[3]; j++){
        const double y = YC(j);
        for(int i = bx[0]; i <= bx[1]; i++){
          const double x = XC(i);
          const double w = eifo_s_weight(h, pa, pb, px, py_, paz, x, y);
          const double ux_p = pux-pvz*(y-py_);
          const double uy_p = puy+pvz*(x-px);
          const double ux_f = 0.5*(UX(i, j)+UX(i+1, j));
          const double uy_f = 0.5*(UY(i, j)+UY(i, j+1));
          const double fx = w*(ux_p-ux_f)/dt;
          const double fy = w*(uy_p-uy_f)/dt;
          wb[2*k+0] = fx*dt;
          wb[2*k+1] = fy*dt;
          k++;
          fux -= +(fx*dx*dy)/pm;
          tvz -= -(y-py_)*(fx*dx*dy)/pim;
          fuy -= +(fy*dx*dy)/pm;
          tvz -= +(x-px)*(fy*dx*dy)/pim;
        }
      }
    }
    PF(FUX, n) = fux;
    PF(FUY, n) = fuy;
    PF(TVZ, n) = tvz;
  }
  /* field response: per cell, contributions in (particle, image) order */
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int n = 0; n < c->np; n++){
      size_t base = 0;
      for(int per = -1; per <= 1; per++){
        const int *bx = box[n][per+1];
        const int wdt = bx[1]-bx[0]+1;
        const int hgt = bx[3]-bx[2]+1;
        if(wdt > 0 && hgt > 0){
          if(j >= bx[2] && j <= bx[3]){
            const double *wb = c->wbox[n]+2*(base+(size_t)(j-bx[2])*wdt);
            for(int i = bx[0]; i <= bx[1]; i++){
              DUX(i, j) += wb[2*(i-bx[0])+0];
              DUY(i, j) += wb[2*(i-bx[0])+1];
            }
          }
          base += (size_t)wdt*hgt;
        }
      }
    }
  }
  for(int n = 0; n < c->np; n++) free(c->wbox[n]);
  free(c->wbox);
  c->wbox = NULL;
  free(box);
  bc_p(c, c->dux);
  bc_p(c, c->duy);
  return EIF_OK;
}

/* src/suspensions/update.c:36-59 */
int eifo_update_momentum_field(eifo_ctx *c){
  const int itot = c->itot, jtot = c->jtot;
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int i = 2; i <= itot; i++) UX(i, j) += 0.5*(DUX(i-1, j)+DUX(i, j));
  }
  bc_ux(c, c->ux);
  #pragma omp parallel for num_threads(nthreads_of(c)) schedule(static)
  for(int j = 1; j <= jtot; j++){
    for(int i = 1; i <= itot; i++) UY(i, j) += 0.5*(DUY(i, j-1)+DUY(i, j));
  }
  bc_uy(c, c->uy);
  return EIF_OK;
}

/* ------------------------------------------------------------------------- */
/* collisions (src/suspensions/collision.c:63-367) */
typedef struct { double a, b, x, y, angle; } ell_t;
typedef struct { double x, y, r; } circ_t;

/* centre of curvature of e at the foot of the normal from (x, y) (collision.c:75-109) */
static void evolute(const ell_t *e, double x, double y, double *ex, double *ey, double *ix, double *iy, double *r){
  const double x__ = x-e->x, y__ = y-e->y;
  double x_ = cos(-e->angle)*x__-sin(-e->angle)*y__;
  double y_ = sin(-e->angle)*x__+cos(-e->angle)*y__;
  const double t = eifo_find_normal_t(e->a, e->b, x_, y_);
  *r = 1./fmax(ell_curvature(e->a, e->b, t), DBL_EPSILON);
  x_ = ell_ex(e->a, e->b, t);
  y_ = ell_ey(e->a, e->b, t);
  *ex = cos(+e->angle)*x_-sin(+e->angle)*y_;
  *ey = sin(+e->angle)*x_+cos(+e->angle)*y_;
  *ex = *ex+e->x;
  *ey = *ey+e->y;
  x_ = e->a*cos(t);
  y_ = e->b*sin(t);
  *ix = cos(+e->angle)*x_-sin(+e->angle)*y_;
  *iy = sin(+e->angle)*x_+cos(+e->angle)*y_;
}

#define EIF_FIT_MAX_ITER 10000

/* equivalent circles of two ellipses (collision.c:111-135); returns 0 or EIF_ERR_NOCONV */
static int fit_pair(const ell_t *e0, const ell_t *e1, circ_t *c0, circ_t *c1, double *ix0, double *iy0, double *ix1, double *iy1){
  c0->x = e0->x; c0->y = e0->y;
  c1->x = e1->x; c1->y = e1->y;
  for(int n = 0; n < EIF_FIT_MAX_ITER; n++){
    double c0x, c0y, c1x, c1y;
    evolute(e0, c1->x, c1->y, &c0x, &c0y, ix0, iy0, &c0->r);
    evolute(e1, c0->x, c0->y, &c1x, &c1y, ix1, iy1, &c1->r);
    const double d0x = c0x-c0->x, d0y = c0y-c0->y;
    const double d1x = c1x-c1->x, d1y = c1y-c1->y;
    c0->x += d0x; c0->y += d0y;
    c1->x += d1x; c1->y += d1y;
    if(fmax(fmax(fabs(d0x), fabs(d0y)), fmax(fabs(d1x), fabs(d1y))) < 1.e-8) return 0;
  }
  return EIF_ERR_NOCONV;
}

/* equivalent circle against a wall (collision.c:137-154) */
static int fit_wall(const ell_t *e, double wallx, circ_t *cc, double *ix, double *iy){
  cc->x = e->x; cc->y = e->y;
  for(int n = 0; n < EIF_FIT_MAX_ITER; n++){
    double cx, cy;
    evolute(e, 2.*wallx-cc->x, cc->y, &cx, &cy, ix, iy, &cc->r);
    const double dcx = cx-cc->x, dcy = cy-cc->y;
    cc->x += dcx; cc->y += dcy;
    if(fmax(fabs(dcx), fabs(dcy)) < 1.e-8) return 0;
  }
  return EIF_ERR_NOCONV;
}

static double harmonic(double v0, double v1){ return 1./(0.5*(1./v0+1./v1)); }

/* pair n0 < n1 (collision.c:156-247); adds into the cn slot of both */
static int collide_pair(eifo_ctx *c, int cn, int n0, int n1){
  const double ly = c->ly;
  const double p0y = PF(Y, n0)+PF(DY, n0);
  const double p1y = PF(Y, n1)+PF(DY, n1);
  double yoff = 0., minval = DBL_MAX;
  for(int per = -1; per <= 1; per++){
    const double v = fabs((p1y+ly*per)-p0y);
    if(v < minval){ minval = v; yoff = ly*per; }
  }
  {
    const double x0 = PF(X, n0)+PF(DX, n0), y0 = PF(Y, n0)+PF(DY, n0);
    const double r0 = fmax(PF(A, n0), PF(B, n0));
    const double x1 = PF(X, n1)+PF(DX, n1), y1 = PF(Y, n1)+PF(DY, n1)+yoff;
    const double r1 = fmax(PF(A, n1), PF(B, n1));
    const double norm = fmax(hypot(x1-x0, y1-y0), DBL_EPSILON);
    if(r0+r1-norm < 0.) return 0;
  }
  const ell_t e0 = {PF(A, n0), PF(B, n0), PF(X, n0)+PF(DX, n0), PF(Y, n0)+PF(DY, n0), PF(AZ, n0)};
  const ell_t e1 = {PF(A, n1), PF(B, n1), PF(X, n1)+PF(DX, n1), PF(Y, n1)+PF(DY, n1)+yoff, PF(AZ, n1)};
  circ_t c0, c1;
  double ix0, iy0, ix1, iy1;
  const int rc = fit_pair(&e0, &e1, &c0, &c1, &ix0, &iy0, &ix1, &iy1);
  const double m0 = mass_of(PF(DEN, n0), PF(A, n0), PF(B, n0));
  const double m1 = mass_of(PF(DEN, n1), PF(A, n1), PF(B, n1));
  const double i0 = moi_of(PF(DEN, n0), PF(A, n0), PF(B, n0));
  const double i1 = moi_of(PF(DEN, n1), PF(A, n1), PF(B, n1));
  const double mass = harmonic(m0, m1);
  const double reft = pow(harmonic(sqrt(PF(A, n0)*PF(B, n0)), sqrt(PF(A, n1)*PF(B, n1))), 1.5);
  const double k = mass*pow(M_PI, 2.)/pow(reft, 2.);
  double nx = c1.x-c0.x, ny = c1.y-c0.y;
  const double norm = fmax(hypot(nx, ny), DBL_EPSILON);
  nx /= norm;
  ny /= norm;
  const double overlap = c0.r+c1.r-norm;
  if(overlap > 0.){
    const double cfx = k*overlap*nx, cfy = k*overlap*ny;
    c->P[EIF_P_CFX0+cn][n0] += 1./m0*(-cfx);
    c->P[EIF_P_CFX0+cn][n1] += 1./m1*(+cfx);
    c->P[EIF_P_CFY0+cn][n0] += 1./m0*(-cfy);
    c->P[EIF_P_CFY0+cn][n1] += 1./m1*(+cfy);
    c->P[EIF_P_CTZ0+cn][n0] += 1./i0*(ix0*(-cfy)-iy0*(-cfx));
    c->P[EIF_P_CTZ0+cn][n1] += 1./i1*(ix1*(+cfy)-iy1*(+cfx));
  }
  return rc;
}

/* particle against the wall at x = wallx (collision.c:249-304) */
static int collide_wall(eifo_ctx *c, int cn, int n, double wallx){
  {
    const double x = PF(X, n)+PF(DX, n);
    const double r = fmax(PF(A, n), PF(B, n));
    const double norm = fabs(wallx-x);
    if(r-norm < 0.) return 0;
  }
  const ell_t e = {PF(A, n), PF(B, n), PF(X, n)+PF(DX, n), PF(Y, n)+PF(DY, n), PF(AZ, n)};
  circ_t cc;
  double ix, iy;
  const int rc = fit_wall(&e, wallx, &cc, &ix, &iy);
  const double pm = mass_of(PF(DEN, n), PF(A, n), PF(B, n));
  const double pim = moi_of(PF(DEN, n), PF(A, n), PF(B, n));
  const double reft = pow(sqrt(PF(A, n)*PF(B, n)), 1.5);
  const double k = pm*pow(M_PI, 2.)/pow(reft, 2.);
  double nx = wallx-cc.x;
  const double norm = fabs(nx);
  nx /= norm;
  const double overlap = cc.r-norm;
  if(overlap > 0.){
    const double cfx = k*overlap*nx, cfy = 0.;
    c->P[EIF_P_CFX0+cn][n] += 1./pm*(-cfx);
    c->P[EIF_P_CFY0+cn][n] += 1./pm*(-cfy);
    c->P[EIF_P_CTZ0+cn][n] += 1./pim*(ix*(-cfy)-iy*(-cfx));
  }
  return rc;
}

int eifo_compute_collision_force(eifo_ctx *c, int cn){
  if(cn < 0 || cn > 1) return EIF_ERR_ARG;
  int rc = 0;
  for(int n = 0; n < c->np; n++){
    c->P[EIF_P_CFX0+cn][n] = 0.;
    c->P[EIF_P_CFY0+cn][n] = 0.;
    c->P[EIF_P_CTZ0+cn][n] = 0.;
  }
  /* pairs in the order of the collision pair matrix (collision.c:27-38) */
  for(int n0 = 0; n0 < c->np; n0++){
    for(int n1 = n0+1; n1 < c->np; n1++){
      if(collide_pair(c, cn, n0, n1)) rc = EIF_ERR_NOCONV;
    }
  }
  const double walls[2] = {0., c->lx};
  for(int w = 0; w < 2; w++){
    for(int n = 0; n < c->np; n++){
      if(collide_wall(c, cn, n, walls[w])) rc = EIF_ERR_NOCONV;
    }
  }
  if(rc) snprintf(c->err, sizeof(c->err), "circle fit did not converge in %d iterations", EIF_FIT_MAX_ITER);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* particle increments (src/suspensions/increment.c:10-72), reset (reset.c:7-18),
 * update (update.c:8-34,61-65) */
int eifo_reset_particle_increments(eifo_ctx *c){
  for(int n = 0; n < c->np; n++){
    PF(DUX, n) = 0.; PF(DUY, n) = 0.; PF(DVZ, n) = 0.;
    PF(DX, n) = 0.; PF(DY, n) = 0.; PF(DAZ, n) = 0.;
  }
  return EIF_OK;
}

int eifo_increment_particles(eifo_ctx *c, int rk, double *residual){
  if(rk < 0 || rk > 2) return EIF_ERR_ARG;
  const double Fr = c->cfg.Fr, dt = c->dt, g = c->gamma[rk];
  double res = 0.;
  for(int n = 0; n < c->np; n++){
    const double den = PF(DEN, n);
    const double px = PF(DUX, n), py = PF(DUY, n), pz = PF(DVZ, n);
    PF(DUX, n) = +0.5*g*dt*(PF(CFX0, n)+PF(CFX1, n))+dt*PF(FUX, n)+(PF(IUX1, n)-PF(IUX0, n))
                 +1.0*g*dt*(1.-den)/pow(Fr, 2.);
    PF(DUY, n) = +0.5*g*dt*(PF(CFY0, n)+PF(CFY1, n))+dt*PF(FUY, n)+(PF(IUY1, n)-PF(IUY0, n));
    PF(DVZ, n) = +0.5*g*dt*(PF(CTZ0, n)+PF(CTZ1, n))+dt*PF(TVZ, n)+(PF(IVZ1, n)-PF(IVZ0, n));
    res = fmax(res, fabs(PF(DUX, n)-px));
    res = fmax(res, fabs(PF(DUY, n)-py));
    res = fmax(res, fabs(PF(DVZ, n)-pz));
  }
  for(int n = 0; n < c->np; n++){
    const double ux0 = PF(UX, n), uy0 = PF(UY, n), vz0 = PF(VZ, n);
    const double ux1 = PF(UX, n)+PF(DUX, n), uy1 = PF(UY, n)+PF(DUY, n), vz1 = PF(VZ, n)+PF(DVZ, n);
    PF(DX, n) = 0.5*g*dt*(ux0+ux1);
    PF(DY, n) = 0.5*g*dt*(uy0+uy1);
    PF(DAZ, n) = 0.5*g*dt*(vz0+vz1);
  }
  if(residual) *residual = res;
  return EIF_OK;
}

int eifo_update_particles(eifo_ctx *c){
  const double ly = c->ly;
  for(int n = 0; n < c->np; n++){
    PF(UX, n) += PF(DUX, n);
    PF(UY, n) += PF(DUY, n);
    PF(VZ, n) += PF(DVZ, n);
  }
  for(int n = 0; n < c->np; n++){
    PF(X, n) += PF(DX, n);
    PF(Y, n) += PF(DY, n);
    PF(AZ, n) += PF(DAZ, n);
    if(PF(Y, n) < 0.) PF(Y, n) += ly;
    if(PF(Y, n) > ly) PF(Y, n) -= ly;
    if(PF(AZ, n) < 0.) PF(AZ, n) += 2.*M_PI;
    if(PF(AZ, n) > 2.*M_PI) PF(AZ, n) -= 2.*M_PI;
  }
  return EIF_OK;
}

/* ------------------------------------------------------------------------- */
/* time step size (src/param/decide_dt.c:11-81) */
int eifo_decide_dt(eifo_ctx *c, double *dt){
  const int itot = c->itot, jtot = c->jtot;
  const double small = 1.e-8, Re = c->cfg.Re, dy = c->dy;
  double dt_adv = 5.e-2;
  for(int j = 1; j <= jtot; j++){
    for(int i = 2; i <= itot; i++){
      const double vel = fmax(fabs(UX(i, j)), small);
      dt_adv = fmin(dt_adv, DXC(i)/vel);
    }
  }
  for(int j = 1; j <= jtot; j++){
    for(int i = 1; i <= itot; i++){
      const double vel = fmax(fabs(UY(i, j)), small);
      dt_adv = fmin(dt_adv, dy/vel);
    }
  }
  dt_adv *= c->cfg.safefactors[0];
  double dxmin = c->lx;
  for(int i = 2; i <= itot; i++) dxmin = fmin(dxmin, DXC(i));
  double dt_dif_x = 0.25*Re*pow(dxmin, 2.);
  double dt_dif_y = 0.25*Re*pow(dy, 2.);
  dt_dif_x *= c->cfg.safefactors[1];
  dt_dif_y *= c->cfg.safefactors[1];
  const double delta = fmin(c->dx, c->dy);
  double dt_par = DBL_MAX;
  for(int n = 0; n < c->np; n++){
    const double r = fmax(PF(A, n), PF(B, n));
    const double pux = fmax(fabs(PF(UX, n))+fabs(r*PF(VZ, n)), small);
    const double puy = fmax(fabs(PF(UY, n))+fabs(r*PF(VZ, n)), small);
    dt_par = fmin(dt_par, delta/fmax(pux, puy));
  }
  dt_par *= c->cfg.safefactors[2];
  c->dt = fmin(fmin(dt_adv, fmin(dt_dif_x, dt_dif_y)), dt_par);
  if(dt) *dt = c->dt;
  return EIF_OK;
}

/* ------------------------------------------------------------------------- */
/* one time step of RK stages (src/main.c:13-55) */
int eifo_integrate(eifo_ctx *c, int *substeps){
  int rc = EIF_OK;
  for(int rk = 0; rk < 3; rk++){
    eifo_reset_particle_increments(c);
    eifo_update_boundaries(c);
    eifo_compute_inertia(c, 0);
    eifo_update_velocity(c, rk);
    eifo_exchange_momentum(c);
    eifo_update_momentum_field(c);
    eifo_compute_potential(c, rk);
    eifo_correct_velocity(c, rk);
    eifo_update_pressure(c);
    if(eifo_compute_collision_force(c, 0)) rc = EIF_ERR_NOCONV;
    int sub;
    for(sub = 0; ; sub++){
      eifo_compute_inertia(c, 1);
      if(eifo_compute_collision_force(c, 1)) rc = EIF_ERR_NOCONV;
      double residual;
      eifo_increment_particles(c, rk, &residual);
      if(residual < 1.e-8) break;
      if(sub > 100) break;
    }
    if(substeps) substeps[rk] = sub+1;
    eifo_update_particles(c);
  }
  return rc;
}

int eifo_advance(eifo_ctx *c, int nsteps){
  int rc = EIF_OK;
  for(int s = 0; s < nsteps; s++){
    eifo_decide_dt(c, NULL);
    int r = eifo_integrate(c, NULL);
    if(r) rc = r;
    c->step += 1;
    c->time += c->dt;
  }
  return rc;
}

/* ------------------------------------------------------------------------- */
/* lifetime and state transfer */
int eifo_create(const eif_config_t *cfg, eifo_ctx **out){
  if(!cfg || !out || cfg->itot < 2 || cfg->jtot < 3 || !(cfg->ly > 0.)) return EIF_ERR_ARG;
  eifo_ctx *c = calloc(1, sizeof(eifo_ctx));
  c->cfg = *cfg;
  c->itot = cfg->itot;
  c->jtot = cfg->jtot;
  c->lx = 1.;
  c->ly = cfg->ly;
  c->nthreads = 1;
  setup_grid(c);
  const size_t nx = (size_t)(c->itot+1)*(c->jtot+2);
  const size_t ny = (size_t)(c->itot+2)*(c->jtot+2);
  c->ux = calloc(nx, sizeof(double));
  c->uy = calloc(ny, sizeof(double));
  c->p = calloc(ny, sizeof(double));
  c->psi = calloc(ny, sizeof(double));
  c->dux = calloc(ny, sizeof(double));
  c->duy = calloc(ny, sizeof(double));
  const size_t sx = (size_t)(c->itot-1)*c->jtot, sy = (size_t)c->itot*c->jtot;
  c->sxa = calloc(sx, sizeof(double)); c->sxb = calloc(sx, sizeof(double)); c->sxg = calloc(sx, sizeof(double));
  c->sya = calloc(sy, sizeof(double)); c->syb = calloc(sy, sizeof(double)); c->syg = calloc(sy, sizeof(double));
  c->q = calloc(sy, sizeof(double));
  for(int f = 0; f < EIF_NFIELDS; f++) c->P[f] = calloc(1, sizeof(double));
  eifo_update_boundaries(c);
  *out = c;
  return EIF_OK;
}

int eifo_destroy(eifo_ctx *c){
  if(!c) return EIF_OK;
  free(c->xf); free(c->xc); free(c->dxf); free(c->dxc); free(c->yf); free(c->yc);
  free(c->ux); free(c->uy); free(c->p); free(c->psi); free(c->dux); free(c->duy);
  free(c->sxa); free(c->sxb); free(c->sxg); free(c->sya); free(c->syb); free(c->syg);
  free(c->q);
  for(int f = 0; f < EIF_NFIELDS; f++) free(c->P[f]);
  free(c);
  return EIF_OK;
}

const char *eifo_last_error(const eifo_ctx *c){ return c ? c->err : "null context"; }
int eifo_set_threads(eifo_ctx *c, int n){ c->nthreads = n > 0 ? n : 1; return EIF_OK; }

int eifo_push_fluid(eifo_ctx *c, const double *ux, const double *uy, const double *p){
  const size_t nx = (size_t)(c->itot+1)*(c->jtot+2);
  const size_t ny = (size_t)(c->itot+2)*(c->jtot+2);
  memcpy(c->ux, ux, nx*sizeof(double));
  memcpy(c->uy, uy, ny*sizeof(double));
  memcpy(c->p, p, ny*sizeof(double));
  return eifo_update_boundaries(c);
}

int eifo_pull_fluid(eifo_ctx *c, double *ux, double *uy, double *p, double *psi){
  const size_t nx = (size_t)(c->itot+1)*(c->jtot+2);
  const size_t ny = (size_t)(c->itot+2)*(c->jtot+2);
  if(ux) memcpy(ux, c->ux, nx*sizeof(double));
  if(uy) memcpy(uy, c->uy, ny*sizeof(double));
  if(p) memcpy(p, c->p, ny*sizeof(double));
  if(psi) memcpy(psi, c->psi, ny*sizeof(double));
  return EIF_OK;
}

int eifo_push_particles(eifo_ctx *c, int n, const double *rec){
  if(n < 0) return EIF_ERR_ARG;
  c->np = n;
  for(int f = 0; f < EIF_NFIELDS; f++){
    free(c->P[f]);
    c->P[f] = calloc(n > 0 ? n : 1, sizeof(double));
    for(int k = 0; k < n; k++) c->P[f][k] = rec[(size_t)k*EIF_NFIELDS+f];
  }
  return EIF_OK;
}

int eifo_pull_particles(eifo_ctx *c, int n, double *rec){
  if(n != c->np) return EIF_ERR_ARG;
  for(int f = 0; f < EIF_NFIELDS; f++){
    for(int k = 0; k < n; k++) rec[(size_t)k*EIF_NFIELDS+f] = c->P[f][k];
  }
  return EIF_OK;
}

int eifo_pull_src(eifo_ctx *c, double *uxa, double *uxb, double *uya, double *uyb){
  const size_t sx = (size_t)(c->itot-1)*c->jtot, sy = (size_t)c->itot*c->jtot;
  if(uxa) memcpy(uxa, c->sxa, sx*sizeof(double));
  if(uxb) memcpy(uxb, c->sxb, sx*sizeof(double));
  if(uya) memcpy(uya, c->sya, sy*sizeof(double));
  if(uyb) memcpy(uyb, c->syb, sy*sizeof(double));
  return EIF_OK;
}

int eifo_push_src(eifo_ctx *c, const double *uxa, const double *uya){
  const size_t sx = (size_t)(c->itot-1)*c->jtot, sy = (size_t)c->itot*c->jtot;
  memcpy(c->sxa, uxa, sx*sizeof(double));
  memcpy(c->sya, uya, sy*sizeof(double));
  return EIF_OK;
}

int eifo_pull_ibm_fields(eifo_ctx *c, double *dux, double *duy){
  const size_t ny = (size_t)(c->itot+2)*(c->jtot+2);
  memcpy(dux, c->dux, ny*sizeof(double));
  memcpy(duy, c->duy, ny*sizeof(double));
  return EIF_OK;
}

int eifo_set_dt(eifo_ctx *c, double dt){ c->dt = dt; return EIF_OK; }
int eifo_get_dt(eifo_ctx *c, double *dt){ *dt = c->dt; return EIF_OK; }
int eifo_get_time(eifo_ctx *c, int *step, double *time){ *step = c->step; *time = c->time; return EIF_OK; }
int eifo_set_time(eifo_ctx *c, int step, double time){ c->step = step; c->time = time; return EIF_OK; }

/* maximum and sum of the discrete divergence (src/logging.c:40-66) */
int eifo_divergence(eifo_ctx *c, double *divmax, double *divsum){
  const int itot = c->itot, jtot = c->jtot;
  double mx = 0., sm = 0.;
  for(int j = 1; j <= jtot; j++){
    for(int i = 1; i <= itot; i++){
      const double div = (UX(i+1, j)-UX(i, j))/DXF(i)+(UY(i, j+1)-UY(i, j))/c->dy;
      mx = fmax(mx, fabs(div));
      sm += div;
    }
  }
  *divmax = mx;
  *divsum = sm;
  return EIF_OK;
}
