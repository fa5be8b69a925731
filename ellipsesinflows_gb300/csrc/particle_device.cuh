// Device code of the collision forces and the Crank-Nicolson increments, shared by
// the stand-alone kernels (particles.cu) and the batch's per-stage sub-iteration
// kernel (subiter.cu).
//
// Reference functions restated here (NaokiHori/EllipsesInFlows):
//   compute_evolute, find_equivalent_circle(s)   src/suspensions/collision.c:75-154
//   compute_collision_force_p_p / _p_w           src/suspensions/collision.c:156-304
//   suspensions_compute_collision_force          src/suspensions/collision.c:306-367
//   compute_curvature                            src/ellipse.c:17-28
//   suspensions_increment_particles              src/suspensions/increment.c:10-72
//
// The particle records are read with ordinary loads: the persistent sub-iteration
// kernel writes them between its phases.
#pragma once
#include "eif_internal.cuh"
#include <cfloat>

namespace {

struct EllD { double a, b, x, y, angle; };

using eifd::pmass;
using eifd::pmoi;

// ellipse.c:30-65 with per-call evaluation of the evolute coefficients
__device__ double normal_t_d(double a, double b, double x_, double y_) {
  const double px = fabs(x_), py = fabs(y_);
  const double kex = a * (1. - (b / a) * (b / a));
  const double key = b * (1. - (a / b) * (a / b));
  const double ab2 = a * a + b * b;
  double t = 0.25 * M_PI;
  for (int n = 0;; n++) {
    double st, ct;
    sincos(t, &st, &ct);
    const double x = a * ct, y = b * st;
    const double ex = kex * (ct * ct * ct), ey = key * (st * st * st);
    const double rx = x - ex, ry = y - ey, qx = px - ex, qy = py - ey;
    const double r = sqrt(ry * ry + rx * rx);
    const double q = sqrt(qy * qy + qx * qx);
    const double dc = r * asin((rx * qy - ry * qx) / (r * q));
    const double dt = dc / sqrt(ab2 - x * x - y * y);
    t += dt;
    t = fmin(0.5 * M_PI, t);
    t = fmax(0., t);
    if (fabs(dt) < 1.e-8) break;
    if (n > EIF_NORMAL_MAX_ITER - 1) break;
  }
  if (x_ < 0.) t = M_PI - t;
  if (y_ < 0.) t = -t;
  return t;
}

// ellipse.c:17-28
__device__ __forceinline__ double curvature(double a, double b, double t) {
  double st, ct;
  sincos(t, &st, &ct);
  const double ct2 = ct * ct, st2 = st * st;
  return a * b * (ct2 + st2) / pow(a * a * st2 + b * b * ct2, 1.5);
}

// collision.c:75-109
__device__ void evolute(const EllD &e, double x, double y, double &ex, double &ey, double &ix, double &iy, double &r) {
  double sn, cs;
  sincos(-e.angle, &sn, &cs);
  const double x__ = x - e.x, y__ = y - e.y;
  double x_ = cs * x__ - sn * y__;
  double y_ = sn * x__ + cs * y__;
  const double t = normal_t_d(e.a, e.b, x_, y_);
  r = 1. / fmax(curvature(e.a, e.b, t), DBL_EPSILON);
  double st, ct;
  sincos(t, &st, &ct);
  x_ = e.a * (1. - (e.b / e.a) * (e.b / e.a)) * (ct * ct * ct);
  y_ = e.b * (1. - (e.a / e.b) * (e.a / e.b)) * (st * st * st);
  double sp, cp;
  sincos(e.angle, &sp, &cp);
  ex = cp * x_ - sp * y_;
  ey = sp * x_ + cp * y_;
  ex = ex + e.x;
  ey = ey + e.y;
  x_ = e.a * ct;
  y_ = e.b * st;
  ix = cp * x_ - sp * y_;
  iy = sp * x_ + cp * y_;
}

// collision.c:111-135; returns false when the iteration cap is reached
__device__ bool fit_pair(const EllD &e0, const EllD &e1, double c0[3], double c1[3], double &ix0, double &iy0,
                         double &ix1, double &iy1) {
  c0[0] = e0.x; c0[1] = e0.y;
  c1[0] = e1.x; c1[1] = e1.y;
  for (int n = 0; n < EIF_FIT_MAX_ITER; n++) {
    double c0x, c0y, c1x, c1y;
    evolute(e0, c1[0], c1[1], c0x, c0y, ix0, iy0, c0[2]);
    evolute(e1, c0[0], c0[1], c1x, c1y, ix1, iy1, c1[2]);
    const double d0x = c0x - c0[0], d0y = c0y - c0[1];
    const double d1x = c1x - c1[0], d1y = c1y - c1[1];
    c0[0] += d0x; c0[1] += d0y;
    c1[0] += d1x; c1[1] += d1y;
    if (fmax(fmax(fabs(d0x), fabs(d0y)), fmax(fabs(d1x), fabs(d1y))) < 1.e-8) return true;
  }
  return false;
}

// collision.c:137-154
__device__ bool fit_wall(const EllD &e, double wallx, double cc[3], double &ix, double &iy) {
  cc[0] = e.x; cc[1] = e.y;
  for (int n = 0; n < EIF_FIT_MAX_ITER; n++) {
    double cx, cy;
    evolute(e, 2. * wallx - cc[0], cc[1], cx, cy, ix, iy, cc[2]);
    const double dcx = cx - cc[0], dcy = cy - cc[1];
    cc[0] += dcx; cc[1] += dcy;
    if (fmax(fabs(dcx), fabs(dcy)) < 1.e-8) return true;
  }
  return false;
}

__device__ __forceinline__ double harmonic(double v0, double v1) { return 1. / (0.5 * (1. / v0 + 1. / v1)); }

struct PV {  // particle view at the positions X^k + dX
  double den, a, b, x, y, az;
};

__device__ __forceinline__ PV load_pv(const double *P, int pc, int n) {
  PV v;
  v.den = P[EIF_P_DEN * pc + n];
  v.a = P[EIF_P_A * pc + n];
  v.b = P[EIF_P_B * pc + n];
  v.x = P[EIF_P_X * pc + n] + P[EIF_P_DX * pc + n];
  v.y = P[EIF_P_Y * pc + n] + P[EIF_P_DY * pc + n];
  v.az = P[EIF_P_AZ * pc + n];
  return v;
}

// y-offset of the nearest periodic image of p1 seen from p0 (collision.c:158-171)
__device__ __forceinline__ double image_offset(double p0y, double p1y, double ly) {
  double yoff = 0., minval = DBL_MAX;
  for (int per = -1; per <= 1; per++) {
    const double v = fabs((p1y + ly * per) - p0y);
    if (v < minval) { minval = v; yoff = ly * per; }
  }
  return yoff;
}

// exact early-out of collision.c:173-189: true when the bounding circles overlap
__device__ __forceinline__ bool bounding_overlap(const PV &p0, const PV &p1, double ly) {
  const double yoff = image_offset(p0.y, p1.y, ly);
  const double nx = p1.x - p0.x, ny = (p1.y + yoff) - p0.y;
  const double norm = fmax(hypot(nx, ny), DBL_EPSILON);
  return !(fmax(p0.a, p0.b) + fmax(p1.a, p1.b) - norm < 0.);
}

// Pairs whose bounding circles overlap (collision.c:173-189) but whose ellipses are
// apart. The reference then iterates the equivalent-circle fit (collision.c:111-135) to
// the circles of curvature at the mutually nearest points, whose overlap is minus the
// gap, and the pair adds no force; for nearly touching ellipses that fixed point
// converges slowly (thousands of iterations in double precision). A line that separates
// the two ellipses with a gap above a hundredth of the smaller minor semi-axis (far above
// the fit's stopping error) proves the same zero contribution without the iteration.
// Candidate normals: the centre line, the four semi-axis directions and 16 fixed
// directions; along a unit normal n the ellipses' extents are their support values
// sqrt(a^2 (n.u)^2 + b^2 (n.v)^2) about the centres.
__device__ bool apart(const PV &p0, const PV &p1, double ly) {
  const double yoff = image_offset(p0.y, p1.y, ly);
  const double dx = p1.x - p0.x, dy = (p1.y + yoff) - p0.y;
  double s0, c0, s1, c1;
  sincos(p0.az, &s0, &c0);
  sincos(p1.az, &s1, &c1);
  const double margin = 0.01 * fmin(fmin(p0.a, p0.b), fmin(p1.a, p1.b));
  auto gap = [&](double nx, double ny) {
    const double u0 = nx * c0 + ny * s0, v0 = ny * c0 - nx * s0;
    const double u1 = nx * c1 + ny * s1, v1 = ny * c1 - nx * s1;
    const double h0 = sqrt(p0.a * p0.a * u0 * u0 + p0.b * p0.b * v0 * v0);
    const double h1 = sqrt(p1.a * p1.a * u1 * u1 + p1.b * p1.b * v1 * v1);
    return fabs(nx * dx + ny * dy) - h0 - h1;
  };
  const double d = hypot(dx, dy);
  if (d > 0. && gap(dx / d, dy / d) > margin) return true;
  if (gap(c0, s0) > margin || gap(-s0, c0) > margin || gap(c1, s1) > margin || gap(-s1, c1) > margin) return true;
  for (int q = 0; q < 16; q++) {
    double s, c;
    sincospi(q / 16., &s, &c);
    if (gap(c, s) > margin) return true;
  }
  return false;
}

// force/torque contribution of pair (n0 < n1) on particle `self` (collision.c:190-246)
__device__ void pair_contribution(const PV &p0, const PV &p1, bool self_is_0, double ly, double out[3], bool &ok) {
  out[0] = out[1] = out[2] = 0.;
  const double yoff = image_offset(p0.y, p1.y, ly);
  EllD e0{p0.a, p0.b, p0.x, p0.y, p0.az};
  EllD e1{p1.a, p1.b, p1.x, p1.y + yoff, p1.az};
  double c0[3], c1[3], ix0, iy0, ix1, iy1;
  ok = fit_pair(e0, e1, c0, c1, ix0, iy0, ix1, iy1);
  const double m0 = pmass(p0.den, p0.a, p0.b), m1 = pmass(p1.den, p1.a, p1.b);
  const double i0 = pmoi(p0.den, p0.a, p0.b), i1 = pmoi(p1.den, p1.a, p1.b);
  const double mass = harmonic(m0, m1);
  const double reft = pow(harmonic(sqrt(p0.a * p0.b), sqrt(p1.a * p1.b)), 1.5);
  const double k = mass * (M_PI * M_PI) / (reft * reft);
  double nx = c1[0] - c0[0], ny = c1[1] - c0[1];
  const double norm = fmax(hypot(nx, ny), DBL_EPSILON);
  nx /= norm;
  ny /= norm;
  const double overlap = c0[2] + c1[2] - norm;
  if (overlap > 0.) {
    const double cfx = k * overlap * nx, cfy = k * overlap * ny;
    if (self_is_0) {
      out[0] = 1. / m0 * (-cfx);
      out[1] = 1. / m0 * (-cfy);
      out[2] = 1. / i0 * (ix0 * (-cfy) - iy0 * (-cfx));
    } else {
      out[0] = 1. / m1 * (+cfx);
      out[1] = 1. / m1 * (+cfy);
      out[2] = 1. / i1 * (ix1 * (+cfy) - iy1 * (+cfx));
    }
  }
}

// collision.c:249-304
__device__ void wall_contribution(const PV &p, double wallx, double out[3], bool &ok) {
  out[0] = out[1] = out[2] = 0.;
  ok = true;
  const double r = fmax(p.a, p.b);
  if (r - fabs(wallx - p.x) < 0.) return;
  EllD e{p.a, p.b, p.x, p.y, p.az};
  double cc[3], ix, iy;
  ok = fit_wall(e, wallx, cc, ix, iy);
  const double pm = pmass(p.den, p.a, p.b), pim = pmoi(p.den, p.a, p.b);
  const double reft = pow(sqrt(p.a * p.b), 1.5);
  const double k = pm * (M_PI * M_PI) / (reft * reft);
  double nx = wallx - cc[0];
  const double norm = fabs(nx);
  nx /= norm;
  const double overlap = cc[2] - norm;
  if (overlap > 0.) {
    const double cfx = k * overlap * nx, cfy = 0.;
    out[0] = 1. / pm * (-cfx);
    out[1] = 1. / pm * (-cfy);
    out[2] = 1. / pim * (ix * (-cfy) - iy * (-cfx));
  }
}

// Collision forces (collision.c:306-367) in one launch, one warp per particle k:
//  1. candidate partners: the lanes test the partners m = lane, lane + 32, ... in order
//     against single-precision centres (at X^k + dX) and bounding radii, staged in shared
//     memory tile by tile (every block forms them from the records as it loads a tile);
//     the pairs that pass this conservative test are listed in partner order (ballot and
//     prefix count);
//  2. the lanes give the listed pairs the exact double-precision bounding-circle test of
//     collision.c:173-189 (canonical orientation) and compact the hits in order;
//  3. the hits are evaluated one per lane (circle fit, force and torque) and summed in
//     partner order by lane 0, then the walls at x = 0 and x = lx are added.
constexpr int CAND_CAP = EIF_CAND_CAP;   // candidates per particle
constexpr int PAIR_WARPS = 8;
constexpr int PAIR_TILE = 1024;
constexpr int PAIR_LOADS = PAIR_TILE / (PAIR_WARPS * 32);

__device__ __forceinline__ float4 pair_prefilter(const double *P, int pcap, int n) {
  const double x = P[EIF_P_X * pcap + n] + P[EIF_P_DX * pcap + n];
  const double y = P[EIF_P_Y * pcap + n] + P[EIF_P_DY * pcap + n];
  return make_float4(eifd::d2f(x), eifd::d2f(y), eifd::d2f(fmax(P[EIF_P_A * pcap + n], P[EIF_P_B * pcap + n])), 0.f);
}

// One block of PAIR_WARPS warps: particles block * PAIR_WARPS ...
__device__ __forceinline__ void collision_block(double *P, int pcap, int np, int cn, double ly, double lx,
                                                unsigned *flags, int block) {
  __shared__ float4 tile[PAIR_TILE];
  __shared__ int list[PAIR_WARPS][CAND_CAP];
  __shared__ double cval[PAIR_WARPS][32][3];
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int k = block * PAIR_WARPS + wl;
  const bool on = k < np;   // uniform over the warp
  const float4 fk = on ? pair_prefilter(P, pcap, k) : make_float4(0.f, 0.f, 0.f, 0.f);
  const float lyf = eifd::d2f(ly);
  int nmaybe = 0;
  for (int t0 = 0; t0 < np; t0 += PAIR_TILE) {
    const int nt = min(PAIR_TILE, np - t0);
    float4 st[PAIR_LOADS];
#pragma unroll
    for (int r = 0; r < PAIR_LOADS; r++) {
      const int q = threadIdx.x + r * PAIR_WARPS * 32;
      st[r] = q < nt ? pair_prefilter(P, pcap, t0 + q) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PAIR_LOADS; r++) tile[threadIdx.x + r * PAIR_WARPS * 32] = st[r];
    __syncthreads();
    if (!on) continue;
#pragma unroll 2
    for (int base = 0; base < nt; base += 32) {
      const int m = t0 + base + lane;
      bool maybe = false;
      if (base + lane < nt && m != k) {
        const float4 fm = tile[base + lane];
        // conservative single-precision test: skip only pairs clearly apart for every image
        const float rs = fk.z + fm.z;
        const float dxf = fm.x - fk.x;
        const float lim = rs * rs * 1.001f + 1e-6f;
#pragma unroll
        for (int per = -1; per <= 1; per++) {
          const float dyf = fm.y + lyf * per - fk.y;
          maybe |= dxf * dxf + dyf * dyf <= lim;
        }
      }
      const unsigned mask = __ballot_sync(0xffffffffu, maybe);
      if (maybe) {
        const int r = nmaybe + __popc(mask & ((1u << lane) - 1u));
        if (r < CAND_CAP) list[wl][r] = m;
      }
      nmaybe += __popc(mask);
    }
  }
  if (!on) return;
  __syncwarp();
  if (nmaybe > CAND_CAP && lane == 0) atomicOr(flags, EIF_FLAG_NOCONV);
  nmaybe = min(nmaybe, CAND_CAP);
  const PV pk = load_pv(P, pcap, k);
  // exact test, hits compacted in place (a write never passes the entries still to read)
  int cnt = 0;
  for (int base = 0; base < nmaybe; base += 32) {
    const int q = base + lane;
    bool hit = false;
    int m = 0;
    if (q < nmaybe) {
      m = list[wl][q];
      const PV pm_ = load_pv(P, pcap, m);
      hit = m < k ? bounding_overlap(pm_, pk, ly) : bounding_overlap(pk, pm_, ly);
    }
    const unsigned mask = __ballot_sync(0xffffffffu, hit);
    if (hit) list[wl][cnt + __popc(mask & ((1u << lane) - 1u))] = m;
    cnt += __popc(mask);
    __syncwarp();
  }
  // forces of the hits, summed in partner order
  double acc0 = 0., acc1 = 0., acc2 = 0.;
  bool ok_all = true;
  for (int base = 0; base < cnt; base += 32) {
    const int q = base + lane;
    const int ncand = min(32, cnt - base);
    if (q < cnt) {
      const int mm = list[wl][q];
      const PV pmm = load_pv(P, pcap, mm);
      double out[3] = {0., 0., 0.};
      bool ok = true;
      if (mm < k) {
        if (!apart(pmm, pk, ly)) pair_contribution(pmm, pk, false, ly, out, ok);
      } else {
        if (!apart(pk, pmm, ly)) pair_contribution(pk, pmm, true, ly, out, ok);
      }
      ok_all &= ok;
      cval[wl][lane][0] = out[0];
      cval[wl][lane][1] = out[1];
      cval[wl][lane][2] = out[2];
    }
    __syncwarp();
    if (lane == 0) {
      for (int t = 0; t < ncand; t++) {
        acc0 += cval[wl][t][0];
        acc1 += cval[wl][t][1];
        acc2 += cval[wl][t][2];
      }
    }
    __syncwarp();
  }
  const bool ok_warp = __all_sync(0xffffffffu, ok_all);
  if (lane == 0) {
    double out[3];
    bool ok0, ok1;
    wall_contribution(pk, 0., out, ok0);
    acc0 += out[0]; acc1 += out[1]; acc2 += out[2];
    wall_contribution(pk, lx, out, ok1);
    acc0 += out[0]; acc1 += out[1]; acc2 += out[2];
    P[(EIF_P_CFX0 + cn) * pcap + k] = acc0;
    P[(EIF_P_CFY0 + cn) * pcap + k] = acc1;
    P[(EIF_P_CTZ0 + cn) * pcap + k] = acc2;
    if (!(ok_warp && ok0 && ok1)) atomicOr(flags, EIF_FLAG_NOCONV);
  }
}

// increment.c:10-72 for particle n: new increments from the forces, inertia integrals
// and collision forces of the sub-iteration, the position increments from them; returns
// res raised to the largest change of the velocity increments
__device__ __forceinline__ double increment_particle(double *p, int pcap, int n, double gamma, double Fr2, double dt,
                                                     double res) {
  const double den = p[EIF_P_DEN * pcap + n];
  const double px = p[EIF_P_DUX * pcap + n], py = p[EIF_P_DUY * pcap + n], pz = p[EIF_P_DVZ * pcap + n];
  const double hgd = 0.5 * gamma * dt;
  const double dux = hgd * (p[EIF_P_CFX0 * pcap + n] + p[EIF_P_CFX1 * pcap + n]) + dt * p[EIF_P_FUX * pcap + n] +
                     (p[EIF_P_IUX1 * pcap + n] - p[EIF_P_IUX0 * pcap + n]) + 1.0 * gamma * dt * (1. - den) / Fr2;
  const double duy = hgd * (p[EIF_P_CFY0 * pcap + n] + p[EIF_P_CFY1 * pcap + n]) + dt * p[EIF_P_FUY * pcap + n] +
                     (p[EIF_P_IUY1 * pcap + n] - p[EIF_P_IUY0 * pcap + n]);
  const double dvz = hgd * (p[EIF_P_CTZ0 * pcap + n] + p[EIF_P_CTZ1 * pcap + n]) + dt * p[EIF_P_TVZ * pcap + n] +
                     (p[EIF_P_IVZ1 * pcap + n] - p[EIF_P_IVZ0 * pcap + n]);
  p[EIF_P_DUX * pcap + n] = dux;
  p[EIF_P_DUY * pcap + n] = duy;
  p[EIF_P_DVZ * pcap + n] = dvz;
  res = fmax(res, fabs(dux - px));
  res = fmax(res, fabs(duy - py));
  res = fmax(res, fabs(dvz - pz));
  const double ux0 = p[EIF_P_UX * pcap + n], uy0 = p[EIF_P_UY * pcap + n], vz0 = p[EIF_P_VZ * pcap + n];
  p[EIF_P_DX * pcap + n] = hgd * (ux0 + (ux0 + dux));
  p[EIF_P_DY * pcap + n] = hgd * (uy0 + (uy0 + duy));
  p[EIF_P_DAZ * pcap + n] = hgd * (vz0 + (vz0 + dvz));
  return res;
}

// reset.c:7-18 for particle n: increments of the new stage start at zero
__device__ __forceinline__ void reset_particle(double *P, int pcap, int n) {
  P[EIF_P_DUX * pcap + n] = 0.; P[EIF_P_DUY * pcap + n] = 0.; P[EIF_P_DVZ * pcap + n] = 0.;
  P[EIF_P_DX * pcap + n] = 0.; P[EIF_P_DY * pcap + n] = 0.; P[EIF_P_DAZ * pcap + n] = 0.;
}

// update.c:8-34 for particle n: velocities and positions advanced by the increments,
// the centre wrapped into [0, ly] and the angle into [0, 2 pi]
__device__ __forceinline__ void update_particle(double *P, int pcap, int n, double ly) {
  P[EIF_P_UX * pcap + n] += P[EIF_P_DUX * pcap + n];
  P[EIF_P_UY * pcap + n] += P[EIF_P_DUY * pcap + n];
  P[EIF_P_VZ * pcap + n] += P[EIF_P_DVZ * pcap + n];
  double x = P[EIF_P_X * pcap + n] + P[EIF_P_DX * pcap + n];
  double y = P[EIF_P_Y * pcap + n] + P[EIF_P_DY * pcap + n];
  double az = P[EIF_P_AZ * pcap + n] + P[EIF_P_DAZ * pcap + n];
  if (y < 0.) y += ly;
  if (y > ly) y -= ly;
  if (az < 0.) az += 2. * M_PI;
  if (az > 2. * M_PI) az -= 2. * M_PI;
  P[EIF_P_X * pcap + n] = x;
  P[EIF_P_Y * pcap + n] = y;
  P[EIF_P_AZ * pcap + n] = az;
}

}  // namespace
