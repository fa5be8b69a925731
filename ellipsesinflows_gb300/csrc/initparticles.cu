// Particle placement of the reference's initial-condition generator
// (initparticles/RandomGenerator/src/main.c:160-256), host code. Each new ellipse gets
// uniformly random centre candidates (x from max(a,b) to lx - max(a,b), y in [0, ly),
// two rand() draws each) until no earlier ellipse (nearest periodic image in y) has an
// overlapping bounding circle or an overlapping equivalent circle (the circles of
// curvature at the mutually nearest points, found by the evolute fixed point of
// main.c:138-158). The reference tests every earlier ellipse, O(N^2) per candidate;
// here the earlier ellipses are binned in y, and only those within reach of the
// candidate are tested: the equivalent circle of an ellipse lies within
// 2 max(a,b)^2 / min(a,b) - min(a,b) of its centre (evolute point plus radius of
// curvature at the minor-axis vertex), so the others pass both tests. The decisions,
// and hence the rand() stream and the result, are the reference's.
#include "eif_internal.cuh"
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <vector>

namespace {

struct EllipseG {
  double x, y, a, b, angle;
};
struct CircleG {
  double x, y, r;
};

double gen_random(double mn, double mx) { return (mx - mn) * rand() / RAND_MAX + mn; }

// main.c:45-64 (evolute offsets and curvature of the parametric ellipse)
double evolute_x(double a, double b, double t) { return a * (1. - std::pow(b / a, 2.)) * std::pow(std::cos(t), 3.); }
double evolute_y(double a, double b, double t) { return b * (1. - std::pow(a / b, 2.)) * std::pow(std::sin(t), 3.); }
double curvature(double a, double b, double t) {
  const double ct = std::cos(t), st = std::sin(t);
  const double ct2 = std::pow(ct, 2.), st2 = std::pow(st, 2.);
  const double a2 = std::pow(a, 2.), b2 = std::pow(b, 2.);
  return a * b * (ct2 + st2) / std::pow(a2 * st2 + b2 * ct2, 1.5);
}

// main.c:66-98: parameter of the normal foot of (x_, y_) in the body frame
double normal_foot(double a, double b, double x_, double y_) {
  const double px = std::fabs(x_), py = std::fabs(y_);
  double t = 0.25 * M_PI;
  for (int n = 0;; n++) {
    const double x = a * std::cos(t), y = b * std::sin(t);
    const double ex = evolute_x(a, b, t), ey = evolute_y(a, b, t);
    const double rx = x - ex, ry = y - ey, qx = px - ex, qy = py - ey;
    const double r = std::sqrt(std::pow(ry, 2.) + std::pow(rx, 2.));
    const double q = std::sqrt(std::pow(qy, 2.) + std::pow(qx, 2.));
    const double dc = r * std::asin((rx * qy - ry * qx) / (r * q));
    const double dt = dc / std::sqrt(a * a + b * b - x * x - y * y);
    t += dt;
    t = std::fmin(0.5 * M_PI, t);
    t = std::fmax(0., t);
    if (std::fabs(dt) < 1.e-8) break;
    if (n > 100) break;
  }
  if (x_ < 0.) t = M_PI - t;
  if (y_ < 0.) t = -t;
  return t;
}

// main.c:100-131: centre and radius of the circle of curvature at the foot of (x, y)
void evolute_circle(const EllipseG &e, double x, double y, double &ex, double &ey, double &r) {
  const double dx = x - e.x, dy = y - e.y;
  const double x_ = std::cos(-e.angle) * dx - std::sin(-e.angle) * dy;
  const double y_ = std::sin(-e.angle) * dx + std::cos(-e.angle) * dy;
  const double t = normal_foot(e.a, e.b, x_, y_);
  r = 1. / std::fmax(curvature(e.a, e.b, t), DBL_EPSILON);
  const double vx = evolute_x(e.a, e.b, t), vy = evolute_y(e.a, e.b, t);
  ex = std::cos(+e.angle) * vx - std::sin(+e.angle) * vy + e.x;
  ey = std::sin(+e.angle) * vx + std::cos(+e.angle) * vy + e.y;
}

// main.c:133-158: equivalent circles by fixed-point iteration (capped here)
bool equivalent_circles(const EllipseG &e0, const EllipseG &e1, CircleG &c0, CircleG &c1) {
  c0.x = e0.x; c0.y = e0.y;
  c1.x = e1.x; c1.y = e1.y;
  for (int n = 0; n < 100000; n++) {
    double c0x, c0y, c1x, c1y;
    evolute_circle(e0, c1.x, c1.y, c0x, c0y, c0.r);
    evolute_circle(e1, c0.x, c0.y, c1x, c1y, c1.r);
    const double d0x = c0x - c0.x, d0y = c0y - c0.y, d1x = c1x - c1.x, d1y = c1y - c1.y;
    c0.x += d0x; c0.y += d0y;
    c1.x += d1x; c1.y += d1y;
    if (std::fmax(std::fmax(std::fabs(d0x), std::fabs(d0y)), std::fmax(std::fabs(d1x), std::fabs(d1y))) < 1.e-8)
      return true;
  }
  return false;
}

double reach(double a, double b);

// main.c:199-239 for one earlier ellipse: true when the candidate must be redrawn
bool rejects(const EllipseG &cand, const EllipseG &old, double ly) {
  double yoffset = 0., minval = DBL_MAX;
  for (int periodic = -1; periodic <= 1; periodic++) {
    const double v = std::fabs((old.y + ly * periodic) - cand.y);
    if (v < minval) { minval = v; yoffset = ly * periodic; }
  }
  const double r0 = std::fmax(cand.a, cand.b), r1 = std::fmax(old.a, old.b);
  {
    const double nx = old.x - cand.x, ny = (old.y + yoffset) - cand.y;
    const double norm = std::fmax(std::hypot(nx, ny), DBL_EPSILON);
    if (norm - r0 - r1 < 0.) return true;
    // beyond the reach of both equivalent circles the fit cannot find an overlap
    if (norm > (reach(cand.a, cand.b) + reach(old.a, old.b)) * (1. + 1e-9)) return false;
  }
  EllipseG e1 = old;
  e1.y = old.y + yoffset;
  CircleG c0, c1;
  equivalent_circles(cand, e1, c0, c1);
  const double nx = c1.x - c0.x, ny = c1.y - c0.y;
  const double norm = std::fmax(std::hypot(nx, ny), DBL_EPSILON);
  return norm - c0.r - c1.r < 0.;
}

double reach(double a, double b) {
  const double mx = std::fmax(a, b), mn = std::fmin(a, b);
  return std::fmax(mx, 2. * mx * mx / mn - mn);
}

}  // namespace

extern "C" int eif_place_particles(double lx, double ly, int n, const double *as, const double *bs, const double *azs,
                                   double *xs, double *ys, long long max_tries) {
  if (n < 0 || !(lx > 0.) || !(ly > 0.) || (n > 0 && (!as || !bs || !azs || !xs || !ys))) return EIF_ERR_ARG;
  double rmax = 0.;
  for (int k = 0; k < n; k++) rmax = std::fmax(rmax, reach(as[k], bs[k]));
  // bins in y of at least twice the largest reach: candidates test the ellipses of their
  // own bin and the two neighbours (periodic)
  const int nb = std::max(1, (int)std::floor(ly / std::fmax(2. * rmax, 1e-300)));
  const double bw = ly / nb;
  std::vector<std::vector<int>> bins(nb);
  auto bin_of = [&](double y) {
    int b = (int)std::floor(y / bw);
    return ((b % nb) + nb) % nb;
  };
  long long tries = 0;
  for (int n0 = 0; n0 < n; n0++) {
    EllipseG cand{0., 0., as[n0], bs[n0], azs[n0]};
    const double r0 = std::fmax(as[n0], bs[n0]);
    for (;;) {
      if (++tries > max_tries) return EIF_ERR_NOCONV;
      cand.x = gen_random(r0, lx - r0);
      cand.y = gen_random(0., ly);
      const int b = bin_of(cand.y);
      bool bad = false;
      for (int db = -1; db <= 1 && !bad; db++) {
        if (nb < 3 && db != 0 && (nb == 1 || db == 1)) continue;   // each bin once
        for (int n1 : bins[((b + db) % nb + nb) % nb]) {
          const EllipseG old{xs[n1], ys[n1], as[n1], bs[n1], azs[n1]};
          if (rejects(cand, old, ly)) { bad = true; break; }
        }
      }
      if (!bad) break;
    }
    xs[n0] = cand.x;
    ys[n0] = cand.y;
    bins[bin_of(cand.y)].push_back(n0);
  }
  return EIF_OK;
}
