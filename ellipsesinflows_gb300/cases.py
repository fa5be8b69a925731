"""Initial states of the benchmark configurations.

A ``Case`` holds the run parameters (the environment variables of the
reference's load_config, src/param/init.c:67-103, plus the wall velocities),
the initial fluid fields in the reference's haloed layouts and the particle
records. Particle placement is a seeded random sequential addition with the
bounding-circle clearance test; the reference's own generator
(initparticles/RandomGenerator/src/main.c) uses C rand() with hard-coded
sizes, so seeds here do not reproduce its layouts.
"""
import math

import numpy as np

from .capi import F, NFIELDS, PREC_FP64, make_config

DBL_MAX = float(np.finfo(np.float64).max)


class Case:
    def __init__(self, name, itot, jtot, ly, Re, extfrcy=0.0, Fr=DBL_MAX, safefactors=(0.75, 0.75, 0.95),
                 uy_wall=(0.0, 0.0), particles=None, couette_init=False, steps=1):
        self.name, self.itot, self.jtot, self.ly = name, itot, jtot, ly
        self.Re, self.extfrcy, self.Fr = Re, extfrcy, Fr
        self.safefactors, self.uy_wall = tuple(safefactors), tuple(uy_wall)
        self.particles = np.zeros((0, NFIELDS)) if particles is None else np.asarray(particles, dtype=np.float64)
        self.couette_init = couette_init
        self.steps = steps

    @property
    def n_particles(self):
        return self.particles.shape[0]

    @property
    def cells(self):
        return self.itot * self.jtot

    def config(self, precision=PREC_FP64, device=0):
        return make_config(self.itot, self.jtot, ly=self.ly, Re=self.Re, Fr=self.Fr, extfrcy=self.extfrcy,
                           safefactors=self.safefactors, uy_wall=self.uy_wall, precision=precision, device=device)

    def xc(self):
        """Cell-centre x coordinates XC(0..itot+1) as set_coordinate computes them."""
        it = self.itot
        dx = 1.0 / it
        xf = np.array([1.0 * (i - 1) * dx for i in range(1, it + 2)])
        xf[0], xf[it] = 0.0, 1.0
        xc = np.empty(it + 2)
        xc[0] = xf[0]
        xc[1:it + 1] = 0.5 * (xf[:it] + xf[1:it + 1])
        xc[it + 1] = xf[it]
        return xc

    def fluid(self):
        """(ux, uy, p) initial fields, haloed reference layouts."""
        it, jt = self.itot, self.jtot
        ux = np.zeros((jt + 2, it + 1))
        uy = np.zeros((jt + 2, it + 2))
        p = np.zeros((jt + 2, it + 2))
        if self.couette_init:
            # docs/source/examples/case1/config/src_fluid_init.c:59-66
            uy[:, 1:it + 1] = -0.5 + self.xc()[1:it + 1][None, :]
        return ux, uy, p


def particle_records(den, a, b, x, y, az, ux=None, uy=None, vz=None):
    n = len(den)
    rec = np.zeros((n, NFIELDS))
    rec[:, F["den"]], rec[:, F["a"]], rec[:, F["b"]] = den, a, b
    rec[:, F["x"]], rec[:, F["y"]], rec[:, F["az"]] = x, y, az
    if ux is not None:
        rec[:, F["ux"]] = ux
    if uy is not None:
        rec[:, F["uy"]] = uy
    if vz is not None:
        rec[:, F["vz"]] = vz
    return rec


def place(n, radius, ly, clearance, rng, xmargin, max_tries=2_000_000):
    """Random sequential addition of n centres with pairwise distance >= r_i + r_j + clearance
    (periodic in y, centres kept xmargin + r_i away from the walls)."""
    radius = np.broadcast_to(np.asarray(radius, dtype=np.float64), (n,)).copy()
    rmax = float(radius.max())
    cell = 2 * rmax + clearance
    ncy = max(1, int(ly // cell))
    ncx = max(1, int(1.0 // cell))
    grid = {}
    xs, ys = np.empty(n), np.empty(n)
    placed, tries = 0, 0
    while placed < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place %d particles (placed %d)" % (n, placed))
        r = radius[placed]
        x = rng.uniform(r + xmargin, 1.0 - r - xmargin)
        y = rng.uniform(0.0, ly)
        cx, cy = min(int(x / (1.0 / ncx)), ncx - 1), min(int(y / (ly / ncy)), ncy - 1)
        ok = True
        for dxc in (-1, 0, 1):
            for dyc in (-1, 0, 1):
                for k in grid.get((cx + dxc, (cy + dyc) % ncy), ()):
                    ddy = abs(ys[k] - y)
                    ddy = min(ddy, ly - ddy)
                    if math.hypot(xs[k] - x, ddy) < r + radius[k] + clearance:
                        ok = False
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            xs[placed], ys[placed] = x, y
            grid.setdefault((cx, cy), []).append(placed)
            placed += 1
    return xs, ys


def _boundary(a, b, az, x, y, k=72):
    """k points on the ellipse (a, b) turned by az about (x, y)"""
    t = np.linspace(0.0, 2 * math.pi, k, endpoint=False)
    c, s = math.cos(az), math.sin(az)
    bx, by = a * np.cos(t), b * np.sin(t)
    return x + c * bx - s * by, y + s * bx + c * by


def _inside(px, py, a, b, az, x, y):
    """mask of the points (px, py) inside the ellipse (a, b) turned by az about (x, y)"""
    c, s = math.cos(-az), math.sin(-az)
    dx, dy = px - x, py - y
    u, v = c * dx - s * dy, s * dx + c * dy
    return (u / a) ** 2 + (v / b) ** 2 < 1.0


def place_ellipses(a, b, az, ly, clearance, rng, xmargin, max_tries=20_000_000):
    """Random sequential addition of ellipses (semi-axes a, b, angles az; arrays) with
    no ellipse closer than `clearance` to another (periodic in y, nearest image): a
    candidate is kept when, for every earlier ellipse whose bounding circle comes
    within reach, neither ellipse, grown by the clearance, contains any of 72 boundary
    points of the other. Bounding circles may overlap, so elongated ellipses pack
    beyond the bounding-circle rule (centres kept max(a, b) + xmargin from the walls)."""
    n = len(a)
    r = np.maximum(a, b)
    cell = 2 * r.max() + clearance
    ncy = max(1, int(ly // cell))
    grid = {}
    xs, ys = np.empty(n), np.empty(n)
    placed, tries = 0, 0
    while placed < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place %d ellipses (placed %d)" % (n, placed))
        k = placed
        x = rng.uniform(r[k] + xmargin, 1.0 - r[k] - xmargin)
        y = rng.uniform(0.0, ly)
        cy = min(int(y / (ly / ncy)), ncy - 1)
        ok = True
        for dyc in (-1, 0, 1):
            for m in grid.get((cy + dyc) % ncy, ()):
                ddy = y - ys[m]
                ddy -= ly * round(ddy / ly)
                ym = y - ddy     # the earlier ellipse's nearest image, seen from the candidate
                if math.hypot(xs[m] - x, ym - y) >= r[k] + r[m] + clearance:
                    continue
                c = clearance
                px, py = _boundary(a[k], b[k], az[k], x, y)
                qx, qy = _boundary(a[m], b[m], az[m], xs[m], ym)
                if (_inside(px, py, a[m] + c, b[m] + c, az[m], xs[m], ym).any() or
                        _inside(qx, qy, a[k] + c, b[k] + c, az[k], x, y).any()):
                    ok = False
                    break
            if not ok:
                break
        if ok:
            xs[k], ys[k] = x, y
            grid.setdefault(cy, []).append(k)
            placed += 1
    return xs, ys


def couette_circle(itot=64, jtot=128, steps=200):
    """Single neutrally buoyant circle in Couette flow (lateral migration, case1)."""
    rec = particle_records([1.0], [0.125], [0.125], [0.3], [1.0], [0.0])
    return Case("couette_circle_%dx%d" % (itot, jtot), itot, jtot, 2.0, 100.0, safefactors=(0.4, 0.4, 0.95),
                uy_wall=(-0.5, 0.5), particles=rec, couette_init=True, steps=steps)


def poiseuille(itot=512, jtot=1024, n=128, a=0.04, b=0.02, Re=200.0, seed=0, steps=1000):
    """Plane Poiseuille suspension of identical ellipses, fluid at rest, extfrcy = 8/Re."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / itot
    xs, ys = place(n, a, 2.0, dx, rng, dx)
    az = rng.uniform(0.0, math.pi, n)
    rec = particle_records(np.ones(n), np.full(n, a), np.full(n, b), xs, ys, az)
    return Case("poiseuille_%dx%d_n%d" % (itot, jtot, n), itot, jtot, 2.0, Re, extfrcy=8.0 / Re, particles=rec,
                steps=steps)


def mixed_target(itot=2048, jtot=4096, n=2048, a=0.012, Re=400.0, seed=1, steps=500):
    """Dense suspension of ellipses with aspect ratio U[1,3] and density ratio U[1,1.2]."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / itot
    xs, ys = place(n, a, 2.0, dx, rng, dx)
    ar = rng.uniform(1.0, 3.0, n)
    den = rng.uniform(1.0, 1.2, n)
    az = rng.uniform(0.0, math.pi, n)
    rec = particle_records(den, np.full(n, a), a / ar, xs, ys, az)
    return Case("suspension_%dx%d_n%d" % (itot, jtot, n), itot, jtot, 2.0, Re, extfrcy=8.0 / Re, particles=rec,
                steps=steps)


def adjoint_channel(n=8, itot=64, jtot=128, seed=11):
    """The inputs of the adjoint checks at 64x128: a channel (walls at rest) with n
    ellipses a = 0.07, b = 0.035 moving at random velocities, and a sheared,
    rotating initial flow with noise, so that every advective and coupling term is
    active. Returns (case, (ux, uy, p), records)."""
    case = poiseuille(itot=itot, jtot=jtot, n=max(n, 1), a=0.07, b=0.035, Re=150.0, seed=seed)
    rng = np.random.default_rng(seed + 100)
    rec = case.particles[:n].copy()
    rec[:, F["ux"]] = rng.uniform(-0.1, 0.1, n)
    rec[:, F["uy"]] = rng.uniform(-0.1, 0.1, n)
    rec[:, F["vz"]] = rng.uniform(-0.5, 0.5, n)
    case.particles = rec
    ux, uy, p = (np.array(a, dtype=np.float64) for a in case.fluid())
    jj, ii = np.meshgrid(np.arange(jtot + 2), np.arange(itot + 1), indexing="ij")
    ux += 0.2 * np.sin(2 * np.pi * jj / jtot) * np.sin(np.pi * ii / itot) + 0.02 * rng.standard_normal(ux.shape)
    jj, ii = np.meshgrid(np.arange(jtot + 2), np.arange(itot + 2), indexing="ij")
    uy += 0.3 * np.cos(np.pi * (ii - 0.5) / itot) + 0.02 * rng.standard_normal(uy.shape)
    p += 0.05 * rng.standard_normal(p.shape)
    return case, (ux, uy, p), rec


def adjoint_couette(itot=256, jtot=512, n=8, a=0.06, b=0.03, seed=2, steps=400):
    """Couette flow (walls -0.5, 0.5, linear initial profile), Re = 100, with n ellipses
    whose centres are at least 4a apart: the configuration of the adjoint checks."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / itot
    xs, ys = place(n, a, 2.0, 2.0 * a, rng, 2 * dx)
    az = rng.uniform(0.0, math.pi, n)
    rec = particle_records(np.ones(n), np.full(n, a), np.full(n, b), xs, ys, az)
    return Case("couette_%dx%d_n%d" % (itot, jtot, n), itot, jtot, 2.0, 100.0, uy_wall=(-0.5, 0.5), particles=rec,
                couette_init=True, steps=steps)


def contact_cluster(itot=64, jtot=128, seed=7):
    """Small case with ellipses overlapping tip to tip, across the periodic
    boundary and into a wall, so that every branch of the collision model is
    exercised from the first step."""
    rng = np.random.default_rng(seed)
    den = [1.0, 1.1, 1.0, 1.05, 1.0, 1.0]
    a = [0.10, 0.09, 0.08, 0.10, 0.07, 0.06]
    b = [0.05, 0.06, 0.04, 0.10, 0.035, 0.03]
    x = [0.30, 0.485, 0.60, 0.15, 0.935, 0.60]
    y = [1.00, 1.01, 1.90, 1.50, 0.60, 0.02]
    az = [0.05, 0.1, 0.5 * math.pi + 0.1, 0.0, 0.08, 0.5 * math.pi - 0.05]
    ux = list(rng.uniform(-0.1, 0.1, 6))
    uy = list(rng.uniform(-0.1, 0.1, 6))
    vz = list(rng.uniform(-0.5, 0.5, 6))
    rec = particle_records(den, a, b, x, y, az, ux, uy, vz)
    return Case("contact_cluster_%dx%d" % (itot, jtot), itot, jtot, 2.0, 150.0, extfrcy=0.02, Fr=3.0, particles=rec,
                steps=20)


def batch_c5(count=64, seed=3, n_max=256, steps=300):
    """Many independent suspensions of uneven sizes: grids drawn from 128x256, 256x512,
    384x768 and 512x1024; ellipse counts proportional to the cell count (4 .. n_max =
    256); a = 0.04, aspect ratio U[1, 2.5], Re U[100, 400], Poiseuille forcing 8/Re,
    fluid at rest. 256 bounding discs of a = 0.04 would cover 64 % of the 1 x 2 domain,
    beyond what random sequential addition of discs reaches (about 55 %), so the
    ellipses themselves are kept apart (place_ellipses, clearance one cell)."""
    rng = np.random.default_rng(seed)
    grids = [(128, 256), (256, 512), (384, 768), (512, 1024)]
    max_cells = 512 * 1024
    out = []
    for k in range(count):
        itot, jtot = grids[int(rng.integers(len(grids)))]
        n = int(round(4 + (n_max - 4) * (itot * jtot) / max_cells))
        a = 0.04
        ar = rng.uniform(1.0, 2.5, n)
        Re = float(rng.uniform(100.0, 400.0))
        dx = 1.0 / itot
        az = rng.uniform(0.0, math.pi, n)
        xs, ys = place_ellipses(np.full(n, a), a / ar, az, 2.0, dx, rng, dx)
        rec = particle_records(np.ones(n), np.full(n, a), a / ar, xs, ys, az)
        out.append(Case("batch%02d_%dx%d_n%d" % (k, itot, jtot, n), itot, jtot, 2.0, Re, extfrcy=8.0 / Re,
                        particles=rec, steps=steps))
    return out


def adjoint_large(itot=2048, jtot=4096, n=2048, a=0.012, b=0.006, seed=1, steps=10):
    """2048 x 4096 channel with 2048 ellipses of aspect ratio 2 (about 4.6 % area, so
    the motion stays contact-free over the measured steps), fluid sheared by a
    uniform 0.3 in y: the large workload of the adjoint cost measurement."""
    c = poiseuille(itot=itot, jtot=jtot, n=n, a=a, b=b, Re=400.0, seed=seed, steps=steps)
    c.name = "adjoint_channel_%dx%d_n%d" % (itot, jtot, n)
    c.uy_offset = 0.3
    return c


CONFIGS = {
    "couette_circle": couette_circle,
    "poiseuille": poiseuille,
    "mixed_target": mixed_target,
    "contact_cluster": contact_cluster,
    "adjoint_couette": adjoint_couette,
    "adjoint_large": adjoint_large,
}
