"""Generate the golden vectors in tests/golden/ from the reference solver.

Run where the reference sources are available (it builds oracle/_ref/ from
them with oracle/ref/Makefile):

    python tests/golden/make_golden.py

Every fixture is the output of the reference's own code (compiled unmodified
with single-rank MPI/FFTW shims) for a seeded input described in the file.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ellipsesinflows_gb300 import cases  # noqa: E402
from oracle import build, ref  # noqa: E402


def ref_solver(case):
    variant = "couette" if case.uy_wall != (0.0, 0.0) else "default"
    if case.uy_wall not in ((0.0, 0.0), (-0.5, 0.5)):
        raise ValueError("the reference has fixed wall-velocity variants only")
    s = ref.RefSolver(case.itot, case.jtot, case.ly, case.Re, case.Fr, case.extfrcy, case.safefactors, variant=variant)
    s.set_fluid(*case.fluid())
    s.set_particles(case.particles)
    return s


def run_case(case, checkpoints):
    s = ref_solver(case)
    out = {}
    dts, subs = [], []
    nmax = max(checkpoints)
    for k in range(1, nmax + 1):
        subs.append(s.step())
        dts.append(s.dt)
        if k in checkpoints:
            ux, uy, p, psi = s.get_fluid()
            out["ux_%d" % k], out["uy_%d" % k], out["p_%d" % k] = ux, uy, p
            out["particles_%d" % k] = s.get_particles()
    out["dt"] = np.array(dts)
    out["substeps"] = np.array(subs, dtype=np.int32)
    return out


def geometry():
    """find_normal_t and the two weights on a seeded set of points and ellipses."""
    rng = np.random.default_rng(11)
    n = 400
    a = rng.uniform(0.02, 0.2, n)
    b = a / rng.uniform(1.0, 3.0, n)
    # points from deep inside to well outside, all quadrants
    ang = rng.uniform(0, 2 * np.pi, n)
    rad = rng.uniform(0.0, 2.0, n)
    x = rad * a * np.cos(ang)
    y = rad * b * np.sin(ang) * rng.uniform(0.5, 1.5, n)
    t = np.array([ref.find_normal_t(a[k], b[k], x[k], y[k]) for k in range(n)])
    px, py, az = rng.uniform(0.2, 0.8, n), rng.uniform(0.2, 1.8, n), rng.uniform(0, 2 * np.pi, n)
    h = 1.0 / 64
    qx = px + rng.uniform(-0.3, 0.3, n)
    qy = py + rng.uniform(-0.3, 0.3, n)
    sw = np.array([ref.s_weight(h, a[k], b[k], px[k], py[k], az[k], qx[k], qy[k]) for k in range(n)])
    vw = np.array([ref.v_weight(h, a[k], b[k], px[k], py[k], az[k], qx[k], qy[k]) for k in range(n)])
    return dict(a=a, b=b, x=x, y=y, t=t, px=px, py=py, az=az, h=np.array(h), qx=qx, qy=qy, s_weight=sw, v_weight=vw)


def main():
    if not build.build_ref():
        raise SystemExit("reference sources not found")
    c1 = cases.couette_circle()
    np.savez_compressed(os.path.join(HERE, "couette_circle_64x128.npz"), **run_case(c1, (1, 200)))
    cc = cases.contact_cluster()
    np.savez_compressed(os.path.join(HERE, "contact_cluster_64x128.npz"), **run_case(cc, (1, 20)))
    pc = cases.poiseuille(itot=64, jtot=128, n=6, a=0.08, b=0.05, seed=5)
    np.savez_compressed(os.path.join(HERE, "poiseuille_64x128_n6.npz"), **run_case(pc, (1, 10)))
    np.savez_compressed(os.path.join(HERE, "geometry.npz"), **geometry())
    for f in sorted(os.listdir(HERE)):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
