"""Central differences of the reference solver for the adjoint objective of the
256 x 512 Couette configuration.

Run where the reference sources are available (it builds oracle/_ref/ from them
with oracle/ref/Makefile):

    python tests/golden/make_adjoint_c4_fd.py

The reference's own integrate (src/main.c:13-55, compiled unmodified with
single-rank MPI/FFTW shims, the Couette boundary variant of its case 1 with walls
moving at -0.5 and 0.5) advances ellipsesinflows_gb300.cases.adjoint_couette (256 x
512, Re 100, 8 ellipses a = 0.06, b = 0.03 at least 4a apart) NSTEPS = 400 steps at
the fixed dt DT (half the reference's param_decide_dt of the initial state). The
objective is the mean ellipse x-centre plus the fluid's kinetic energy as the
reference logs it (check_energy, src/logging.c:130-172). The script records the
objective, the sub-iteration counts, and the central differences along seeded
directions of the initial angles and of the initial centres (step 1e-7, with the
sub-iteration counts of both perturbed runs). The runs go in parallel processes.
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ellipsesinflows_gb300 import cases  # noqa: E402
from ellipsesinflows_gb300.capi import F  # noqa: E402

NSTEPS = 400
SEED = 31
EPS = 1e-7
OUT = os.path.join(HERE, "adjoint_fd_c4_256x512.npz")


def grid(itot, jtot, ly):
    """DXF(1..itot), DXC(1..itot+1) and dy of set_coordinate (src/param/init.c:105-167)"""
    dx = 1.0 / itot
    xf = np.array([1.0 * (i - 1) * dx for i in range(1, itot + 2)])
    xf[0], xf[itot] = 0.0, 1.0
    xc = np.concatenate([[xf[0]], 0.5 * (xf[:-1] + xf[1:]), [xf[itot]]])
    return xf[1:] - xf[:-1], xc[1:] - xc[:-1], ly / jtot


def objective(ux, uy, rec, ly):
    """mean x-centre + kinetic energy (src/logging.c:130-172, summed over both components)"""
    jtot, itot = uy.shape[0] - 2, uy.shape[1] - 2
    dxf, dxc, dy = grid(itot, jtot, ly)
    ex = float(np.sum(0.5 * ux[1:-1, :] ** 2 * dxc[None, :]) * dy)
    ey = float(np.sum(0.5 * uy[1:-1, 1:-1] ** 2 * dxf[None, :]) * dy)
    return float(np.mean(rec[:, F["x"]])) + ex + ey


def inputs():
    """case, state, records and the seeded directions of the angles and the centres"""
    case = cases.adjoint_couette()
    state = tuple(np.array(a, dtype=np.float64) for a in case.fluid())
    rec = case.particles.copy()
    n = rec.shape[0]
    rng = np.random.default_rng(SEED)
    d_ang = np.zeros_like(rec)
    d_ang[:, F["az"]] = rng.standard_normal(n)
    d_cen = np.zeros_like(rec)
    d_cen[:, [F["x"], F["y"]]] = rng.standard_normal((n, 2))
    return case, state, rec, {"angles": d_ang, "centres": d_cen}


def time_step(case, state, rec):
    from oracle import ref
    s = ref.RefSolver(case.itot, case.jtot, case.ly, case.Re, case.Fr, case.extfrcy, case.safefactors,
                      variant="couette")
    s.set_fluid(*state)
    s.set_particles(rec)
    dt = 0.5 * s.decide_dt()
    # one step before the solver is released: the reference's fluid_finalise frees the
    # Poisson solver's buffers, which its first integrate allocates
    s.integrate()
    s.close()
    return dt


def run(args):
    """one reference run of NSTEPS steps from (state, rec); returns (objective, substeps)"""
    case, state, rec, dt = args
    from oracle import ref
    s = ref.RefSolver(case.itot, case.jtot, case.ly, case.Re, case.Fr, case.extfrcy, case.safefactors,
                      variant="couette")
    s.set_fluid(*state)
    s.set_particles(rec)
    s.dt = dt
    subs = [s.integrate_counted() for _ in range(NSTEPS)]
    ux, uy, _, _ = s.get_fluid()
    out = objective(ux, uy, s.get_particles(), case.ly)
    s.close()
    return out, np.array(subs, dtype=np.int32)


def main():
    from oracle import build
    if not build.build_ref():
        raise SystemExit("reference sources not found")
    case, state, rec, dirs = inputs()
    dt = time_step(case, state, rec)
    jobs = [(case, state, rec, dt)]
    names = sorted(dirs)
    for name in names:
        for sgn in (1, -1):
            jobs.append((case, state, rec + sgn * EPS * dirs[name], dt))
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        res = pool.map(run, jobs)
    base, subs = res[0]
    out = {"loss": np.array(base), "substeps": subs, "nsteps": np.array(NSTEPS), "dt": np.array(dt),
           "eps": np.array(EPS)}
    for k, name in enumerate(names):
        (lp, sp), (lm, sm) = res[1 + 2 * k], res[2 + 2 * k]
        out["fd_" + name] = np.array((lp - lm) / (2 * EPS))
        out["substeps_" + name] = np.stack([sp, sm])
        print(name, out["fd_" + name], "substeps kept:", np.array_equal(sp, subs) and np.array_equal(sm, subs))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, "objective", base, "dt", dt)


if __name__ == "__main__":
    main()
