"""Central differences of the reference solver for the adjoint checks.

Run where the reference sources are available (it builds oracle/_ref/ from them
with oracle/ref/Makefile):

    python tests/golden/make_adjoint_fd.py

The reference's own integrate (src/main.c:13-55, compiled unmodified with
single-rank MPI/FFTW shims) advances the adjoint channel inputs
(ellipsesinflows_gb300.cases.adjoint_channel: 64x128, 8 moving ellipses, walls at
rest) NSTEPS steps at the fixed dt DT. For a linear functional of the final
fluid fields and particle states (weights from a seeded generator) the script
records the central difference along seeded directions of the initial fields,
particle positions and particle velocities, with the sub-iteration counts of the
base and perturbed runs. The GPU adjoint's directional derivatives are compared
with these values (tests/test_gpu_adjoint.py).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ellipsesinflows_gb300 import cases  # noqa: E402
from ellipsesinflows_gb300.capi import F, NFIELDS  # noqa: E402
from oracle import build, ref  # noqa: E402

NSTEPS = 8
DT = 2e-3
SEED = 21
DIFF = [F[k] for k in ("x", "y", "az", "ux", "uy", "vz")]


def inputs():
    """case, state, records, loss weights and directions (all seeded)"""
    case, state, rec = cases.adjoint_channel()
    it, jt = case.itot, case.jtot
    sx, sy = (jt + 2, it + 1), (jt + 2, it + 2)
    n = rec.shape[0]
    rng = np.random.default_rng(SEED)
    cx, cy, cp = rng.standard_normal(sx), rng.standard_normal(sy), rng.standard_normal(sy)
    cp[0, :] = cp[-1, :] = 0.
    cp[:, 0] = cp[:, -1] = 0.
    cp[1:-1, 1:-1] -= cp[1:-1, 1:-1].mean()
    cr = np.zeros((n, NFIELDS))
    cr[:, DIFF] = rng.standard_normal((n, len(DIFF)))
    z = (np.zeros(sx), np.zeros(sy), np.zeros(sy), np.zeros((n, NFIELDS)))
    dpos = np.zeros((n, NFIELDS))
    dpos[:, [F["x"], F["y"], F["az"]]] = rng.standard_normal((n, 3))
    dvel = np.zeros((n, NFIELDS))
    dvel[:, [F["ux"], F["uy"], F["vz"]]] = rng.standard_normal((n, 3))
    dirs = {
        "all": (rng.standard_normal(sx), rng.standard_normal(sy), rng.standard_normal(sy), z[3]),
        "uy": (z[0], rng.standard_normal(sy), z[2], z[3]),
        "positions": (z[0], z[1], z[2], dpos),
        "velocities": (z[0], z[1], z[2], dvel),
    }
    return case, state, rec, (cx, cy, cp, cr), dirs


def ref_run(case, state, rec):
    s = ref.RefSolver(case.itot, case.jtot, case.ly, case.Re, case.Fr, case.extfrcy, case.safefactors)
    s.set_fluid(*state)
    s.set_particles(rec)
    s.dt = DT
    subs = []
    for _ in range(NSTEPS):
        subs.append(s.integrate_counted())
    ux, uy, p, _ = s.get_fluid()
    out = (ux, uy, p, s.get_particles())
    s.close()
    return out, np.array(subs, dtype=np.int32)


def loss(out, w):
    return sum(float(np.sum(o * c)) for o, c in zip(out, w))


def main():
    if not build.build_ref():
        raise SystemExit("reference sources not found")
    case, state, rec, w, dirs = inputs()
    out, subs = ref_run(case, state, rec)
    res = {"loss": np.array(loss(out, w)), "substeps": subs, "nsteps": np.array(NSTEPS), "dt": np.array(DT)}
    for name, d in dirs.items():
        eps = 1e-7 if name == "positions" else 1e-5
        vals, ss = [], []
        for sgn in (1, -1):
            pert = tuple(a + sgn * eps * e for a, e in zip(state + (rec,), d))
            o, sb = ref_run(case, pert[:3], pert[3])
            vals.append(loss(o, w))
            ss.append(sb)
        res["fd_" + name] = np.array((vals[0] - vals[1]) / (2 * eps))
        res["eps_" + name] = np.array(eps)
        res["substeps_" + name] = np.stack(ss)
        print(name, res["fd_" + name], "substeps kept:", all(np.array_equal(x, subs) for x in ss))
    np.savez_compressed(os.path.join(HERE, "adjoint_fd_64x128.npz"), **res)


if __name__ == "__main__":
    main()
