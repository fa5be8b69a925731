"""The reference central differences of the adjoint checks, reproduced by the C
restatement oracle on the CPU (no GPU): the fixture in tests/golden/ comes from the
reference's own step, and the restatement is bit-identical to it, so the same
perturbed runs give the same central differences."""
import importlib.util
import os

import numpy as np

from oracle import port

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    spec = importlib.util.spec_from_file_location("make_adjoint_fd", os.path.join(HERE, "golden", "make_adjoint_fd.py"))
    G = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(G)
    return G


def _run(G, case, state, rec):
    s = port.PortSolver(case.config(), threads=1)
    s.push_fluid(*state)
    s.push_particles(rec)
    s.dt = G.DT
    subs = [s.integrate() for _ in range(G.NSTEPS)]
    out = s.pull_fluid()[:3] + (s.pull_particles(),)
    s.close()
    return out, np.array(subs, dtype=np.int32)


def test_port_reproduces_reference_central_differences():
    G = _golden()
    ref = np.load(os.path.join(HERE, "golden", "adjoint_fd_64x128.npz"))
    case, state, rec, w, dirs = G.inputs()
    out, subs = _run(G, case, state, rec)
    assert np.array_equal(subs, ref["substeps"])
    assert G.loss(out, w) == float(ref["loss"])
    for name in ("all", "positions"):
        d, eps = dirs[name], float(ref["eps_" + name])
        vals = []
        for sgn in (1, -1):
            pert = tuple(a + sgn * eps * e for a, e in zip(state + (rec,), d))
            o, sb = _run(G, case, pert[:3], pert[3])
            assert np.array_equal(sb, ref["substeps_" + name][0 if sgn > 0 else 1])
            vals.append(G.loss(o, w))
        assert (vals[0] - vals[1]) / (2 * eps) == float(ref["fd_" + name])


def test_port_reproduces_reference_c4_objective_differences():
    """The 256 x 512 Couette fixture (400 steps, objective mean x-centre + kinetic
    energy): the restatement gives the reference's objective, sub-iteration counts and
    central difference along the angle direction bit for bit."""
    import os as _os
    spec = importlib.util.spec_from_file_location("make_c4", os.path.join(HERE, "golden", "make_adjoint_c4_fd.py"))
    G = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(G)
    ref = np.load(os.path.join(HERE, "golden", "adjoint_fd_c4_256x512.npz"))
    case, state, rec, dirs = G.inputs()
    dt = float(ref["dt"])

    def run(r):
        s = port.PortSolver(case.config(), threads=_os.cpu_count() or 1)
        s.push_fluid(*state)
        s.push_particles(r)
        s.dt = dt
        subs = [s.integrate() for _ in range(G.NSTEPS)]
        ux, uy, _, _ = s.pull_fluid()
        out = G.objective(ux, uy, s.pull_particles(), case.ly)
        s.close()
        return out, np.array(subs, dtype=np.int32)

    base, subs = run(rec)
    assert np.array_equal(subs, ref["substeps"])
    assert base == float(ref["loss"])
    eps = float(ref["eps"])
    (vp, sp), (vm, sm) = run(rec + eps * dirs["angles"]), run(rec - eps * dirs["angles"])
    assert np.array_equal(sp, ref["substeps_angles"][0]) and np.array_equal(sm, ref["substeps_angles"][1])
    assert (vp - vm) / (2 * eps) == float(ref["fd_angles"])
