"""GPU parity of the double-precision form at the sizes and lengths of the benchmark
configurations, against the C restatement (pinned bit-for-bit to the reference
build by tests/test_oracle.py), run with OpenMP over all host cores.

* 2048 x 4096 with 2048 ellipses (the mixed-precision target's workload): the first
  step from the seeded initial state; two steps from the state after 300 steps (at this
  grid the time step is diffusion-limited, 1.8e-5, so the flow is still weak there and
  the fixed point takes two sub-iterations); and two steps from a stirred state with
  ellipses in contact (a channel profile in the fluid, particles moving against it,
  128 ellipses pushed into overlap with a neighbour), where collisions act and the
  fixed point takes more sub-iterations;
* 512 x 1024 with 128 ellipses (plane Poiseuille suspension): 1000 steps, compared at
  steps 1, 200 and 1000;
* 64 x 128 Couette circle: every one of its 200 steps.

Every comparison covers u, v, p (mean removed) and all 30 particle fields. The
tolerances are the ones the double-precision form promises for the state (1e-11
relative after one step, 1e-8 after 200 steps); the record fields that are
intermediates of the step (forces, torques, integrals, increments) are held to 1e-10
where that is looser, and the 1000-step figure is printed and held to 1e-6.
"""
import os

import numpy as np
import pytest

from conftest import interior_p, rel_err
from ellipsesinflows_gb300 import PREC_MIXED, Simulation, cases
from ellipsesinflows_gb300.capi import F, FIELDS
from oracle import port

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-11
TOL_LONG = 1e-8
TOL_1000 = 1e-6
THREADS = os.cpu_count() or 1

# components of one vector quantity share a scale (a near-cancelling component is
# compared against the magnitude of the vector)
GROUPS = [("dx", "dy"), ("dux", "duy"), ("ux", "uy"), ("fux", "fuy"), ("iux0", "iuy0"), ("iux1", "iuy1"),
          ("cfx0", "cfy0"), ("cfx1", "cfy1")]


def field_errors(g, o):
    gu, gv, gp, _ = g.pull_fluid()
    ou, ov, op, _ = o.pull_fluid()
    return {"u": rel_err(gu, ou), "v": rel_err(gv, ov), "p": rel_err(interior_p(gp), interior_p(op))}


def particle_errors(gp, op):
    """max |difference| of every record field over the particles, relative to the largest
    magnitude of its group in the oracle (absolute where that magnitude is zero);
    positions and angles are compared absolutely (they are O(1))."""
    out = {}
    for f in FIELDS:
        d = float(np.max(np.abs(gp[:, F[f]] - op[:, F[f]]))) if len(op) else 0.0
        if f in ("x", "y", "az", "den", "a", "b"):
            out[f] = d
            continue
        group = next((gr for gr in GROUPS if f in gr), (f,))
        scale = max(float(np.max(np.abs(op[:, F[q]]))) for q in group) if len(op) else 0.0
        out[f] = d / scale if scale > 0 else d
    return out


# the state a step leaves (what the tolerances of the double-precision form are stated
# for); the other record fields are intermediates of the step (forces, torques, inertia
# integrals, increments), held to the stage tests' tolerance for sums over many cells or
# over a fixed-point iteration where that is looser
STATE = ("x", "y", "az", "ux", "uy", "vz")
TOL_INTERMEDIATE = 1e-10


def assert_state(g, o, tol, what):
    fe = field_errors(g, o)
    pe = particle_errors(g.pull_particles(), o.pull_particles())
    print("%s: fields %s, worst state field %s = %.3g, worst intermediate %s = %.3g" % (
        what, {k: "%.3g" % v for k, v in fe.items()}, max(STATE, key=pe.get), max(pe[f] for f in STATE),
        max((f for f in pe if f not in STATE), key=pe.get), max(v for f, v in pe.items() if f not in STATE)))
    bad = {k: v for k, v in fe.items() if v >= tol}
    bad.update({f: v for f, v in pe.items() if v >= (tol if f in STATE else max(tol, TOL_INTERMEDIATE))})
    assert not bad, (what, bad)


def pair_from(case, fluid, records):
    g = Simulation(case.config())
    g.push_fluid(*fluid)
    g.push_particles(records)
    o = port.PortSolver(case.config(), threads=THREADS)
    o.push_fluid(*fluid)
    o.push_particles(records)
    return g, o


def contacts(records):
    """particles with a non-zero collision force in the last evaluation at X^k"""
    return int(np.count_nonzero(np.abs(records[:, F["cfx0"]]) + np.abs(records[:, F["cfy0"]]) +
                                np.abs(records[:, F["ctz0"]])))


def test_c3_first_step_matches_oracle(gpu_lib):
    case = cases.mixed_target()
    g, o = pair_from(case, case.fluid(), case.particles)
    gs, os_ = g.step(), o.step()
    assert gs == os_, (gs, os_)
    assert_state(g, o, TOL_STEP, "2048x4096 step 1")


def stirred_contact_state(case, pairs=128, seed=5):
    """The workload's ellipses in a stirred channel: uy = 6 x (1 - x) (bulk velocity 1)
    plus noise in the fluid, particle velocities that differ from the fluid's, and
    `pairs` ellipses moved next to their nearest neighbour tip to tip: both turned to
    the direction between the centres, at a centre distance of 0.99 times the sum of
    the major semi-axes (a slight overlap at the tips, as in a collision)."""
    rng = np.random.default_rng(seed)
    ux, uy, p = (np.array(a) for a in case.fluid())
    xc = case.xc()
    uy[:, 1:-1] = 6.0 * xc[None, 1:-1] * (1.0 - xc[None, 1:-1])
    uy += 0.01 * rng.standard_normal(uy.shape)
    ux += 0.01 * rng.standard_normal(ux.shape)
    rec = case.particles.copy()
    n = len(rec)
    rec[:, F["uy"]] = 6.0 * rec[:, F["x"]] * (1.0 - rec[:, F["x"]]) + 0.05 * rng.standard_normal(n)
    rec[:, F["ux"]] = 0.05 * rng.standard_normal(n)
    rec[:, F["vz"]] = 0.5 * rng.standard_normal(n)
    moved = set()
    for k in rng.permutation(n):
        if len(moved) >= pairs:
            break
        if k in moved:
            continue
        dxs = rec[:, F["x"]] - rec[k, F["x"]]
        dys = rec[:, F["y"]] - rec[k, F["y"]]
        dys -= case.ly * np.round(dys / case.ly)
        d = np.hypot(dxs, dys)
        d[k] = np.inf
        m = int(np.argmin(d))
        if m in moved:
            continue
        dist = 0.99 * (rec[k, F["a"]] + rec[m, F["a"]])
        ex, ey = -dxs[m] / d[m], -dys[m] / d[m]   # unit vector from m to k
        x = rec[m, F["x"]] + dist * ex
        if not (rec[k, F["a"]] < x < 1.0 - rec[k, F["a"]]):
            continue
        rec[k, F["x"]] = x
        rec[k, F["y"]] = (rec[m, F["y"]] + dist * ey) % case.ly
        rec[k, F["az"]] = rec[m, F["az"]] = np.arctan2(ey, ex) % np.pi
        moved.update((k, m))
    return (ux, uy, p), rec


def test_c3_stirred_contact_steps_match_oracle(gpu_lib):
    case = cases.mixed_target()
    fluid, rec = stirred_contact_state(case)
    g, o = pair_from(case, fluid, rec)
    subs = []
    for k in range(2):
        gs, os_ = g.step(), o.step()
        assert gs == os_, (k, gs, os_)
        subs.append(gs)
        assert_state(g, o, TOL_STEP, "2048x4096 stirred with contacts, step %d" % (k + 1))
    n_contact = contacts(o.pull_particles())
    print("stirred state: sub-iterations per stage %s, ellipses in contact %d" % (subs, n_contact))
    assert n_contact >= 100
    assert max(max(s) for s in subs) >= 3


def test_c3_after_300_steps_match_oracle(gpu_lib):
    """Two steps from the state after 300 steps (taken from a mixed-precision run, which
    is only the source of the input state here)."""
    case = cases.mixed_target()
    src = Simulation.from_case(case, precision=PREC_MIXED)
    src.advance(300)
    ux, uy, p, _ = src.pull_fluid()
    rec = src.pull_particles()
    src.close()
    g, o = pair_from(case, (ux, uy, p), rec)
    subs = []
    for k in range(2):
        gs, os_ = g.step(), o.step()
        assert gs == os_, (k, gs, os_)
        subs.append(gs)
        assert_state(g, o, TOL_STEP, "2048x4096 developed, step %d" % (k + 1))
    print("state after 300 steps: sub-iterations per stage %s, ellipses in contact %d"
          % (subs, contacts(o.pull_particles())))


def test_c2_1000_steps_match_oracle(gpu_lib):
    case = cases.poiseuille()
    g, o = pair_from(case, case.fluid(), case.particles)
    for k in range(1, 1001):
        gs, os_ = g.step(), o.step()
        assert gs == os_, (k, gs, os_)
        if k == 1:
            assert_state(g, o, TOL_STEP, "512x1024 step 1")
        elif k == 200:
            assert_state(g, o, TOL_LONG, "512x1024 step 200")
        elif k == 1000:
            assert_state(g, o, TOL_1000, "512x1024 step 1000")


def test_couette_every_step_matches_oracle(gpu_lib):
    case = cases.couette_circle()
    g, o = pair_from(case, case.fluid(), case.particles)
    for k in range(1, case.steps + 1):
        gs, os_ = g.step(), o.step()
        assert gs == os_, (k, gs, os_)
        fe = field_errors(g, o)
        pe = particle_errors(g.pull_particles(), o.pull_particles())
        worst = max(list(fe.values()) + [pe[f] for f in ("x", "y", "az", "ux", "uy", "vz")])
        assert worst < (TOL_STEP if k == 1 else TOL_LONG), (k, fe, pe)
