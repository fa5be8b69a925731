"""GPU parity: the CUDA library against the CPU oracles.

Stage by stage against the C restatement (which is pinned bit-for-bit to the
reference build), whole steps against the golden vectors produced by the
reference build, and at larger sizes against the restatement and through
size-independent properties. Tolerances are the ones the FP64 form promises:
1e-11 relative in u, v, p (mean removed) and particle centre/angle after one
step, 1e-8 after 200 steps; stage-level outputs within 1e-12 (fields) or 1e-10
(quantities that involve a sum over many cells).
"""
import numpy as np
import pytest

from conftest import interior_p, rel_err
from ellipsesinflows_gb300 import Simulation, cases
from ellipsesinflows_gb300.capi import F
from oracle import port

pytestmark = pytest.mark.gpu

TOL_FIELD = 1e-12
TOL_SUM = 1e-10
TOL_STEP = 1e-11
TOL_LONG = 1e-8


def pair(case):
    g = Simulation(case.config())
    g.push_fluid(*case.fluid())
    g.push_particles(case.particles)
    o = port.PortSolver(case.config(), threads=4)
    o.push_fluid(*case.fluid())
    o.push_particles(case.particles)
    return g, o


def assert_fluid(g, o, tol=TOL_FIELD, tol_p=None, psi=False):
    gu, gv, gp, gpsi = g.pull_fluid()
    ou, ov, op, opsi = o.pull_fluid()
    assert rel_err(gu, ou) < tol, rel_err(gu, ou)
    assert rel_err(gv, ov) < tol, rel_err(gv, ov)
    tp = tol if tol_p is None else tol_p
    assert rel_err(interior_p(gp), interior_p(op)) < tp, rel_err(interior_p(gp), interior_p(op))
    if psi:
        assert rel_err(interior_p(gpsi), interior_p(opsi)) < tp


# components of one vector quantity share a scale: a near-cancelling component
# (e.g. the x-momentum of a particle carried by a y-directed shear flow) is
# compared against the magnitude of the vector, not against itself
GROUPS = [("iux0", "iuy0"), ("iux1", "iuy1"), ("fux", "fuy"), ("cfx0", "cfy0"), ("cfx1", "cfy1"),
          ("ux", "uy"), ("x",), ("y",)]


def particle_err(gp, op, fields):
    out = {}
    for f in fields:
        group = next((g for g in GROUPS if f in g), (f,))
        scale = max(np.max(np.abs(op[:, F[g]])) for g in group)
        diff = np.max(np.abs(gp[:, F[f]] - op[:, F[f]]))
        out[f] = diff / scale if scale > 0 else diff
    return out


@pytest.mark.parametrize("builder", [
    lambda: cases.contact_cluster(),
    lambda: cases.couette_circle(),
    lambda: cases.poiseuille(itot=96, jtot=192, n=10, a=0.05, b=0.03, seed=9),
], ids=["contact_cluster", "couette_circle", "poiseuille_96x192"])
def test_stages_match_oracle(builder, gpu_lib):
    case = builder()
    g, o = pair(case)
    dt = 1.0e-3
    g.dt = dt
    o.dt = dt
    for rk in range(3):
        g.reset_particle_increments(); o.reset_particle_increments()
        g.compute_inertia(0); o.compute_inertia(0)
        e = particle_err(g.pull_particles(), o.pull_particles(), ["iux0", "iuy0", "ivz0"])
        assert max(e.values()) < TOL_SUM, e
        g.update_velocity(rk); o.update_velocity(rk)
        assert_fluid(g, o)
        for a, b in zip(g.pull_src(), o.pull_src()):
            assert rel_err(a, b) < TOL_FIELD
        g.exchange_momentum(); o.exchange_momentum()
        for a, b in zip(g.pull_ibm_fields(), o.pull_ibm_fields()):
            assert rel_err(a, b) < TOL_FIELD, rel_err(a, b)
        e = particle_err(g.pull_particles(), o.pull_particles(), ["fux", "fuy", "tvz"])
        assert max(e.values()) < TOL_SUM, e
        g.update_momentum_field(); o.update_momentum_field()
        assert_fluid(g, o)
        g.compute_potential(rk); o.compute_potential(rk)
        g.correct_velocity(rk); o.correct_velocity(rk)
        assert_fluid(g, o, tol=TOL_STEP)
        g.update_pressure(); o.update_pressure()
        assert_fluid(g, o, tol=TOL_STEP, psi=True)
        g.compute_collision_force(0); o.compute_collision_force(0)
        g.compute_inertia(1); o.compute_inertia(1)
        g.compute_collision_force(1); o.compute_collision_force(1)
        e = particle_err(g.pull_particles(), o.pull_particles(), ["cfx0", "cfy0", "ctz0", "cfx1", "cfy1", "ctz1",
                                                                  "iux1", "iuy1", "ivz1"])
        assert max(e.values()) < TOL_SUM, e
        rg, ro = g.increment_particles(rk), o.increment_particles(rk)
        assert abs(rg - ro) <= 1e-10 * max(abs(ro), 1e-12)
        g.update_particles(); o.update_particles()
        e = particle_err(g.pull_particles(), o.pull_particles(), ["x", "y", "az", "ux", "uy", "vz"])
        assert max(e.values()) < TOL_STEP, e


def test_decide_dt_matches_oracle(gpu_lib):
    case = cases.contact_cluster()
    g, o = pair(case)
    for _ in range(2):
        o.step()
    ux, uy, p, _ = o.pull_fluid()
    g.push_fluid(ux, uy, p)
    g.push_particles(o.pull_particles())
    assert g.decide_dt() == o.decide_dt()


@pytest.mark.parametrize("name,builder", [
    ("couette_circle_64x128.npz", lambda: cases.couette_circle()),
    ("contact_cluster_64x128.npz", lambda: cases.contact_cluster()),
    ("poiseuille_64x128_n6.npz", lambda: cases.poiseuille(itot=64, jtot=128, n=6, a=0.08, b=0.05, seed=5)),
])
def test_first_step_matches_reference_golden(name, builder, golden, gpu_lib):
    gref = golden(name)
    case = builder()
    g = Simulation.from_case(case)
    sub = g.step()
    assert sub == list(gref["substeps"][0])
    assert g.dt == gref["dt"][0]
    ux, uy, p, _ = g.pull_fluid()
    assert rel_err(ux, gref["ux_1"]) < TOL_STEP
    assert rel_err(uy, gref["uy_1"]) < TOL_STEP
    assert rel_err(interior_p(p), interior_p(gref["p_1"])) < TOL_STEP
    P, R = g.pull_particles(), gref["particles_1"]
    for f in ("x", "y", "az"):
        assert np.max(np.abs(P[:, F[f]] - R[:, F[f]])) < TOL_STEP * max(1.0, np.max(np.abs(R[:, F[f]])))


def test_couette_200_steps_match_reference_golden(golden, gpu_lib):
    gref = golden("couette_circle_64x128.npz")
    g = Simulation.from_case(cases.couette_circle())
    for _ in range(200):
        g.step()
    ux, uy, p, _ = g.pull_fluid()
    assert rel_err(ux, gref["ux_200"]) < TOL_LONG
    assert rel_err(uy, gref["uy_200"]) < TOL_LONG
    assert rel_err(interior_p(p), interior_p(gref["p_200"])) < TOL_LONG
    P, R = g.pull_particles(), gref["particles_200"]
    for f in ("x", "y", "az"):
        assert abs(P[0, F[f]] - R[0, F[f]]) < TOL_LONG


def test_contact_cluster_20_steps_match_reference_golden(golden, gpu_lib):
    gref = golden("contact_cluster_64x128.npz")
    g = Simulation.from_case(cases.contact_cluster())
    for _ in range(20):
        g.step()
    ux, uy, p, _ = g.pull_fluid()
    assert rel_err(ux, gref["ux_20"]) < TOL_LONG
    assert rel_err(uy, gref["uy_20"]) < TOL_LONG
    P, R = g.pull_particles(), gref["particles_20"]
    for f in ("x", "y", "az"):
        assert np.max(np.abs(P[:, F[f]] - R[:, F[f]])) < TOL_LONG


def test_advance_equals_repeated_steps(gpu_lib):
    case = cases.contact_cluster()
    a = Simulation.from_case(case)
    b = Simulation.from_case(case)
    a.advance(3)
    for _ in range(3):
        b.step()
    for x, y in zip(a.pull_fluid(), b.pull_fluid()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.pull_particles(), b.pull_particles())
    sa, ta = a.time_state()
    sb, tb = b.time_state()
    assert sa == sb == 3 and ta == tb


def test_step_graph_equals_host_driven_steps_mixed(gpu_lib):
    """eif_advance runs each step as one CUDA graph with a device-driven sub-iteration
    loop; step() drives the same kernels from the host. Both give identical bits."""
    from ellipsesinflows_gb300 import PREC_MIXED
    case = cases.contact_cluster()
    a = Simulation.from_case(case, precision=PREC_MIXED)
    b = Simulation.from_case(case, precision=PREC_MIXED)
    a.advance(4)
    subs = [b.step() for _ in range(4)]
    assert max(max(s) for s in subs) >= 2   # the loop ran more than once somewhere
    for x, y in zip(a.pull_fluid(), b.pull_fluid()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.pull_particles(), b.pull_particles())
    assert a.time_state() == b.time_state()


def test_repush_between_steps_equals_uninterrupted_advance(gpu_lib):
    """A driver that pulls the state and pushes it back between steps (same particle
    count, so the device buffers and step graphs are kept) gets the same bits as an
    uninterrupted advance."""
    from ellipsesinflows_gb300 import PREC_MIXED
    for prec in (None, PREC_MIXED):
        case = cases.contact_cluster()
        a = Simulation.from_case(case) if prec is None else Simulation.from_case(case, precision=prec)
        b = Simulation.from_case(case) if prec is None else Simulation.from_case(case, precision=prec)
        a.advance(3)
        for _ in range(3):
            ux, uy, p, _ = b.pull_fluid()
            parts = b.pull_particles()
            b.push_fluid(ux, uy, p)
            b.push_particles(parts)
            b.advance(1)
        for x, y in zip(a.pull_fluid(), b.pull_fluid()):
            assert np.array_equal(x, y)
        assert np.array_equal(a.pull_particles(), b.pull_particles())


def test_page_locked_transfers_equal_pageable(gpu_lib):
    """Page-locked host arrays are moved by the library's transfer kernels, pageable ones
    by pitched copies: the same state goes in and comes out either way."""
    torch = pytest.importorskip("torch")
    from ellipsesinflows_gb300 import PREC_MIXED

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        out = t.numpy()
        out[...] = a
        return out

    case = cases.contact_cluster()
    a = Simulation.from_case(case, precision=PREC_MIXED)
    b = Simulation.from_case(case, precision=PREC_MIXED)
    a.advance(1)
    ux, uy, p, _ = a.pull_fluid()
    parts = a.pull_particles()
    b.push_fluid(pinned(ux), pinned(uy), pinned(p))
    b.push_particles(pinned(parts))
    outs = tuple(pinned(np.full_like(x, np.nan)) for x in (ux, uy, p, p))
    hp = pinned(np.full_like(parts, np.nan))
    b.pull_fluid(out=outs)
    b.pull_particles(out=hp)
    for x, y in zip(a.pull_fluid()[:3], outs[:3]):   # psi is not part of the pushed state
        assert np.array_equal(x, y)
    assert np.array_equal(parts, hp)
    a.advance(2)
    b.advance(2)
    b.pull_fluid(out=outs)
    b.pull_particles(out=hp)
    for x, y in zip(a.pull_fluid(), outs):
        assert np.array_equal(x, y)
    assert np.array_equal(a.pull_particles(), hp)


def test_runs_are_deterministic(gpu_lib):
    case = cases.poiseuille(itot=128, jtot=256, n=16, a=0.04, b=0.02, seed=3)
    runs = []
    for _ in range(2):
        g = Simulation.from_case(case)
        g.advance(2)
        runs.append((g.pull_fluid(), g.pull_particles()))
    for x, y in zip(runs[0][0], runs[1][0]):
        assert np.array_equal(x, y)
    assert np.array_equal(runs[0][1], runs[1][1])


@pytest.mark.parametrize("shape", [(128, 96), (384, 768)])
def test_odd_sizes_match_oracle(shape, gpu_lib):
    """radix-3 DCT length (384), and a column length without a 16-row block (96 -> 8-row blocks)."""
    itot, jtot = shape
    case = cases.poiseuille(itot=itot, jtot=jtot, n=4, a=0.06, b=0.03, seed=2)
    g, o = pair(case)
    g.step(); o.step()
    assert_fluid(g, o, tol=TOL_STEP)


def test_poiseuille_c2_one_step_matches_oracle(gpu_lib):
    """The 512 x 1024, 128-ellipse configuration: one step against the restatement."""
    case = cases.poiseuille()
    g, o = pair(case)
    assert g.step() == o.step()
    assert_fluid(g, o, tol=TOL_STEP)
    e = particle_err(g.pull_particles(), o.pull_particles(), ["x", "y", "az", "ux", "uy", "vz"])
    assert max(e.values()) < TOL_STEP, e


def test_full_size_properties(gpu_lib):
    """2048 x 4096 with 2048 ellipses: projection leaves a divergence-free field,
    state stays finite, and the solution is reproducible."""
    case = cases.mixed_target()
    g = Simulation.from_case(case)
    g.advance(1)
    divmax, divsum = g.divergence()
    ux, uy, p, _ = g.pull_fluid()
    assert np.all(np.isfinite(ux)) and np.all(np.isfinite(uy)) and np.all(np.isfinite(p))
    umax = max(np.abs(ux).max(), np.abs(uy).max())
    assert divmax < 1e-8 * max(umax, 1e-3) * case.itot
    P = g.pull_particles()
    assert np.all(np.isfinite(P))
    assert np.all((P[:, F["y"]] >= 0) & (P[:, F["y"]] <= case.ly))
