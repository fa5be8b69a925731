"""Discrete adjoint of the double-precision step (dt fixed).

The gradient of a linear functional of the state after N steps, taken through
the transposed steps (eif_adjoint_* behind adjoint.Steps), is checked against
central differences of the same forward map along random directions of the
initial fields, of the particle positions and velocities, and of the wall
velocities. Coupled mode: particles move, contact-free. Frozen mode: particle
records are parameters. The bar is a relative difference of 1e-5; the central
difference itself is accurate to about 1e-9 at the steps chosen (truncation
O(eps^2), round-off 1e-16 |L| / eps). A central difference is only comparable
when both perturbed runs take the sub-iteration counts of the recorded run (a
different count changes the step by up to the fixed point's 1e-8 tolerance); the
tests check that.
"""
import ctypes

import numpy as np
import pytest
import torch

from ellipsesinflows_gb300 import EifError, PREC_MIXED, Simulation, cases
from ellipsesinflows_gb300.adjoint import ADJOINT_COUPLED, ADJOINT_FROZEN, DIFF_FIELDS, Steps
from ellipsesinflows_gb300.capi import F, NFIELDS

pytestmark = pytest.mark.gpu

TOL_FD = 1e-5
EPS = (1e-5, 3e-6, 3e-5)
# The integration boxes of the reference (auxiliary.c:11-17) move in whole cells
# with the particles and cut the weights off (by about 6e-6 in the volume weight
# three cells outside), so the forward map has small jumps where a box shifts.
# Perturbed positions that make a box shift at another step than in the recorded
# run give a central difference that is no derivative; the chance of that scales
# with the step, so position directions use small steps.
EPS_POS = (1e-7, 3e-8, 3e-7)
DT = 2e-3


def make_case(n_particles=8, itot=64, jtot=128, seed=11, wall=(-0.1, 0.2)):
    case, state, rec = cases.adjoint_channel(n_particles, itot, jtot, seed)
    rng = np.random.default_rng(seed + 200)
    cfg = case.config()
    cfg.uy_wall[0], cfg.uy_wall[1] = wall
    return cfg, state, rec, rng


def new_sim(cfg, wall=None):
    c = type(cfg)()
    ctypes.memmove(ctypes.addressof(c), ctypes.addressof(cfg), ctypes.sizeof(cfg))
    if wall is not None:
        c.uy_wall[0], c.uy_wall[1] = wall
    return Simulation(c)


def loss_weights(sim, n, rng):
    sx, sy = sim.shapes()
    cx, cy, cp = rng.standard_normal(sx), rng.standard_normal(sy), rng.standard_normal(sy)
    # pressure enters through its differences only: zero weight on the copies and mean-free
    cp[0, :] = cp[-1, :] = 0.
    cp[:, 0] = cp[:, -1] = 0.
    cp[1:-1, 1:-1] -= cp[1:-1, 1:-1].mean()
    cr = np.zeros((n, NFIELDS))
    cr[:, DIFF_FIELDS] = rng.standard_normal((n, len(DIFF_FIELDS)))
    return cx, cy, cp, cr


def run(sim, state, rec, nsteps, dt, mode):
    """forward map; returns the state and the sub-iteration counts of every stage"""
    sim.push_fluid(*state)
    sim.push_particles(rec)
    sim.dt = dt
    subs = []
    for _ in range(nsteps):
        if mode == ADJOINT_COUPLED:
            subs.append(tuple(sim.integrate()))
        else:
            sim.adjoint_forward(record=False)
    return sim.pull_fluid()[:3] + (sim.pull_particles(),), subs


def loss(out, w):
    return sum(float(np.sum(o * c)) for o, c in zip(out, w))


def gradients(sim, state, rec, w, nsteps, every, mode):
    t = [torch.tensor(a, requires_grad=True) for a in state + (rec,)]
    wall = torch.tensor([sim.cfg.uy_wall[0], sim.cfg.uy_wall[1]], dtype=torch.float64, requires_grad=True)
    out = Steps.apply(t[0], t[1], t[2], t[3], wall, sim, nsteps, every, mode)
    L = sum((o * torch.from_numpy(c)).sum() for o, c in zip(out, w))
    L.backward()
    return [a.grad.numpy().copy() for a in t] + [wall.grad.numpy().copy()], float(L.detach())


def directions(sim, n, rng, mode):
    sx, sy = sim.shapes()
    z = (np.zeros(sx), np.zeros(sy), np.zeros(sy), np.zeros((n, NFIELDS)))
    out = {
        "all": (rng.standard_normal(sx), rng.standard_normal(sy), rng.standard_normal(sy), z[3]),
        "ux": (rng.standard_normal(sx), z[1], z[2], z[3]),
        "p": (z[0], z[1], rng.standard_normal(sy), z[3]),
    }
    if mode == ADJOINT_COUPLED and n:
        dpos = np.zeros((n, NFIELDS))
        dpos[:, [F["x"], F["y"], F["az"]]] = rng.standard_normal((n, 3))
        dvel = np.zeros((n, NFIELDS))
        dvel[:, [F["ux"], F["uy"], F["vz"]]] = rng.standard_normal((n, 3))
        out["positions"] = (z[0], z[1], z[2], dpos)
        out["velocities"] = (z[0], z[1], z[2], dvel)
    return out


def fd_along(cfg, state, rec, w, nsteps, dt, mode, d=None, dwall=None, ref_subs=None):
    """central difference of the loss along d (state) or dwall (wall velocities);
    tries a few step sizes until both runs keep the recorded sub-iteration counts"""
    moves_particles = d is not None and bool(d[3][:, [F["x"], F["y"], F["az"]]].any())
    for eps in (EPS_POS if moves_particles else EPS):
        vals, subs = [], []
        for sgn in (1, -1):
            if dwall is None:
                sim = new_sim(cfg)
                pert = tuple(s + sgn * eps * e for s, e in zip(state + (rec,), d))
            else:
                wall = (cfg.uy_wall[0] + sgn * eps * dwall[0], cfg.uy_wall[1] + sgn * eps * dwall[1])
                sim = new_sim(cfg, wall)
                pert = state + (rec,)
            if mode == ADJOINT_FROZEN:
                sim.push_fluid(*pert[:3])
                sim.push_particles(pert[3])
                sim.adjoint_begin(1, ADJOINT_FROZEN)
            out, sb = run(sim, pert[:3], pert[3], nsteps, dt, mode)
            sim.close()
            vals.append(loss(out, w))
            subs.append(sb)
        if ref_subs is None or (subs[0] == ref_subs and subs[1] == ref_subs):
            return (vals[0] - vals[1]) / (2 * eps)
    pytest.fail("no step size kept the sub-iteration counts")


def check(cfg, state, rec, w, grads, nsteps, dt, mode, rng, ref_subs):
    n = rec.shape[0]
    sim = new_sim(cfg)
    ref = None
    for name, d in directions(sim, n, rng, mode).items():
        fd = fd_along(cfg, state, rec, w, nsteps, dt, mode, d=d, ref_subs=ref_subs)
        adj = sum(float(np.sum(g * e)) for g, e in zip(grads[:4], d))
        ref = abs(fd) if ref is None else ref
        # without particles the state after a step does not depend on the initial
        # pressure at all (the projection removes G p0 and the pressure update
        # subtracts p0 again): that derivative is compared on the all-field scale
        scale = max(abs(fd), ref) if name == "p" else abs(fd)
        print("adjoint vs central difference [%s]: %.15e %.15e rel %.2e" % (name, adj, fd, abs(adj - fd) / scale))
        assert abs(adj - fd) <= TOL_FD * scale, (name, adj, fd, abs(adj - fd) / scale)
    dwall = rng.standard_normal(2)
    fd = fd_along(cfg, state, rec, w, nsteps, dt, mode, dwall=dwall, ref_subs=ref_subs)
    adj = float(np.dot(grads[4], dwall))
    print("adjoint vs central difference [wall]: %.15e %.15e rel %.2e" % (adj, fd, abs(adj - fd) / abs(fd)))
    assert abs(adj - fd) <= TOL_FD * abs(fd), ("wall", adj, fd)
    sim.close()


@pytest.mark.parametrize("n_particles", [8, 0])
def test_coupled_adjoint_matches_central_differences(n_particles):
    cfg, state, rec, rng = make_case(n_particles)
    sim = new_sim(cfg)
    w = loss_weights(sim, n_particles, rng)
    nsteps = 8
    out, subs = run(sim, state, rec, nsteps, DT, ADJOINT_COUPLED)
    grads, L = gradients(sim, state, rec, w, nsteps, 3, ADJOINT_COUPLED)
    # the forward value of the autograd function is the plain forward map
    assert L == pytest.approx(loss(out, w), rel=1e-14)
    check(cfg, state, rec, w, grads, nsteps, DT, ADJOINT_COUPLED, rng, subs)
    sim.close()


@pytest.mark.parametrize("n_particles", [8, 0])
def test_frozen_adjoint_matches_central_differences(n_particles):
    cfg, state, rec, rng = make_case(n_particles, seed=12)
    sim = new_sim(cfg)
    w = loss_weights(sim, n_particles, rng)
    nsteps = 10
    sim.push_fluid(*state)
    sim.push_particles(rec)
    sim.dt = DT
    grads, L = gradients(sim, state, rec, w, nsteps, 4, ADJOINT_FROZEN)
    out, _ = run(sim, state, rec, nsteps, DT, ADJOINT_FROZEN)
    assert L == pytest.approx(loss(out, w), rel=1e-14)
    check(cfg, state, rec, w, grads, nsteps, DT, ADJOINT_FROZEN, rng, None)
    sim.close()


def test_adjoint_gradients_do_not_depend_on_checkpoint_spacing():
    cfg, state, rec, rng = make_case(6, seed=5)
    sim = new_sim(cfg)
    w = loss_weights(sim, 6, rng)
    sim.push_fluid(*state)
    sim.push_particles(rec)
    sim.dt = DT
    g1, _ = gradients(sim, state, rec, w, 6, 1, ADJOINT_COUPLED)
    g6, _ = gradients(sim, state, rec, w, 6, 6, ADJOINT_COUPLED)
    g4, _ = gradients(sim, state, rec, w, 6, 4, ADJOINT_COUPLED)
    for a, b, c in zip(g1, g6, g4):
        # each segment is recomputed from a bit-exact checkpoint: same tape, same bits
        assert np.array_equal(a, b) and np.array_equal(a, c)
    sim.close()


def test_adjoint_forward_is_the_step():
    # the recorded forward of the coupled mode is eif_integrate with the same dt
    cfg, state, rec, rng = make_case(8, seed=3)
    a, b = new_sim(cfg), new_sim(cfg)
    for s in (a, b):
        s.push_fluid(*state)
        s.push_particles(rec)
        s.dt = DT
    a.adjoint_begin(3)
    subs = []
    for _ in range(3):
        a.adjoint_forward(record=True)
        subs.append(b.integrate())
    for x, y in zip(a.pull_fluid()[:3], b.pull_fluid()[:3]):
        assert np.array_equal(x, y)
    assert np.array_equal(a.pull_particles(), b.pull_particles())
    assert a.adjoint_recorded() == 3
    assert [a.adjoint_substeps(k) for k in range(3)] == subs
    a.close()
    b.close()


def test_adjoint_leaves_the_forward_state():
    cfg, state, rec, rng = make_case(4, seed=2)
    sim = new_sim(cfg)
    w = loss_weights(sim, 4, rng)
    sim.push_fluid(*state)
    sim.push_particles(rec)
    sim.dt = DT
    t = [torch.tensor(x, requires_grad=True) for x in state + (rec,)]
    wall = torch.tensor([cfg.uy_wall[0], cfg.uy_wall[1]], dtype=torch.float64, requires_grad=True)
    out = Steps.apply(t[0], t[1], t[2], t[3], wall, sim, 5, 2, ADJOINT_COUPLED)
    before = [o.detach().numpy().copy() for o in out]
    step_before = sim.time_state()
    sum((o * torch.from_numpy(c)).sum() for o, c in zip(out, w)).backward()
    after = list(sim.pull_fluid()[:3]) + [sim.pull_particles()]
    for x, y in zip(before, after):
        assert np.array_equal(x, y)
    assert sim.time_state() == step_before
    # halo rows and wall columns of the gradient are zero (push recomputes them), and
    # particle gradients only on x, y, az, ux, uy, vz
    gu, gv, gp, gr = (x.grad.numpy() for x in t)
    for g in (gu, gv, gp):
        assert not g[0].any() and not g[-1].any()
    assert not gu[:, 0].any() and not gu[:, -1].any()
    assert not gv[:, 0].any() and not gv[:, -1].any()
    assert not gp[:, 0].any() and not gp[:, -1].any()
    other = [k for k in range(NFIELDS) if k not in DIFF_FIELDS]
    assert not gr[:, other].any() and gr[:, DIFF_FIELDS].any()
    sim.close()


def test_adjoint_reports_contact():
    case = cases.contact_cluster()
    sim = Simulation(case.config())
    sim.push_fluid(*case.fluid())
    sim.push_particles(case.particles)
    sim.dt = 1e-3
    sim.adjoint_begin(1)
    sim.adjoint_forward(record=True)
    sx, sy = sim.shapes()
    sim.adjoint_seed(np.ones(sx), np.ones(sy))
    with pytest.raises(EifError):
        sim.adjoint_backward()
    sim.close()


def test_adjoint_rejects_mixed_form_and_misuse():
    case = cases.poiseuille(itot=64, jtot=128, n=2, a=0.05, b=0.03)
    sim = Simulation(case.config(precision=PREC_MIXED))
    sim.push_fluid(*case.fluid())
    with pytest.raises(EifError):
        sim.adjoint_begin(2)
    sim.close()
    sim = Simulation(case.config())
    sim.push_fluid(*case.fluid())
    sim.push_particles(case.particles)
    with pytest.raises(EifError):
        sim.adjoint_begin(2, 7)   # no such mode
    sim.adjoint_begin(1)
    with pytest.raises(EifError):
        sim.adjoint_backward()
    sim.dt = 1e-3
    sim.adjoint_forward()
    with pytest.raises(EifError):
        sim.adjoint_forward()   # tape of one step is full
    assert sim.adjoint_recorded() == 1
    with pytest.raises(ValueError):
        sim.adjoint_seed_particles(np.zeros((3, NFIELDS)))   # wrong particle count
    sim.adjoint_end()
    sim.close()


def test_adjoint_couette_256x512_400_steps():
    """256x512 Couette flow (walls -0.5, 0.5), Re = 100, 8 ellipses a = 0.06, b = 0.03,
    centres at least 4a apart; 400 steps with checkpoints every 50."""
    case = cases.adjoint_couette()
    cfg = case.config()
    sim = Simulation(cfg)
    state = tuple(np.array(a, dtype=np.float64) for a in case.fluid())
    rec = case.particles.copy()
    rng = np.random.default_rng(4)
    n = rec.shape[0]
    w = loss_weights(sim, n, rng)
    sim.push_fluid(*state)
    sim.push_particles(rec)
    dt = 0.5 * sim.decide_dt()
    nsteps = 400
    _, subs = run(sim, state, rec, nsteps, dt, ADJOINT_COUPLED)
    sim.push_fluid(*state)
    sim.push_particles(rec)
    sim.dt = dt
    grads, _ = gradients(sim, state, rec, w, nsteps, 50, ADJOINT_COUPLED)
    sx, sy = sim.shapes()
    dpos = np.zeros((n, NFIELDS))
    dpos[:, [F["x"], F["y"], F["az"]]] = rng.standard_normal((n, 3))
    for name, d in {"fluid": (rng.standard_normal(sx), rng.standard_normal(sy), np.zeros(sy), np.zeros((n, NFIELDS))),
                    "positions": (np.zeros(sx), np.zeros(sy), np.zeros(sy), dpos)}.items():
        fd = fd_along(cfg, state, rec, w, nsteps, dt, ADJOINT_COUPLED, d=d, ref_subs=subs)
        adj = sum(float(np.sum(g * e)) for g, e in zip(grads[:4], d))
        print("Couette adjoint vs central difference [%s]: %.15e %.15e rel %.2e" % (name, adj, fd, abs(adj - fd) / abs(fd)))
        assert abs(adj - fd) <= TOL_FD * abs(fd), (name, adj, fd)
    dwall = np.array([1.0, -1.0])
    fd = fd_along(cfg, state, rec, w, nsteps, dt, ADJOINT_COUPLED, dwall=dwall, ref_subs=subs)
    adj = float(np.dot(grads[4], dwall))
    print("Couette adjoint vs central difference [wall]: %.15e %.15e rel %.2e" % (adj, fd, abs(adj - fd) / abs(fd)))
    assert abs(adj - fd) <= TOL_FD * abs(fd)
    sim.close()


def test_adjoint_matches_reference_central_differences():
    """Directional derivatives of the GPU adjoint against central differences of the
    reference solver's own CPU step (fixture written by tests/golden/make_adjoint_fd.py)."""
    import importlib.util
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location("make_adjoint_fd", os.path.join(here, "golden", "make_adjoint_fd.py"))
    G = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(G)
    ref = np.load(os.path.join(here, "golden", "adjoint_fd_64x128.npz"))
    case, state, rec, w, dirs = G.inputs()
    sim = Simulation(case.config())
    out, subs = run(sim, state, rec, G.NSTEPS, G.DT, ADJOINT_COUPLED)
    # the same sub-iteration counts as the reference run, and the same loss (1e-11 parity)
    assert np.array_equal(np.array(subs), ref["substeps"])
    assert loss(out, w) == pytest.approx(float(ref["loss"]), rel=1e-11)
    grads, _ = gradients(sim, state, rec, w, G.NSTEPS, 3, ADJOINT_COUPLED)
    for name, d in dirs.items():
        fd = float(ref["fd_" + name])
        adj = sum(float(np.sum(g * e)) for g, e in zip(grads[:4], d))
        print("adjoint vs reference central difference [%s]: %.15e %.15e rel %.2e" % (name, adj, fd, abs(adj - fd) / abs(fd)))
        assert abs(adj - fd) <= TOL_FD * abs(fd), (name, adj, fd)
    sim.close()


def c4_objective_run(cfg, state, rec, nsteps, dt, wall=None):
    """objective (mean x-centre + kinetic energy) after nsteps forward steps, and the
    sub-iteration counts"""
    from ellipsesinflows_gb300.adjoint import mean_x_plus_energy
    sim = new_sim(cfg, wall)
    out, subs = run(sim, state, rec, nsteps, dt, ADJOINT_COUPLED)
    sim.close()
    val = mean_x_plus_energy(torch.from_numpy(out[0]), torch.from_numpy(out[1]), torch.from_numpy(out[3]),
                             cfg.ly)
    return float(val), subs


def test_adjoint_c4_objective_matches_central_differences():
    """256x512 Couette flow (walls at -0.5 and 0.5, Re 100), 8 ellipses a = 0.06, b = 0.03
    at least 4a apart, 400 steps with a checkpoint every 50: the gradient of the mean
    ellipse x-centre plus the fluid's kinetic energy (src/logging.c:130-172) with
    respect to the initial angles, the initial centres and the wall speed s (walls at
    -s and s), against central differences of the GPU step (step 1e-7 for angles and
    centres, 1e-5 for the wall speed) and of the reference's own CPU step (fixture
    written by tests/golden/make_adjoint_c4_fd.py: the same 400 steps)."""
    import importlib.util
    import os
    from ellipsesinflows_gb300.adjoint import mean_x_plus_energy
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location("make_c4", os.path.join(here, "golden", "make_adjoint_c4_fd.py"))
    G = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(G)
    ref = np.load(os.path.join(here, "golden", "adjoint_fd_c4_256x512.npz"))
    case, state, rec, dirs = G.inputs()
    cfg = case.config()
    nsteps, dt = int(ref["nsteps"]), float(ref["dt"])
    sim = Simulation(cfg)
    sim.push_fluid(*state)
    sim.push_particles(rec)
    assert 0.5 * sim.decide_dt() == dt       # the reference's dt, bit for bit
    base, subs = c4_objective_run(cfg, state, rec, nsteps, dt)
    assert np.array_equal(np.array(subs), ref["substeps"])
    assert base == pytest.approx(float(ref["loss"]), rel=1e-10)
    # gradients through the adjoint (checkpoints every 50 steps)
    sim.push_fluid(*state)
    sim.push_particles(rec)
    sim.dt = dt
    t = [torch.tensor(a, requires_grad=True) for a in state + (rec,)]
    wall = torch.tensor([cfg.uy_wall[0], cfg.uy_wall[1]], dtype=torch.float64, requires_grad=True)
    ux, uy, p, r = Steps.apply(t[0], t[1], t[2], t[3], wall, sim, nsteps, 50, ADJOINT_COUPLED)
    J = mean_x_plus_energy(ux, uy, r, cfg.ly)
    assert float(J) == pytest.approx(base, rel=1e-13)
    J.backward()
    grec, gwall = t[3].grad.numpy(), wall.grad.numpy()
    sim.close()
    for name in ("angles", "centres"):
        d = dirs[name]
        adj = float(np.sum(grec * d))
        # against the reference's central difference
        fd_ref = float(ref["fd_" + name])
        assert np.array_equal(ref["substeps_" + name][0], ref["substeps"])
        assert np.array_equal(ref["substeps_" + name][1], ref["substeps"])
        print("C4 objective, adjoint vs reference central difference [%s]: %.15e %.15e rel %.2e"
              % (name, adj, fd_ref, abs(adj - fd_ref) / abs(fd_ref)))
        assert abs(adj - fd_ref) <= TOL_FD * abs(fd_ref), (name, adj, fd_ref)
        # against the GPU step's own central difference
        eps = float(ref["eps"])
        vp, sp = c4_objective_run(cfg, state, rec + eps * d, nsteps, dt)
        vm, sm = c4_objective_run(cfg, state, rec - eps * d, nsteps, dt)
        assert sp == subs and sm == subs
        fd = (vp - vm) / (2 * eps)
        print("C4 objective, adjoint vs GPU central difference [%s]: %.15e %.15e rel %.2e"
              % (name, adj, fd, abs(adj - fd) / abs(fd)))
        assert abs(adj - fd) <= TOL_FD * abs(fd), (name, adj, fd)
    # wall speed s: walls at (-s, s), d/ds = -dJ/d uy_wall[0] + dJ/d uy_wall[1]
    adj = float(-gwall[0] + gwall[1])
    s0, eps = cfg.uy_wall[1], 1e-5
    vp, sp = c4_objective_run(cfg, state, rec, nsteps, dt, wall=(-(s0 + eps), s0 + eps))
    vm, sm = c4_objective_run(cfg, state, rec, nsteps, dt, wall=(-(s0 - eps), s0 - eps))
    assert sp == subs and sm == subs
    fd = (vp - vm) / (2 * eps)
    print("C4 objective, adjoint vs GPU central difference [wall speed]: %.15e %.15e rel %.2e"
          % (adj, fd, abs(adj - fd) / abs(fd)))
    assert abs(adj - fd) <= TOL_FD * abs(fd)
