"""Discrete adjoint of the double-precision step (particles frozen, dt fixed).

The gradient of a linear functional of the state after N steps, taken through
the transposed steps (eif_adjoint_* behind FrozenSteps), is checked against
central differences of the same forward map along random directions of the
initial ux, uy and p. The bar is a relative difference of 1e-5; the central
difference itself is accurate to about 1e-9 at the step chosen (truncation
O(eps^2) of the quadratic advection, round-off 1e-16 |L| / eps).
"""
import numpy as np
import pytest
import torch

from ellipsesinflows_gb300 import Simulation, cases
from ellipsesinflows_gb300.adjoint import FrozenSteps

pytestmark = pytest.mark.gpu

TOL_FD = 1e-5
EPS = 1e-5


def setup(n_particles=8, itot=64, jtot=128, seed=11):
    case = cases.poiseuille(itot=itot, jtot=jtot, n=max(n_particles, 1), a=0.07, b=0.035, Re=150.0, seed=seed)
    sim = Simulation(case.config())
    ux, uy, p = (np.array(a, dtype=np.float64) for a in case.fluid())
    rng = np.random.default_rng(seed)
    # a sheared, rotating initial flow so that every advective partial derivative is active
    jj, ii = np.meshgrid(np.arange(jtot + 2), np.arange(itot + 1), indexing="ij")
    ux += 0.2 * np.sin(2 * np.pi * jj / jtot) * np.sin(np.pi * ii / itot) + 0.02 * rng.standard_normal(ux.shape)
    jj, ii = np.meshgrid(np.arange(jtot + 2), np.arange(itot + 2), indexing="ij")
    uy += 0.3 * np.cos(np.pi * (ii - 0.5) / itot) + 0.02 * rng.standard_normal(uy.shape)
    p += 0.05 * rng.standard_normal(p.shape)
    sim.push_fluid(ux, uy, p)
    sim.push_particles(case.particles[:n_particles])
    sim.dt = 0.5 * sim.decide_dt()
    return sim, (ux, uy, p), rng


def loss_weights(sim, rng):
    sx, sy = sim.shapes()
    cx, cy, cp = rng.standard_normal(sx), rng.standard_normal(sy), rng.standard_normal(sy)
    # pressure enters through its differences only: zero weight on the copies and mean-free
    cp[0, :] = cp[-1, :] = 0.
    cp[:, 0] = cp[:, -1] = 0.
    cp[1:-1, 1:-1] -= cp[1:-1, 1:-1].mean()
    return cx, cy, cp


def run(sim, state, nsteps):
    sim.push_fluid(*state)
    for _ in range(nsteps):
        sim.adjoint_forward(record=False)
    return sim.pull_fluid()[:3]


def loss(out, w):
    return sum(float(np.sum(o * c)) for o, c in zip(out, w))


def gradients(sim, state, w, nsteps, every):
    t = [torch.tensor(a, requires_grad=True) for a in state]
    out = FrozenSteps.apply(t[0], t[1], t[2], sim, nsteps, every)
    L = sum((o * torch.from_numpy(c)).sum() for o, c in zip(out, w))
    L.backward()
    return [a.grad.numpy().copy() for a in t], float(L.detach())


def directions(sim, rng):
    sx, sy = sim.shapes()
    d_all = (rng.standard_normal(sx), rng.standard_normal(sy), rng.standard_normal(sy))
    d_u = (rng.standard_normal(sx), np.zeros(sy), np.zeros(sy))
    d_v = (np.zeros(sx), rng.standard_normal(sy), np.zeros(sy))
    d_p = (np.zeros(sx), np.zeros(sy), rng.standard_normal(sy))
    return {"all": d_all, "ux": d_u, "uy": d_v, "p": d_p}


def check_fd(sim, state, w, grads, nsteps, rng):
    """Directional derivatives along random directions of all fields together and of
    each field alone. Without particles the state after a step does not depend on the
    initial pressure at all (the projection removes G p0 and the pressure update
    subtracts p0 again), so that derivative is compared on the scale of the
    all-field one: its central difference is round-off only."""
    ref = None
    for name, d in directions(sim, rng).items():
        plus = run(sim, tuple(s + EPS * e for s, e in zip(state, d)), nsteps)
        minus = run(sim, tuple(s - EPS * e for s, e in zip(state, d)), nsteps)
        fd = (loss(plus, w) - loss(minus, w)) / (2 * EPS)
        adj = sum(float(np.sum(g * e)) for g, e in zip(grads, d))
        ref = abs(fd) if ref is None else ref
        scale = max(abs(fd), ref) if name == "p" else abs(fd)
        print("adjoint vs central difference [%s]: %.15e %.15e rel %.2e" % (name, adj, fd, abs(adj - fd) / scale))
        assert abs(adj - fd) <= TOL_FD * scale, (name, adj, fd, abs(adj - fd) / scale)


@pytest.mark.parametrize("n_particles", [8, 0])
def test_adjoint_matches_central_differences(n_particles):
    sim, state, rng = setup(n_particles)
    w = loss_weights(sim, rng)
    nsteps = 10
    grads, L = gradients(sim, state, w, nsteps, every=4)
    # the forward value of the autograd function is the plain forward map
    assert L == pytest.approx(loss(run(sim, state, nsteps), w), rel=1e-14)
    check_fd(sim, state, w, grads, nsteps, rng)
    sim.close()


def test_adjoint_gradients_do_not_depend_on_checkpoint_spacing():
    sim, state, rng = setup(6, seed=5)
    w = loss_weights(sim, rng)
    g1, _ = gradients(sim, state, w, 6, every=1)
    g6, _ = gradients(sim, state, w, 6, every=6)
    g4, _ = gradients(sim, state, w, 6, every=4)
    for a, b, c in zip(g1, g6, g4):
        # each segment is recomputed from a bit-exact checkpoint: same tape, same bits
        assert np.array_equal(a, b) and np.array_equal(a, c)
    sim.close()


def test_adjoint_leaves_the_forward_state():
    sim, state, rng = setup(4, seed=2)
    w = loss_weights(sim, rng)
    t = [torch.tensor(a, requires_grad=True) for a in state]
    out = FrozenSteps.apply(t[0], t[1], t[2], sim, 5, 2)
    before = [o.detach().numpy().copy() for o in out]
    step_before = sim.time_state()
    sum((o * torch.from_numpy(c)).sum() for o, c in zip(out, w)).backward()
    after = sim.pull_fluid()[:3]
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    assert sim.time_state() == step_before
    # halo rows and wall columns of the gradient are zero (push recomputes them)
    gu, gv, gp = (a.grad.numpy() for a in t)
    for g in (gu, gv, gp):
        assert not g[0].any() and not g[-1].any()
    assert not gu[:, 0].any() and not gu[:, -1].any()
    assert not gv[:, 0].any() and not gv[:, -1].any()
    assert not gp[:, 0].any() and not gp[:, -1].any()
    sim.close()


def test_adjoint_rejects_mixed_form_and_empty_tape():
    from ellipsesinflows_gb300 import EifError, PREC_MIXED
    case = cases.poiseuille(itot=64, jtot=128, n=2, a=0.05, b=0.03)
    sim = Simulation(case.config(precision=PREC_MIXED))
    sim.push_fluid(*case.fluid())
    with pytest.raises(EifError):
        sim.adjoint_begin(2)
    sim.close()
    sim = Simulation(case.config())
    sim.push_fluid(*case.fluid())
    sim.push_particles(case.particles)
    sim.adjoint_begin(1)
    with pytest.raises(EifError):
        sim.adjoint_backward()
    sim.dt = 1e-3
    sim.adjoint_forward()
    with pytest.raises(EifError):
        sim.adjoint_forward()   # tape of one step is full
    assert sim.adjoint_recorded() == 1
    sim.adjoint_end()
    sim.close()
