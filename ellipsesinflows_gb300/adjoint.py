"""Gradients of the step through the discrete adjoint (eif_adjoint_* in include/eif.h).

The adjoint is the transposed linearisation of the double-precision step with
dt held at the value set on the solver. In the coupled mode the particles move
(inertia, exchange forces, Newton-Euler increments and the recorded
sub-iterations of the particle fixed point are differentiated; collision forces
are constants, so the steps must be contact-free); in the frozen mode the
particle records are parameters of the step. ``Steps`` wraps it in a
``torch.autograd.Function`` so that a gradient harness can differentiate a loss
of the state after ``nsteps`` steps:

    ux, uy, p, rec = Steps.apply(ux0, uy0, p0, rec0, wall, sim, nsteps, every, mode)
    loss(ux, uy, p, rec).backward()   # ux0.grad, uy0.grad, p0.grad, rec0.grad, wall.grad

Tensors are float64 on the CPU: the fields in the eif_push_fluid layouts, the
particle records as (n, NFIELDS), ``wall`` the two wall velocities of the
solver's configuration (its gradient is d/d uy_wall). Particle gradients are
those of x, y, az, ux, uy, vz (the other record fields are outputs of a step);
a loss may depend on those six fields of the output records only.

Memory: the forward keeps the state every ``every`` steps (checkpoints, on the
host); backward re-runs each segment from its checkpoint with the step recorded
on the device (at most ``every`` steps) and goes back through it, so the device
holds one segment at a time.

This module is a harness for checking and using gradients; the time-step path
itself is the CUDA library.
"""
import numpy as np
import torch

from .capi import ADJOINT_COUPLED, ADJOINT_FROZEN, F, NFIELDS  # noqa: F401

DIFF_FIELDS = [F[k] for k in ("x", "y", "az", "ux", "uy", "vz")]


class Steps(torch.autograd.Function):
    """(ux0, uy0, p0, rec0, wall) -> state after ``nsteps`` steps of ``sim``."""

    @staticmethod
    def forward(ctx, ux0, uy0, p0, rec0, wall, sim, nsteps, every, mode):
        nsteps, every = int(nsteps), int(every)
        if nsteps < 1 or every < 1:
            raise ValueError("nsteps and every must be positive")
        cfg_wall = (sim.cfg.uy_wall[0], sim.cfg.uy_wall[1])
        if tuple(float(v) for v in wall.detach().numpy()) != cfg_wall:
            raise ValueError("wall must hold the solver's wall velocities %s" % (cfg_wall,))
        sim.push_fluid(ux0.detach().numpy(), uy0.detach().numpy(), p0.detach().numpy())
        sim.push_particles(rec0.detach().numpy())
        sim.adjoint_begin(min(every, nsteps), mode)
        checkpoints = []
        for s in range(nsteps):
            if s % every == 0:
                checkpoints.append((tuple(a.copy() for a in sim.pull_fluid()[:3]), sim.pull_particles().copy()))
            sim.adjoint_forward(record=False)
        ux, uy, p, _ = sim.pull_fluid()
        rec = sim.pull_particles()
        ctx.sim, ctx.nsteps, ctx.every, ctx.mode, ctx.checkpoints = sim, nsteps, every, mode, checkpoints
        ctx.final = ((ux.copy(), uy.copy(), p.copy()), rec.copy())
        return torch.from_numpy(ux), torch.from_numpy(uy), torch.from_numpy(p), torch.from_numpy(rec)

    @staticmethod
    def backward(ctx, gux, guy, gp, grec):
        sim, nsteps, every = ctx.sim, ctx.nsteps, ctx.every
        sx, sy = sim.shapes()

        def host(g, shape):
            return np.zeros(shape) if g is None else np.ascontiguousarray(g.detach().numpy(), dtype=np.float64)

        step0, time0 = sim.time_state()
        sim.adjoint_seed(host(gux, sx), host(guy, sy), host(gp, sy))
        if ctx.mode == ADJOINT_COUPLED:
            sim.adjoint_seed_particles(host(grec, (sim.n_particles, NFIELDS)))
        for seg in reversed(range(len(ctx.checkpoints))):
            n = min(every, nsteps - seg * every)
            fluid, rec = ctx.checkpoints[seg]
            sim.push_fluid(*fluid)
            sim.push_particles(rec)
            for _ in range(n):
                sim.adjoint_forward(record=True)
            for _ in range(n):
                sim.adjoint_backward()
        ub, vb, pb = sim.adjoint_pull()
        if ctx.mode == ADJOINT_COUPLED:
            rb = sim.adjoint_pull_particles()
        else:
            rb = np.zeros((sim.n_particles, NFIELDS))
        wb = sim.adjoint_wall_gradient()
        # the recomputation leaves the solver at the first segment's end: put back the
        # state and counters the forward left
        sim.push_fluid(*ctx.final[0])
        sim.push_particles(ctx.final[1])
        sim.set_time(step0, time0)
        return (torch.from_numpy(ub), torch.from_numpy(vb), torch.from_numpy(pb), torch.from_numpy(rb),
                torch.from_numpy(wb), None, None, None, None)


def grid_cells(itot, jtot, ly):
    """DXF(1..itot) and DXC(1..itot+1) of the uniform grid with walls at x = 0 and 1 (as
    set_coordinate forms them, src/param/init.c:105-167) and dy, as float64 tensors."""
    dx = 1.0 / itot
    xf = [1.0 * (i - 1) * dx for i in range(1, itot + 2)]
    xf[0], xf[itot] = 0.0, 1.0
    xc = [xf[0]] + [0.5 * (xf[i - 1] + xf[i]) for i in range(1, itot + 1)] + [xf[itot]]
    dxf = torch.tensor([xf[i] - xf[i - 1] for i in range(1, itot + 1)], dtype=torch.float64)
    dxc = torch.tensor([xc[i] - xc[i - 1] for i in range(1, itot + 2)], dtype=torch.float64)
    return dxf, dxc, ly / jtot


def kinetic_energy(ux, uy, ly):
    """Kinetic energy of the fluid as the reference logs it (check_energy,
    src/logging.c:130-172): the sum over the rows j = 1..jtot of UX(i,j)^2/2 DXC(i) dy
    (faces i = 1..itot+1) plus UY(i,j)^2/2 DXF(i) dy (cells i = 1..itot), for fields in
    the eif_push_fluid layouts (torch tensors, differentiable)."""
    jtot, itot = uy.shape[0] - 2, uy.shape[1] - 2
    dxf, dxc, dy = grid_cells(itot, jtot, ly)
    ex = 0.5 * (ux[1:-1, :] ** 2 * dxc[None, :]).sum() * dy
    ey = 0.5 * (uy[1:-1, 1:-1] ** 2 * dxf[None, :]).sum() * dy
    return ex + ey


def mean_x_plus_energy(ux, uy, rec, ly):
    """The mean ellipse x-centre plus the fluid's kinetic energy (kinetic_energy)."""
    return rec[:, F["x"]].mean() + kinetic_energy(ux, uy, ly)


def steps(sim, ux0, uy0, p0, rec0, nsteps, every=16, mode=ADJOINT_COUPLED, wall=None):
    """Functional form of ``Steps.apply``; ``wall`` defaults to the solver's wall velocities."""
    if wall is None:
        wall = torch.tensor([sim.cfg.uy_wall[0], sim.cfg.uy_wall[1]], dtype=torch.float64)
    return Steps.apply(ux0, uy0, p0, rec0, wall, sim, nsteps, every, mode)
