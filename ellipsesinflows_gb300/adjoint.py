"""Gradients of the step through the discrete adjoint (eif_adjoint_* in include/eif.h).

The adjoint is the transposed linearisation of the double-precision step with
the particles frozen (their records are parameters: the immersed-boundary
forcing acts with their rigid-body velocities, nothing moves them) and dt held
at the value set on the solver. ``FrozenSteps`` wraps it in a
``torch.autograd.Function`` so that a gradient harness can differentiate a loss
of the state after ``nsteps`` steps with respect to the initial velocity and
pressure fields:

    ux, uy, p = FrozenSteps.apply(ux0, uy0, p0, sim, nsteps, every)
    loss(ux, uy, p).backward()        # ux0.grad, uy0.grad, p0.grad

Tensors are float64 on the CPU in the eif_push_fluid layouts. Memory: the
forward keeps the state every ``every`` steps (checkpoints, on the host);
backward re-runs each segment from its checkpoint with the stage inputs
recorded on the device (3 velocity pairs per step, at most ``every`` steps) and
goes back through it, so the device holds one segment at a time.

This module is a harness for checking and using gradients; the time-step path
itself is the CUDA library.
"""
import numpy as np
import torch


class FrozenSteps(torch.autograd.Function):
    """(ux0, uy0, p0) -> state after ``nsteps`` frozen-particle steps of ``sim``."""

    @staticmethod
    def forward(ctx, ux0, uy0, p0, sim, nsteps, every):
        nsteps, every = int(nsteps), int(every)
        if nsteps < 1 or every < 1:
            raise ValueError("nsteps and every must be positive")
        sim.push_fluid(ux0.detach().numpy(), uy0.detach().numpy(), p0.detach().numpy())
        sim.adjoint_begin(min(every, nsteps))
        checkpoints = []
        for s in range(nsteps):
            if s % every == 0:
                checkpoints.append(tuple(a.copy() for a in sim.pull_fluid()[:3]))
            sim.adjoint_forward(record=False)
        ux, uy, p, _ = sim.pull_fluid()
        ctx.sim, ctx.nsteps, ctx.every, ctx.checkpoints = sim, nsteps, every, checkpoints
        ctx.final = (ux.copy(), uy.copy(), p.copy())
        return torch.from_numpy(ux), torch.from_numpy(uy), torch.from_numpy(p)

    @staticmethod
    def backward(ctx, gux, guy, gp):
        sim, nsteps, every = ctx.sim, ctx.nsteps, ctx.every
        sx, sy = sim.shapes()

        def host(g, shape):
            return np.zeros(shape) if g is None else np.ascontiguousarray(g.detach().numpy(), dtype=np.float64)

        step0, time0 = sim.time_state()
        sim.adjoint_seed(host(gux, sx), host(guy, sy), host(gp, sy))
        for seg in reversed(range(len(ctx.checkpoints))):
            n = min(every, nsteps - seg * every)
            sim.push_fluid(*ctx.checkpoints[seg])
            for _ in range(n):
                sim.adjoint_forward(record=True)
            for _ in range(n):
                sim.adjoint_backward()
        ub, vb, pb = sim.adjoint_pull()
        # the recomputation leaves the solver at the first segment's end: put back the
        # state and counters the forward left
        sim.push_fluid(*ctx.final)
        sim.set_time(step0, time0)
        return torch.from_numpy(ub), torch.from_numpy(vb), torch.from_numpy(pb), None, None, None


def frozen_steps(sim, ux0, uy0, p0, nsteps, every=16):
    """Functional form of ``FrozenSteps.apply``."""
    return FrozenSteps.apply(ux0, uy0, p0, sim, nsteps, every)
