"""Checkpoint and restart (src/save.c, the reference's restart path): a run saved
after N/2 steps and continued from the files in a new context gives the bits of an
uninterrupted N-step run; an asynchronous snapshot holds the state of the step it
was taken at although steps ran while it was copied."""
import os

import numpy as np
import pytest

from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, cases, restart

pytestmark = pytest.mark.gpu


def _state(sim):
    return [a.copy() for a in sim.pull_fluid()[:3]] + [sim.pull_particles()]


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_restart_is_bit_exact(tmp_path, prec):
    case = cases.poiseuille(itot=128, jtot=256, n=12, a=0.05, b=0.025, seed=4)
    a = Simulation.from_case(case, precision=prec)
    a.advance(10)
    ref = _state(a)
    b = Simulation.from_case(case, precision=prec)
    b.advance(5)
    d = restart.save(b, str(tmp_path))
    assert os.path.basename(d) == "step%010d" % 5
    c = Simulation(case.config(precision=prec))
    assert restart.load(c, d) == b.time_state()
    c.advance(5)
    out = _state(c)
    for x, y in zip(ref[:3], out[:3]):
        assert np.array_equal(x, y)
    from ellipsesinflows_gb300.capi import F
    keep = [F[k] for k in ("x", "y", "az", "ux", "uy", "vz")]
    assert np.array_equal(ref[3][:, keep], out[3][:, keep])
    assert c.time_state() == a.time_state()
    for s in (a, b, c):
        s.close()


def test_async_snapshot_holds_the_taken_step(tmp_path):
    case = cases.poiseuille(itot=256, jtot=512, n=24, a=0.04, b=0.02, seed=3)
    a = Simulation.from_case(case)
    a.advance(3)
    pending = restart.AsyncSave(a, str(tmp_path / "async"))
    a.advance(4)                       # runs while the snapshot is copied
    d_async = pending.finish()
    b = Simulation.from_case(case)
    b.advance(3)
    d_sync = restart.save(b, str(tmp_path / "sync"))
    names = sorted(os.listdir(d_sync))
    assert names == sorted(os.listdir(d_async))
    for n in names:
        assert open(os.path.join(d_sync, n), "rb").read() == open(os.path.join(d_async, n), "rb").read(), n
    a.close()
    b.close()
