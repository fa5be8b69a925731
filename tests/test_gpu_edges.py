"""Edge cases of the rows next to the step: no particles, precision changes across a
restart, a batch member without particles."""
import os

import numpy as np
import pytest

from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Batch, Simulation, cases, restart
from ellipsesinflows_gb300.logs import LogWriter
from ellipsesinflows_gb300.stats import Statistics
from oracle import logging as olog

pytestmark = pytest.mark.gpu


def _fluid_only(prec=PREC_FP64):
    case = cases.poiseuille(itot=64, jtot=128, n=1, a=0.05, b=0.03, seed=1)
    sim = Simulation(case.config(precision=prec))
    ux, uy, p = case.fluid()
    sim.push_fluid(ux, uy + 0.1, p)
    sim.push_particles(case.particles[:0])
    return case, sim


def test_no_particles_logging_stats_snapshot(tmp_path):
    case, sim = _fluid_only()
    sim.advance(3)
    q = sim.log_quantities()
    gu, gv, _, _ = sim.pull_fluid()
    dm, _, mom, en = olog.log_quantities(gu, gv, case.itot, case.jtot, case.ly)
    assert q["divmax"] == dm and q["energy"][1] == pytest.approx(en[1], rel=1e-13)
    LogWriter(sim, 0.1, dirname=str(tmp_path / "log"), echo=False).write()
    assert not [f for f in os.listdir(tmp_path / "log") if f.startswith("particle")]
    st = Statistics(sim)
    st.collect()
    *_, phi, num = sim.stats_pull()
    assert num == 1 and not phi.any()
    pending = restart.AsyncSave(sim, str(tmp_path / "save"))
    sim.advance(1)
    d = pending.finish()
    _, _, _, rec, step, _ = restart.read_state(d)
    assert rec.shape == (0, 30) and step == 3
    sim.close()


@pytest.mark.parametrize("saved,loaded", [(PREC_FP64, PREC_MIXED), (PREC_MIXED, PREC_FP64)])
def test_restart_across_precisions(tmp_path, saved, loaded):
    case = cases.poiseuille(itot=128, jtot=256, n=8, a=0.05, b=0.025, seed=7)
    a = Simulation.from_case(case, precision=saved)
    a.advance(4)
    d = restart.save(a, str(tmp_path))
    b = Simulation(case.config(precision=loaded))
    restart.load(b, d)
    assert b.time_state() == a.time_state()
    for x, y in zip(a.pull_fluid()[:3], b.pull_fluid()[:3]):
        assert np.array_equal(x[1:-1], y[1:-1])
    b.advance(2)   # continues in the other form
    assert np.isfinite(b.pull_fluid()[0]).all()
    a.close()
    b.close()


def test_batch_member_without_particles():
    _, empty = _fluid_only(PREC_MIXED)
    case = cases.poiseuille(itot=128, jtot=256, n=6, a=0.05, b=0.025, seed=2)
    full = Simulation.from_case(case, precision=PREC_MIXED)
    ref_e, ref_f = _fluid_only(PREC_MIXED)[1], Simulation.from_case(case, precision=PREC_MIXED)
    b = Batch([empty, full])
    b.advance(3)
    ref_e.advance(3)
    ref_f.advance(3)
    for s, r in ((empty, ref_e), (full, ref_f)):
        for x, y in zip(s.pull_fluid()[:3], r.pull_fluid()[:3]):
            assert np.array_equal(x, y)
    b.close()
    for s in (empty, full, ref_e, ref_f):
        s.close()
