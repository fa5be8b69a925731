"""Device reductions of the logging diagnostics (eif_log_quantities) against the
restatement of src/logging.c:40-172 on the pulled fields; the log files written
from them."""
import numpy as np
import pytest

from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, cases
from ellipsesinflows_gb300.logs import LogWriter
from oracle import logging as olog

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_log_quantities_match_restatement(prec):
    case = cases.poiseuille(itot=128, jtot=256, n=12, a=0.05, b=0.025, seed=4)
    sim = Simulation.from_case(case, precision=prec)
    ux, uy, p = case.fluid()
    rng = np.random.default_rng(1)
    sim.push_fluid(ux + 0.01 * rng.standard_normal(ux.shape), uy + 0.2 + 0.01 * rng.standard_normal(uy.shape), p)
    for check_after in (0, 5):
        sim.advance(check_after)
        q = sim.log_quantities()
        gu, gv, _, _ = sim.pull_fluid()
        dm, ds, mom, en = olog.log_quantities(gu, gv, case.itot, case.jtot, case.ly)
        # per-cell divergence with the same operations: the maximum is the same number
        assert q["divmax"] == dm
        assert abs(q["divsum"] - ds) <= 1e-11 * case.cells * max(dm, 1e-300)
        # momentum sums cancel (a channel at rest in x): compared on the sum of |terms|
        cell = case.ly / case.jtot / case.itot
        scales = (np.abs(gu[1:-1]).sum() * cell, np.abs(gv[1:-1, 1:-1]).sum() * cell) + tuple(abs(e) for e in en)
        for a, b, sc in zip(q["momentum"] + q["energy"], mom + en, scales):
            assert abs(a - b) <= 1e-13 * max(sc, 1e-300), (a, b)
        assert sim.divergence() == (q["divmax"], q["divsum"])
        assert sim.momentum() == q["momentum"] and sim.energy() == q["energy"]
    sim.close()


def test_log_writer_on_device(tmp_path):
    case = cases.poiseuille(itot=64, jtot=128, n=4, a=0.06, b=0.03, seed=6)
    sim = Simulation.from_case(case)
    w = LogWriter(sim, 0.1, dirname=str(tmp_path), echo=False)
    w.write()
    sim.advance(3)
    w.write()
    lines = (tmp_path / "energy.dat").read_text().splitlines()
    assert len(lines) == 2
    gu, gv, _, _ = sim.pull_fluid()
    _, _, _, en = olog.log_quantities(gu, gv, case.itot, case.jtot, case.ly)
    vals = [float(v) for v in lines[1].split()[1:]]
    assert vals == pytest.approx(list(en), rel=1e-14, abs=1e-300)
    assert len((tmp_path / "particle0000000003.dat").read_text().splitlines()) == 2
    sim.close()
