"""The logging reductions (src/logging.c:40-172) and log files (:197-208).

CPU only: the restatement in oracle/logging.py against the reference's own
logging() (its files, written by the reference build into a temporary
directory), and the package's LogWriter writing byte-identical files from the
same quantities."""
import os

import numpy as np
import pytest

from ellipsesinflows_gb300 import cases
from ellipsesinflows_gb300.logs import LogWriter
from oracle import build, ref
from oracle import logging as olog

HAVE_REF = build.build_ref() if os.path.isdir(os.path.join(build.REFERENCE_DIR, "src")) else False
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference sources not present")


def _ref_state(steps=3):
    case = cases.poiseuille(itot=64, jtot=128, n=6, a=0.08, b=0.05, seed=5)
    s = ref.RefSolver(case.itot, case.jtot, case.ly, case.Re, case.Fr, case.extfrcy, case.safefactors)
    ux, uy, p = case.fluid()
    rng = np.random.default_rng(2)
    s.set_fluid(ux + 0.01 * rng.standard_normal(ux.shape), uy + 0.1 + 0.01 * rng.standard_normal(uy.shape), p)
    s.set_particles(case.particles)
    for _ in range(steps):
        s.step()
    return case, s


class _OracleSim:
    """the quantities LogWriter reads, from the restatement and the reference state"""

    def __init__(self, case, s, step, time):
        self.case, self.s, self.step, self.time = case, s, step, time
        self.dt = s.dt

    def time_state(self):
        return self.step, self.time

    def log_quantities(self):
        ux, uy, _, _ = self.s.get_fluid()
        dm, ds, mom, en = olog.log_quantities(ux, uy, self.case.itot, self.case.jtot, self.case.ly)
        return {"divmax": dm, "divsum": ds, "momentum": mom, "energy": en}

    def pull_particles(self):
        return self.s.get_particles()


@needs_ref
@pytest.mark.parametrize("step", [0, 7])
def test_log_files_match_reference(tmp_path, monkeypatch, step):
    case, s = _ref_state()
    time, rate = 0.0123456, 0.01
    refdir = tmp_path / "ref"
    (refdir / "output" / "log").mkdir(parents=True)
    monkeypatch.chdir(refdir)
    s.logging(step, time, rate)
    ours = tmp_path / "ours"
    LogWriter(_OracleSim(case, s, step, time), rate, dirname=str(ours), echo=False).write()
    names = sorted(os.listdir(refdir / "output" / "log"))
    assert names == sorted(os.listdir(ours))
    assert "energy.dat" in names and "particle0000000005.dat" in names
    for name in names:
        a = (refdir / "output" / "log" / name).read_text()
        b = (ours / name).read_text()
        assert a == b, (name, a, b)
    s.close()
