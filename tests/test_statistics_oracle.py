"""Statistics (src/statistics/): the restatement in oracle/statistics.py against the
reference's own statistics_collect/statistics_output, and the package's writer
producing the reference's files byte for byte. CPU only."""
import os

import pytest

from ellipsesinflows_gb300 import cases
from ellipsesinflows_gb300.stats import write_stats
from oracle import build, ref
from oracle import statistics as ostat

HAVE_REF = build.build_ref() if os.path.isdir(os.path.join(build.REFERENCE_DIR, "src")) else False
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference sources not present")


@needs_ref
def test_statistics_files_match_reference(tmp_path, monkeypatch):
    case = cases.poiseuille(itot=48, jtot=96, n=5, a=0.09, b=0.05, seed=8)
    s = ref.RefSolver(case.itot, case.jtot, case.ly, case.Re, case.Fr, case.extfrcy, case.safefactors)
    s.set_fluid(*case.fluid())
    s.set_particles(case.particles)
    acc = ostat.Accumulator(case.itot, case.jtot, case.ly)
    for _ in range(3):
        s.step()
        s.stats_collect()
        ux, uy, _, _ = s.get_fluid()
        acc.collect(ux, uy, s.get_particles())
    assert acc.phi.sum() > 0
    step, time = 3, s.time
    (tmp_path / "ref" / "output" / "stat").mkdir(parents=True)
    monkeypatch.chdir(tmp_path / "ref")
    assert s.stats_output(step, time) == 0
    d = write_stats(str(tmp_path / "ours"), case.config(), acc.ux1, acc.ux2, acc.uy1, acc.uy2, acc.phi, acc.num,
                    step, time)
    refdir = tmp_path / "ref" / "output" / "stat" / ("step%010d" % step)
    names = sorted(os.listdir(refdir))
    assert names == sorted(os.listdir(d))
    for name in names:
        assert (refdir / name).read_bytes() == open(os.path.join(d, name), "rb").read(), name
    s.close()
