"""Statistics accumulated on the device (eif_stats_*) against the restatement of
statistics_collect (src/statistics/collect.c:10-95) on the pulled states: the sums
and the particle indicator agree bit for bit, so the written files are identical."""
import os

import numpy as np
import pytest

from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, cases
from ellipsesinflows_gb300.stats import Statistics, write_stats
from oracle import statistics as ostat

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_device_statistics_match_restatement(tmp_path, prec):
    case = cases.poiseuille(itot=64, jtot=128, n=6, a=0.08, b=0.05, seed=5)
    sim = Simulation.from_case(case, precision=prec)
    st = Statistics(sim)
    acc = ostat.Accumulator(case.itot, case.jtot, case.ly)
    for _ in range(3):
        sim.advance(2)
        st.collect()
        ux, uy, _, _ = sim.pull_fluid()
        acc.collect(ux, uy, sim.pull_particles())
    ux1, ux2, uy1, uy2, phi, num = sim.stats_pull()
    assert num == 3 and phi.sum() > 0
    for name, a, b in (("ux1", ux1, acc.ux1), ("ux2", ux2, acc.ux2), ("uy1", uy1, acc.uy1), ("uy2", uy2, acc.uy2),
                       ("phi", phi, acc.phi)):
        assert np.array_equal(a, b), (name, np.abs(a - b).max())
    d = st.output(str(tmp_path / "dev"))
    step, time = sim.time_state()
    o = write_stats(str(tmp_path / "ora"), case.config(), acc.ux1, acc.ux2, acc.uy1, acc.uy2, acc.phi, acc.num,
                    step, time)
    for name in sorted(os.listdir(o)):
        assert open(os.path.join(d, name), "rb").read() == open(os.path.join(o, name), "rb").read(), name
    sim.close()


def test_statistics_at_full_size():
    # 2048 x 4096 with 2048 ellipses: phi counts the covered cells (about the area fraction)
    case = cases.mixed_target()
    sim = Simulation.from_case(case, precision=PREC_MIXED)
    st = Statistics(sim)
    st.collect()
    st.collect()
    ux1, ux2, uy1, uy2, phi, num = sim.stats_pull()
    assert num == 2
    frac = phi[1:-1, 1:-1].sum() / (2 * case.cells)
    area = float(np.sum(np.pi * case.particles[:, 1] * case.particles[:, 2])) / 2.0
    assert abs(frac - area) < 0.01 * area
    sim.close()
