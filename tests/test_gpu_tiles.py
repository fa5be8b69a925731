"""Tile shapes of the stencil and block-Thomas kernels (csrc/tune.cu): the tuner's
choice is reported after the first step, and every shape gives the same bits."""
import numpy as np
import pytest

from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, cases

pytestmark = pytest.mark.gpu


def _run(monkeypatch, case, prec, tiles, steps=4):
    if tiles is None:
        monkeypatch.delenv("EIF_TILES", raising=False)
    else:
        monkeypatch.setenv("EIF_TILES", tiles)
    sim = Simulation.from_case(case, precision=prec)
    sim.advance(steps)
    out = [a.copy() for a in sim.pull_fluid()[:3]] + [sim.pull_particles()]
    t = sim.tiles()
    sim.close()
    return out, t


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_tile_shapes_do_not_change_results(monkeypatch, prec):
    case = cases.poiseuille(itot=256, jtot=512, n=24, a=0.04, b=0.02, seed=3)
    ref, t = _run(monkeypatch, case, prec, None)
    assert t["tuned"] and t["predictor_rows"] in (4, 8, 16) and t["thomas_threads"] in (64, 128, 256)
    for tiles in ("4,16,64", "16,4,256", "8,8,128"):
        out, t = _run(monkeypatch, case, prec, tiles)
        assert (t["predictor_rows"], t["projection_rows"], t["thomas_threads"]) == tuple(int(v) for v in tiles.split(","))
        for a, b in zip(ref, out):
            assert np.array_equal(a, b)


def test_bad_tile_setting_is_an_error(monkeypatch):
    from ellipsesinflows_gb300 import EifError
    case = cases.couette_circle()
    monkeypatch.setenv("EIF_TILES", "5,8,128")
    sim = Simulation.from_case(case)
    with pytest.raises(EifError):
        sim.advance(1)
    sim.close()
