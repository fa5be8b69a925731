"""eif_advance_pull: the steps of eif_advance, then the fields (copied beside the last
stage's particle work) and the records into host arrays; the arrays equal bit for bit
those of eif_advance followed by eif_pull_fluid and eif_pull_particles, into page-locked
and into ordinary host memory, in both forms."""
import numpy as np
import pytest

from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, cases

pytestmark = pytest.mark.gpu


def pinned_like(a):
    torch = pytest.importorskip("torch")
    return torch.zeros(a.shape, dtype=torch.float64).pin_memory().numpy()


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
def test_advance_pull_equals_advance_then_pull(prec, pinned, gpu_lib):
    case = cases.poiseuille(itot=128, jtot=256, n=8, a=0.05, b=0.025, seed=11)
    ref = Simulation.from_case(case, precision=prec)
    sim = Simulation.from_case(case, precision=prec)
    ref.advance(3)
    ux, uy, p, _ = ref.pull_fluid()
    rec = ref.pull_particles()
    outs = [np.zeros_like(ux), np.zeros_like(uy), np.zeros_like(p), np.zeros_like(rec)]
    if pinned:
        outs = [pinned_like(a) for a in outs]
    sim.advance_pull(3, tuple(outs[:3]), outs[3])
    for got, want in zip(outs, (ux, uy, p, rec)):
        assert np.array_equal(got, want)
    assert sim.time_state() == ref.time_state()
    # with a field left out, and the context going on as with eif_advance
    ref.advance(1)
    keep = np.full_like(uy, 7.0)
    sim.advance_pull(1, (outs[0], None, keep), None)
    assert np.array_equal(outs[0], ref.pull_fluid()[0])
    assert np.array_equal(keep, ref.pull_fluid()[2])
