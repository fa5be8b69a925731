"""Batches of independent suspensions (eif_batch_*): one CUDA graph launch per step
advances every suspension, and each gets the same bits as when advanced alone, with
the same sub-iteration counts. The sub-iteration loops of the batch run in one
persistent kernel per RK stage (the default) or as a conditional loop per suspension
(EIF_BATCH_SUBITER=branches); both are checked."""
import numpy as np
import pytest

from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Batch, Simulation, cases

pytestmark = pytest.mark.gpu


def members():
    return [
        (lambda: cases.contact_cluster(), PREC_FP64),
        (lambda: cases.couette_circle(), PREC_MIXED),
        (lambda: cases.poiseuille(itot=128, jtot=256, n=8, a=0.05, b=0.025, seed=11), PREC_MIXED),
        (lambda: cases.poiseuille(itot=96, jtot=192, n=4, a=0.06, b=0.03, seed=12), PREC_FP64),
    ]


def assert_same(a, b):
    for x, y in zip(a.pull_fluid(), b.pull_fluid()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.pull_particles(), b.pull_particles())
    assert a.time_state() == b.time_state()
    assert a.counters()["substeps"] == b.counters()["substeps"]


@pytest.fixture(params=["stage_kernels", "branches"])
def subiter_mode(request, monkeypatch):
    if request.param == "branches":
        monkeypatch.setenv("EIF_BATCH_SUBITER", "branches")
    else:
        monkeypatch.delenv("EIF_BATCH_SUBITER", raising=False)
    return request.param


def test_batch_equals_separate_advance(gpu_lib, subiter_mode):
    specs = members()
    solo = [Simulation.from_case(f(), precision=p) for f, p in specs]
    together = [Simulation.from_case(f(), precision=p) for f, p in specs]
    for s in solo:
        s.advance(3)
    with Batch(together) as batch:
        batch.advance(2)
        batch.advance(1)
    for a, b in zip(solo, together):
        assert_same(a, b)


def test_batch_c5_members_equal_separate_advance(gpu_lib, subiter_mode):
    """Ten suspensions of the uneven batch workload (4 to 256 ellipses, all four grid
    sizes) plus one without particles, five steps."""
    specs = cases.batch_c5(count=10, seed=3)
    empty = cases.poiseuille(itot=128, jtot=256, n=1, seed=2)
    empty.particles = empty.particles[:0]
    solo = [Simulation.from_case(c, precision=PREC_MIXED) for c in specs + [empty]]
    together = [Simulation.from_case(c, precision=PREC_MIXED) for c in specs + [empty]]
    for s in solo:
        s.advance(5)
    with Batch(together) as batch:
        batch.advance(5)
    for a, b in zip(solo, together):
        assert_same(a, b)
    print("sub-iterations per suspension over 5 steps:", [s.counters()["substeps"] for s in solo])


def test_batch_rebuilds_after_a_particle_count_change(gpu_lib):
    """A push with another particle count reallocates that suspension's buffers; the
    batch notices and captures a new step graph."""
    specs = members()[:3]
    solo = [Simulation.from_case(f(), precision=p) for f, p in specs]
    together = [Simulation.from_case(f(), precision=p) for f, p in specs]
    with Batch(together) as batch:
        for s in solo:
            s.advance(1)
        batch.advance(1)
        for s in (solo[2], together[2]):
            parts = s.pull_particles()
            s.push_particles(parts[:-2])
        for s in solo:
            s.advance(2)
        batch.advance(2)
    for a, b in zip(solo, together):
        assert_same(a, b)


def test_batch_with_a_suspension_beyond_the_stage_kernel(gpu_lib):
    """A suspension with more than 8192 ellipses keeps its own sub-iteration loops in its
    graph branch, beside the stage kernels of the other suspensions: every suspension
    still gets the bits of its separate run."""
    big = cases.poiseuille(itot=512, jtot=1024, n=8300, a=0.005, b=0.003, seed=21)
    specs = [(big, PREC_MIXED), (cases.couette_circle(), PREC_MIXED),
             (cases.poiseuille(itot=128, jtot=256, n=8, a=0.05, b=0.025, seed=11), PREC_FP64)]
    solo = [Simulation.from_case(c, precision=p) for c, p in specs]
    together = [Simulation.from_case(c, precision=p) for c, p in specs]
    for s in solo:
        s.advance(2)
    with Batch(together) as batch:
        batch.advance(2)
    for a, b in zip(solo, together):
        assert_same(a, b)


def test_stage_kernel_barrier_timeout_is_reported(gpu_lib, monkeypatch):
    """The stage kernel's grid barrier is a bounded wait. With CTA 0 of the first stage's
    kernel held back from its first barrier (EIF_TEST_HOLD_BARRIER=1, read when the batch's
    graph is built) the other CTAs give up after their 2^22 polls, return, and the step
    reports the bounded wait; the GPU context stays usable: a new batch of fresh
    suspensions then gives the bits of separate runs."""
    from ellipsesinflows_gb300.capi import EifError
    monkeypatch.delenv("EIF_BATCH_SUBITER", raising=False)
    specs = members()[:2]
    held = [Simulation.from_case(f(), precision=p) for f, p in specs]
    monkeypatch.setenv("EIF_TEST_HOLD_BARRIER", "1")
    with Batch(held) as batch:
        with pytest.raises(EifError, match="bounded wait"):
            batch.advance(1)
    monkeypatch.delenv("EIF_TEST_HOLD_BARRIER")
    solo = [Simulation.from_case(f(), precision=p) for f, p in specs]
    together = [Simulation.from_case(f(), precision=p) for f, p in specs]
    for s in solo:
        s.advance(2)
    with Batch(together) as batch:
        batch.advance(2)
    for a, b in zip(solo, together):
        assert_same(a, b)
