"""Mixed-precision form (EIF_PREC_MIXED) against the double-precision form.

The double-precision form is pinned to the reference (test_gpu_parity.py).
The mixed form computes the indicator, the immersed-boundary forcing and the
predictor stencils in single precision while keeping storage, the projection
and the particle dynamics in double precision; its Poisson solve is two
single-precision passes (the second on the residual of the first, formed in
double-float arithmetic) with the reduced tridiagonal systems in double
precision. Its error bars are those of the target: velocity within 1e-4
relative to the double-precision run, maximum divergence below 1e-5.
"""
import numpy as np
import pytest

from conftest import rel_err
from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, cases
from ellipsesinflows_gb300.capi import F

pytestmark = pytest.mark.gpu

TOL_VEL = 1e-4
TOL_DIV = 1e-5


def pair(case):
    a = Simulation.from_case(case, precision=PREC_FP64)
    b = Simulation.from_case(case, precision=PREC_MIXED)
    return a, b


def vec_err(P, Q, fx, fy):
    scale = max(np.max(np.abs(Q[:, F[fx]])), np.max(np.abs(Q[:, F[fy]])))
    return max(np.max(np.abs(P[:, F[fx]] - Q[:, F[fx]])), np.max(np.abs(P[:, F[fy]] - Q[:, F[fy]]))) / scale


@pytest.mark.parametrize("builder", [
    lambda: cases.contact_cluster(),
    lambda: cases.poiseuille(itot=256, jtot=512, n=24, a=0.04, b=0.02, seed=4),
], ids=["contact_cluster", "poiseuille_256x512"])
def test_mixed_ibm_stage_matches_fp64(builder, gpu_lib):
    case = builder()
    d, m = pair(case)
    # drive a few steps in double precision so that the flow is not at rest
    d.advance(2)
    ux, uy, p, _ = d.pull_fluid()
    parts = d.pull_particles()
    m.push_fluid(ux, uy, p)
    m.push_particles(parts)
    for s in (d, m):
        s.dt = 2.0e-4
        s.reset_particle_increments()
        s.compute_inertia(0)
        s.exchange_momentum()
    P, Q = m.pull_particles(), d.pull_particles()
    assert vec_err(P, Q, "iux0", "iuy0") < 1e-5
    assert vec_err(P, Q, "fux", "fuy") < 1e-4
    for a, b in zip(m.pull_ibm_fields(), d.pull_ibm_fields()):
        assert rel_err(a, b) < 1e-4


@pytest.mark.parametrize("builder,steps", [
    (lambda: cases.poiseuille(itot=256, jtot=512, n=24, a=0.04, b=0.02, seed=4), 20),
    (lambda: cases.poiseuille(), 10),
], ids=["poiseuille_256x512", "poiseuille_512x1024"])
def test_mixed_steps_within_error_bars(builder, steps, gpu_lib):
    case = builder()
    d, m = pair(case)
    for _ in range(steps):
        d.advance(1)
        m.advance(1)
    du, dv, _, _ = d.pull_fluid()
    mu, mv, _, _ = m.pull_fluid()
    umag = max(np.abs(du).max(), np.abs(dv).max())
    err = max(np.abs(mu - du).max(), np.abs(mv - dv).max()) / umag
    assert err < TOL_VEL, err
    divmax, _ = m.divergence()
    assert divmax < TOL_DIV, divmax
    P, Q = m.pull_particles(), d.pull_particles()
    assert np.max(np.abs(P[:, F["x"]] - Q[:, F["x"]])) < 1e-6
    assert np.max(np.abs(P[:, F["y"]] - Q[:, F["y"]])) < 1e-6


def test_integer_pipe_conversions_match_hardware(gpu_lib):
    import ctypes
    fn = gpu_lib.eif_selftest_conversions
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
    a, b = ctypes.c_longlong(-1), ctypes.c_longlong(-1)
    assert fn(0, 1 << 24, ctypes.byref(a), ctypes.byref(b)) == 0
    assert a.value == 0 and b.value == 0, (a.value, b.value)


@pytest.mark.parametrize("builder", [
    lambda: cases.couette_circle(),
    lambda: cases.poiseuille(itot=256, jtot=512, n=24, a=0.04, b=0.02, seed=4),
], ids=["couette_circle", "poiseuille_256x512"])
def test_mixed_predictor_matches_fp64(builder, gpu_lib):
    case = builder()
    d, m = pair(case)
    d.advance(3)
    ux, uy, p, _ = d.pull_fluid()
    m.push_fluid(ux, uy, p)
    for s in (d, m):
        s.dt = 1.0e-3
        s.update_velocity(0)
    ga, _, gya, _ = m.pull_src()
    da, _, dya, _ = d.pull_src()
    assert rel_err(ga, da) < 1e-5
    assert rel_err(gya, dya) < 1e-5
    # the stage's velocity increment carries the single-precision error of its terms
    mu, mv = m.pull_fluid()[:2]
    du, dv = d.pull_fluid()[:2]
    inc = max(np.abs(du - ux).max(), np.abs(dv - uy).max())
    assert max(np.abs(mu - du).max(), np.abs(mv - dv).max()) / inc < 1e-5


@pytest.mark.parametrize("builder", [
    lambda: cases.couette_circle(),
    lambda: cases.poiseuille(itot=384, jtot=768, n=8, a=0.05, b=0.03, seed=6),
    lambda: cases.poiseuille(itot=256, jtot=512, n=24, a=0.04, b=0.02, seed=4),
    lambda: cases.poiseuille(itot=32, jtot=64, n=1, a=0.2, b=0.1, seed=2),
    lambda: cases.poiseuille(itot=1024, jtot=2048, n=16, a=0.02, b=0.01, seed=5),
    lambda: cases.poiseuille(itot=2048, jtot=4096, n=32, a=0.012, b=0.006, seed=3),
    lambda: cases.poiseuille(itot=128, jtot=256, n=4, a=0.06, b=0.03, seed=7),
], ids=["couette_circle", "poiseuille_384x768", "poiseuille_256x512", "poiseuille_32x64", "poiseuille_1024x2048",
        "poiseuille_2048x4096", "poiseuille_128x256"])
def test_mixed_poisson_matches_fp64(builder, gpu_lib):
    """The mixed form's Poisson solve agrees with the double-precision form's to 1e-10
    relative in psi and in the projected velocity. The half lengths m = itot/2 cover
    the refined single-precision solve (register-radix, radix-8, transforms, one
    instance per m) with a last pass of radix 2 (m = 16, 128, 1024), of radix 4
    (m = 32) and without one (m = 64, 512), and the double-float radix-4/2/3 transform
    of the other lengths (m = 192)."""
    from conftest import interior_p
    case = builder()
    d, m = pair(case)
    d.advance(2)
    # a predicted velocity u* (not yet projected) carries a divergence to remove
    d.dt = 1.0e-3
    d.update_velocity(0)
    ux, uy, p, _ = d.pull_fluid()
    for s in (d, m):
        s.push_fluid(ux, uy, p)
        s.dt = 1.0e-3
        s.compute_potential(2)
        s.correct_velocity(2)
    assert d.divergence()[0] < 1e-12 * np.abs(ux).max() * case.itot
    _, _, _, dpsi = d.pull_fluid()
    mu, mv, _, mpsi = m.pull_fluid()
    du, dv, _, _ = d.pull_fluid()
    assert rel_err(interior_p(mpsi), interior_p(dpsi)) < 1e-10
    umag = max(np.abs(du).max(), np.abs(dv).max())
    assert max(np.abs(mu - du).max(), np.abs(mv - dv).max()) / umag < 1e-10


@pytest.mark.parametrize("rows", [4, 8, 16])
def test_tensor_copy_predictor_equals_plain_kernel(rows, gpu_lib, monkeypatch):
    """The mixed predictor whose tiles are staged by bulk tensor copies gives the bits of
    the plain kernel (EIF_NO_TMA=1), for every tile height, on a grid with partial tiles
    in x (itot = 96) and in y (jtot = 200)."""
    monkeypatch.setenv("EIF_TILES", "%d,8,128" % rows)
    case = cases.poiseuille(itot=96, jtot=200, n=6, a=0.06, b=0.03, seed=2)
    a = Simulation.from_case(case, precision=PREC_MIXED)
    monkeypatch.setenv("EIF_NO_TMA", "1")
    b = Simulation.from_case(case, precision=PREC_MIXED)
    a.advance(3)
    b.advance(3)
    assert a.tiles()["predictor_rows"] == rows
    assert a.tiles()["predictor_tensor_copies"] and not b.tiles()["predictor_tensor_copies"]
    for x, y in zip(a.pull_fluid(), b.pull_fluid()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.pull_particles(), b.pull_particles())


@pytest.mark.parametrize("itot,jtot", [(96, 200), (2048, 512)])
def test_uniform_x_metrics_equal_loaded_metrics(itot, jtot, gpu_lib, monkeypatch):
    """The mixed predictor that takes the x metrics as uniform arguments away from the wall
    cells gives the bits of the one that loads them from the arrays (EIF_NO_UNIFORM_X=1),
    plain loads both, tiles partial in x at itot = 96."""
    monkeypatch.setenv("EIF_NO_TMA", "1")
    case = cases.poiseuille(itot=itot, jtot=jtot, n=6, a=0.04, b=0.02, seed=2)
    a = Simulation.from_case(case, precision=PREC_MIXED)
    monkeypatch.setenv("EIF_NO_UNIFORM_X", "1")
    b = Simulation.from_case(case, precision=PREC_MIXED)
    assert a.tiles()["predictor_uniform_x"] and not b.tiles()["predictor_uniform_x"]
    a.advance(3)
    b.advance(3)
    for x, y in zip(a.pull_fluid(), b.pull_fluid()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.pull_particles(), b.pull_particles())
    a.close()
    b.close()


def test_weight_memo_gives_the_same_bits(gpu_lib, monkeypatch):
    """The first indicator evaluation of an RK stage takes the weights of the particles
    whose single-precision geometry is bitwise that of the previous loop's last
    evaluation: the states with and without the memo (EIF_NO_MEMO) are equal bit for
    bit, through the step graphs and through the host-driven stages (kernel timing on),
    and with timing on the memo is seen to serve tasks."""
    case = cases.poiseuille(itot=256, jtot=512, n=24, a=0.04, b=0.02, seed=4)

    def make(memo):
        if memo:
            monkeypatch.delenv("EIF_NO_MEMO", raising=False)
        else:
            monkeypatch.setenv("EIF_NO_MEMO", "1")
        s = Simulation.from_case(case, precision=PREC_MIXED)
        monkeypatch.delenv("EIF_NO_MEMO", raising=False)
        return s

    def same(a, b):
        for x, y in zip(a.pull_fluid(), b.pull_fluid()):
            assert np.array_equal(x, y)
        assert np.array_equal(a.pull_particles(), b.pull_particles())

    off, on = make(False), make(True)
    for s in (off, on):
        s.advance(4)
    same(off, on)
    for s in (off, on):
        s._call("profile_enable", s.ctx, 1)
        s.advance(3)
        s._call("profile_enable", s.ctx, 0)
    same(off, on)
    assert off.memo_count() == 0
    print("tasks from the memo:", on.memo_count(), "box cells evaluated:", on.counters()["indicator_cells"],
          "without the memo:", off.counters()["indicator_cells"])
    assert on.memo_count() > 0
    assert on.counters()["indicator_cells"] < off.counters()["indicator_cells"]


def test_mixed_error_bars_in_a_stirred_state_with_contacts(gpu_lib):
    """The target's error bars at 2048 x 4096 with 2048 ellipses beyond a flow from rest:
    from a stirred channel state with more than 100 ellipses in contact (the state of
    tests/test_gpu_scale_parity.py), 20 steps of both forms, in which collisions act and
    the fixed point takes more sub-iterations. Velocity within 1e-4 relative of the
    double-precision form and maximum divergence below 1e-5; the per-field errors are
    printed."""
    from conftest import interior_p
    from test_gpu_scale_parity import contacts, stirred_contact_state
    case = cases.mixed_target()
    fluid, rec = stirred_contact_state(case)
    d = Simulation(case.config(precision=PREC_FP64))
    m = Simulation(case.config(precision=PREC_MIXED))
    for s in (d, m):
        s.push_fluid(*fluid)
        s.push_particles(rec)
        s.advance(20)
    du, dv, dp, _ = d.pull_fluid()
    mu, mv, mp, _ = m.pull_fluid()
    P, Q = m.pull_particles(), d.pull_particles()
    err = {"u": rel_err(mu, du), "v": rel_err(mv, dv), "p": rel_err(interior_p(mp), interior_p(dp))}
    for f in ("x", "y", "az"):
        err[f] = float(np.max(np.abs(P[:, F[f]] - Q[:, F[f]])))
    err["U, V"] = vec_err(P, Q, "ux", "uy")
    err["Omega"] = rel_err(P[:, F["vz"]], Q[:, F["vz"]])
    div = m.divergence()[0]
    print("stirred 2048x4096, 20 steps: %s, max divergence %.3g, time %.9g vs %.9g, ellipses in contact %d" % (
        {k: "%.3g" % v for k, v in err.items()}, div, m.time_state()[1], d.time_state()[1], contacts(Q)))
    assert contacts(Q) >= 50
    assert max(err["u"], err["v"]) < TOL_VEL
    assert div < TOL_DIV
