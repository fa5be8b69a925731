"""The CPU oracles: the reference built from its own sources (oracle/_ref) and
the C restatement (oracle/port). The restatement is pinned bit-for-bit to the
reference build and to the committed golden vectors, which were produced by the
reference build (tests/golden/make_golden.py)."""
import os
import subprocess

import numpy as np
import pytest
import scipy.fft

from conftest import GOLDEN, interior_p, rel_err
from ellipsesinflows_gb300 import cases
from ellipsesinflows_gb300.capi import F, NFIELDS
from oracle import build, port

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HAVE_REF = build.build_ref() if os.path.isdir(os.path.join(build.REFERENCE_DIR, "src")) else False
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference sources not present")


def port_from_case(case, threads=1):
    s = port.PortSolver(case.config(), threads=threads)
    s.push_fluid(*case.fluid())
    s.push_particles(case.particles)
    return s


def ref_from_case(case):
    from oracle import ref
    variant = "couette" if case.uy_wall == (-0.5, 0.5) else "default"
    s = ref.RefSolver(case.itot, case.jtot, case.ly, case.Re, case.Fr, case.extfrcy, case.safefactors, variant=variant)
    s.set_fluid(*case.fluid())
    s.set_particles(case.particles)
    return s


# ---------------------------------------------------------------------------
# shims of the reference build

@needs_ref
@pytest.mark.parametrize("shape", [(64, 128), (3, 5), (384, 768), (1, 1)])
def test_mpi_shim_passes_reference_transpose_selftest(shape):
    exe = os.path.join(ROOT, "oracle", "_ref", "transpose_selftest")
    subprocess.check_call([exe, str(shape[0]), str(shape[1])])


def _dct_via_port_lib(x, kind):
    import ctypes
    lib = ctypes.CDLL(build.build_port())
    lib.fftw_plan_r2r_1d.restype = ctypes.c_void_p
    lib.fftw_plan_r2r_1d.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint]
    lib.fftw_execute.argtypes = [ctypes.c_void_p]
    lib.fftw_destroy_plan.argtypes = [ctypes.c_void_p]
    buf = np.ascontiguousarray(x, dtype=np.float64).copy()
    plan = lib.fftw_plan_r2r_1d(len(buf), buf.ctypes.data, buf.ctypes.data, 4 if kind == 2 else 5, 0)
    lib.fftw_execute(plan)
    lib.fftw_destroy_plan(plan)
    return buf


@pytest.mark.parametrize("n", [1, 2, 3, 8, 12, 64, 96, 128, 384, 1000, 2048])
@pytest.mark.parametrize("kind", [2, 3])
def test_dct_shim_matches_scipy(n, kind):
    x = np.random.default_rng(n).standard_normal(n)
    y = _dct_via_port_lib(x, kind)
    assert rel_err(y, scipy.fft.dct(x, type=kind)) < 5e-15


# ---------------------------------------------------------------------------
# restatement == reference build, bit for bit

@needs_ref
@pytest.mark.parametrize("builder,steps", [
    (lambda: cases.couette_circle(), 20),
    (lambda: cases.contact_cluster(), 20),
    (lambda: cases.poiseuille(itot=64, jtot=128, n=6, a=0.08, b=0.05, seed=5), 10),
    (lambda: cases.poiseuille(itot=96, jtot=192, n=10, a=0.05, b=0.03, seed=9), 3),
])
def test_port_bit_identical_to_reference(builder, steps):
    case = builder()
    p, r = port_from_case(case), ref_from_case(case)
    for _ in range(steps):
        assert p.step() == r.step()
    for a, b in zip(p.pull_fluid(), r.get_fluid()):
        assert np.array_equal(a, b)
    assert np.array_equal(p.pull_particles(), r.get_particles())
    assert p.dt == r.dt


@needs_ref
def test_port_stages_bit_identical_to_reference():
    case = cases.contact_cluster()
    p, r = port_from_case(case), ref_from_case(case)
    p.dt = r.dt = 1.0e-3
    for rk in range(3):
        p.reset_particle_increments(); r.reset_increments()
        p.compute_inertia(0); r.compute_inertia(0)
        p.update_velocity(rk); r.update_velocity(rk)
        pa = p.pull_src(); ra = r.get_src()
        assert np.array_equal(pa[0], ra[0]) and np.array_equal(pa[1], ra[1])
        assert np.array_equal(pa[2], ra[3]) and np.array_equal(pa[3], ra[4])
        p.exchange_momentum(); r.exchange_momentum()
        for a, b in zip(p.pull_ibm_fields(), r.get_ibm_fields()):
            assert np.array_equal(a, b)
        p.update_momentum_field(); r.update_momentum_field()
        p.compute_potential(rk); r.compute_potential(rk)
        p.correct_velocity(rk); r.correct_velocity(rk)
        p.update_pressure(); r.update_pressure()
        p.compute_collision_force(0); r.collision(0)
        p.compute_inertia(1); r.compute_inertia(1)
        p.compute_collision_force(1); r.collision(1)
        assert p.increment_particles(rk) == r.increment(rk)
        p.update_particles(); r.update_particles()
        for a, b in zip(p.pull_fluid(), r.get_fluid()):
            assert np.array_equal(a, b)
        assert np.array_equal(p.pull_particles(), r.get_particles())


@needs_ref
def test_reference_integrate_counted_equals_integrate():
    """The instrumented driver loop (substep counts) is the reference's integrate()."""
    case = cases.contact_cluster()
    a, b = ref_from_case(case), ref_from_case(case)
    for _ in range(3):
        a.decide_dt(); b.decide_dt()
        a.integrate(); b.integrate_counted()
    for x, y in zip(a.get_fluid(), b.get_fluid()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.get_particles(), b.get_particles())


# ---------------------------------------------------------------------------
# restatement == golden vectors (runs anywhere)

@pytest.mark.parametrize("name,builder", [
    ("couette_circle_64x128.npz", lambda: cases.couette_circle()),
    ("contact_cluster_64x128.npz", lambda: cases.contact_cluster()),
    ("poiseuille_64x128_n6.npz", lambda: cases.poiseuille(itot=64, jtot=128, n=6, a=0.08, b=0.05, seed=5)),
])
def test_port_matches_golden_first_step(name, builder, golden):
    g = golden(name)
    p = port_from_case(builder())
    sub = p.step()
    assert sub == list(g["substeps"][0])
    ux, uy, pp, _ = p.pull_fluid()
    # bit-identical on the machine that produced the fixtures; within rounding of libm elsewhere
    assert rel_err(ux, g["ux_1"]) < 1e-13
    assert rel_err(uy, g["uy_1"]) < 1e-13
    assert rel_err(interior_p(pp), interior_p(g["p_1"])) < 1e-12
    assert rel_err(p.pull_particles(), g["particles_1"]) < 1e-13


def test_port_matches_golden_couette_200_steps(golden):
    g = golden("couette_circle_64x128.npz")
    p = port_from_case(cases.couette_circle())
    for k in range(200):
        p.step()
    ux, uy, pp, _ = p.pull_fluid()
    assert rel_err(ux, g["ux_200"]) < 1e-10
    assert rel_err(uy, g["uy_200"]) < 1e-10
    P = p.pull_particles()
    assert abs(P[0, F["x"]] - g["particles_200"][0, F["x"]]) < 1e-10
    assert abs(P[0, F["az"]] - g["particles_200"][0, F["az"]]) < 1e-10


def test_port_geometry_matches_golden(golden):
    g = golden("geometry.npz")
    t = np.array([port.find_normal_t(*v) for v in zip(g["a"], g["b"], g["x"], g["y"])])
    assert np.max(np.abs(t - g["t"])) < 1e-13
    h = float(g["h"])
    args = list(zip(g["a"], g["b"], g["px"], g["py"], g["az"], g["qx"], g["qy"]))
    sw = np.array([port.s_weight(h, *v) for v in args])
    vw = np.array([port.v_weight(h, *v) for v in args])
    assert np.max(np.abs(sw - g["s_weight"])) < 1e-13
    assert np.max(np.abs(vw - g["v_weight"])) < 1e-13


def test_port_thread_count_does_not_change_results():
    case = cases.poiseuille(itot=64, jtot=128, n=6, a=0.08, b=0.05, seed=5)
    a, b = port_from_case(case, threads=1), port_from_case(case, threads=4)
    for _ in range(3):
        a.step(); b.step()
    for x, y in zip(a.pull_fluid(), b.pull_fluid()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.pull_particles(), b.pull_particles())


def test_port_rejects_bad_stage_index():
    from ellipsesinflows_gb300.capi import EifError
    p = port_from_case(cases.couette_circle())
    with pytest.raises(EifError):
        p.update_velocity(3)
    with pytest.raises(EifError):
        p.compute_inertia(2)


def test_port_circle_fit_cap_reports_error():
    """A contact that the reference's uncapped fixed point never leaves
    (src/suspensions/collision.c:141-152) returns an error instead of hanging."""
    from ellipsesinflows_gb300.capi import EifError
    case = cases.contact_cluster()
    P = case.particles[4:5].copy()
    P[0, F["x"]] = 0.95  # ellipse pushed 0.02 through the wall x = 1
    s = port.PortSolver(case.config())
    s.push_fluid(*case.fluid())
    s.push_particles(P)
    with pytest.raises(EifError):
        s.compute_collision_force(0)
