"""eif_decide_dt_noalloc: the time step computed from the caller's own device
arrays with no device allocation (for callers that cannot let a library call
cudaMalloc), checked against eif_decide_dt on the same state.

This file is collected last so that a run which stops at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

from ellipsesinflows_gb300 import Simulation, cases

pytestmark = pytest.mark.gpu

EIF_ERR_TOO_LARGE = -7
EIF_NOALLOC_MAX_ITOT = 16384


def noalloc_fn(lib):
    fn = lib.eif_decide_dt_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                   ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def state_after(case, steps):
    sim = Simulation.from_case(case)
    sim.advance(steps)
    ux, uy, p, _ = sim.pull_fluid()
    return sim, ux, uy, sim.pull_particles()


def call_noalloc(fn, case, ux, uy, parts):
    import torch
    dev = torch.device("cuda:0")
    dux = torch.from_numpy(np.ascontiguousarray(ux)).to(dev)
    duy = torch.from_numpy(np.ascontiguousarray(uy)).to(dev)
    dpart = torch.from_numpy(np.ascontiguousarray(parts)).to(dev)
    dt = torch.zeros(1, dtype=torch.float64, device=dev)
    sf = (ctypes.c_double * 3)(*case.safefactors)
    stream = torch.cuda.current_stream(dev)
    rc = fn(dux.data_ptr(), ux.shape[1], duy.data_ptr(), uy.shape[1], case.itot, case.jtot, case.ly, case.Re, sf,
            dpart.data_ptr(), parts.shape[0], dt.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)
    assert rc == 0, rc
    return float(dt.item())


def test_noalloc_dt_matches_decide_dt_on_two_calls_in_a_row(gpu_lib):
    fn = noalloc_fn(gpu_lib)
    # first state: a suspension driven for a few steps (large velocities)
    case_a = cases.contact_cluster()
    sim_a, ux_a, uy_a, p_a = state_after(case_a, 3)
    # second state on a different grid, with smaller velocities than the first: a
    # call that kept the previous maxima in the shared scratch would return a wrong dt
    case_b = cases.poiseuille(itot=96, jtot=192, n=4, a=0.06, b=0.03, seed=2)
    sim_b, ux_b, uy_b, p_b = state_after(case_b, 1)
    assert max(np.abs(uy_b).max(), np.abs(ux_b).max()) < max(np.abs(uy_a).max(), np.abs(ux_a).max())
    ref_a = sim_a.decide_dt()
    ref_b = sim_b.decide_dt()
    for _ in range(2):
        assert call_noalloc(fn, case_a, ux_a, uy_a, p_a) == ref_a
        assert call_noalloc(fn, case_b, ux_b, uy_b, p_b) == ref_b


def test_noalloc_dt_is_nan_for_a_nonfinite_velocity(gpu_lib):
    """One NaN cell: eif_decide_dt reports EIF_ERR_NONFINITE, this entry point returns a
    NaN step; a following call on a finite state gets its dt again (the marker in the
    shared scratch is cleared by every call)."""
    from ellipsesinflows_gb300.capi import EifError
    fn = noalloc_fn(gpu_lib)
    case = cases.contact_cluster()
    sim, ux, uy, parts = state_after(case, 2)
    ref = sim.decide_dt()
    bad = ux.copy()
    bad[case.jtot // 2, case.itot // 3] = np.nan
    assert np.isnan(call_noalloc(fn, case, bad, uy, parts))
    sim.push_fluid(bad, uy, sim.pull_fluid()[2])
    with pytest.raises(EifError) as err:
        sim.decide_dt()
    assert err.value.code == -6
    assert call_noalloc(fn, case, ux, uy, parts) == ref


def test_noalloc_rejects_grids_beyond_its_scratch(gpu_lib):
    fn = noalloc_fn(gpu_lib)
    sf = (ctypes.c_double * 3)(0.75, 0.75, 0.95)
    # the size check comes before any device access
    rc = fn(ctypes.c_void_p(16), EIF_NOALLOC_MAX_ITOT + 2, ctypes.c_void_p(16), EIF_NOALLOC_MAX_ITOT + 3,
            EIF_NOALLOC_MAX_ITOT + 1, 8, 1.0, 100.0, sf, None, 0, ctypes.c_void_p(16), None)
    assert rc == EIF_ERR_TOO_LARGE
