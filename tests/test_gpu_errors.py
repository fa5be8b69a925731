"""Device error returns: each bounded device-side limit, driven to its error status by
host-made inputs, and the context still usable afterwards.

* the equivalent-circle fit (src/suspensions/collision.c:117-133,141-152 has no cap; a
  contact pushed through a wall never converges there) stops after 10 000 iterations
  and the call returns EIF_ERR_NOCONV;
* the collision partner list (64 candidates per particle) reports an overflow as
  EIF_ERR_NOCONV;
* a NaN in the velocity field is reported as EIF_ERR_NONFINITE by the time-step
  decision (src/param/decide_dt.c:25-56 reads every velocity), through eif_decide_dt
  and through eif_advance, whose counters then include the one step queued after the
  failing one.

The per-band box lists of the field gather hold 3 x (particle count) entries per band,
one per (particle, periodic image) box, so no input can overflow them; their guard is
not reachable from the C ABI and has no test here.
"""
import numpy as np
import pytest

from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, cases
from ellipsesinflows_gb300.capi import EifError, F
from ellipsesinflows_gb300.cases import particle_records

pytestmark = pytest.mark.gpu

NOCONV, NONFINITE = -3, -6


def wall_contact_case():
    case = cases.contact_cluster()
    rec = case.particles[4:5].copy()
    rec[0, F["x"]] = 0.95   # ellipse a = 0.07 pushed 0.02 through the wall x = 1
    return case, rec


def crowded_circles(n=70, r=0.02, seed=4):
    """n circles whose centres lie within 0.75 r of one point: every pair's bounding
    circles overlap, so each particle has n - 1 > 64 collision candidates."""
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0.0, 2 * np.pi, n)
    rad = 0.75 * r * np.sqrt(rng.uniform(0.0, 1.0, n))
    x, y = 0.5 + rad * np.cos(ang), 1.0 + rad * np.sin(ang)
    return particle_records(np.ones(n), np.full(n, r), np.full(n, r), x, y, np.zeros(n))


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED], ids=["fp64", "mixed"])
def test_circle_fit_cap_returns_noconv(prec, gpu_lib):
    case, rec = wall_contact_case()
    g = Simulation(case.config(precision=prec))
    g.push_fluid(*case.fluid())
    g.push_particles(rec)
    with pytest.raises(EifError) as err:
        g.compute_collision_force(0)
    assert err.value.code == NOCONV
    # the same contact inside whole steps
    with pytest.raises(EifError) as err:
        g.advance(1)
    assert err.value.code == NOCONV
    # the context stays usable: a contact-free state steps normally
    ok = case.particles[4:5].copy()
    g.push_fluid(*case.fluid())
    g.push_particles(ok)
    g.advance(2)
    assert np.isfinite(g.pull_particles()).all()


def test_partner_list_overflow_returns_noconv(gpu_lib):
    case = cases.poiseuille(itot=64, jtot=128, n=1, a=0.05, b=0.03, seed=1)
    g = Simulation(case.config())
    g.push_fluid(*case.fluid())
    g.push_particles(crowded_circles())
    with pytest.raises(EifError) as err:
        g.compute_collision_force(0)
    assert err.value.code == NOCONV
    # 64 partners fit: 65 circles give every particle exactly 64 candidates
    g.push_particles(crowded_circles(n=65))
    g.compute_collision_force(0)


def _fluid_state(case):
    ux, uy, p = (np.array(a) for a in case.fluid())
    uy[:, 1:-1] += 0.1
    return ux, uy, p


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED], ids=["fp64", "mixed"])
def test_nonfinite_velocity_returns_nonfinite(prec, gpu_lib):
    case = cases.poiseuille(itot=64, jtot=128, n=1, a=0.05, b=0.03, seed=1)
    g = Simulation(case.config(precision=prec))
    ux, uy, p = _fluid_state(case)
    g.push_particles(case.particles[:0])
    bad = ux.copy()
    bad[40, 20] = np.nan
    g.push_fluid(bad, uy, p)
    with pytest.raises(EifError) as err:
        g.decide_dt()
    assert err.value.code == NONFINITE
    # through the queued step graphs: step 1 fails, step 2 had been launched already
    g.push_fluid(bad, uy, p)
    g.set_time(0, 0.0)
    with pytest.raises(EifError) as err:
        g.advance(3)
    assert err.value.code == NONFINITE
    step, _ = g.time_state()
    assert step == 2
    # a finite state afterwards steps normally
    g.push_fluid(ux, uy, p)
    g.set_time(0, 0.0)
    g.advance(2)
    assert g.time_state()[0] == 2
    assert np.isfinite(g.pull_fluid()[0]).all()
