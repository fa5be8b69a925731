"""Initial-state builders of the benchmark configurations."""
import math

import numpy as np

from ellipsesinflows_gb300 import cases
from ellipsesinflows_gb300.capi import F


def min_gap(P, ly):
    x, y, a, b = P[:, F["x"]], P[:, F["y"]], P[:, F["a"]], P[:, F["b"]]
    r = np.maximum(a, b)
    gap = np.inf
    for i in range(len(x)):
        dy = np.abs(y[i + 1:] - y[i])
        dy = np.minimum(dy, ly - dy)
        d = np.hypot(x[i + 1:] - x[i], dy) - r[i] - r[i + 1:]
        if d.size:
            gap = min(gap, d.min())
    return gap


def test_poiseuille_placement_is_seeded_and_clear():
    c1, c2 = cases.poiseuille(), cases.poiseuille()
    assert np.array_equal(c1.particles, c2.particles)
    assert c1.n_particles == 128
    assert min_gap(c1.particles, 2.0) >= 1.0 / 512 - 1e-12
    x, r = c1.particles[:, F["x"]], c1.particles[:, F["a"]]
    assert np.all(x - r > 0) and np.all(x + r < 1)


def test_mixed_target_statistics():
    c = cases.mixed_target()
    P = c.particles
    assert c.n_particles == 2048
    ar = P[:, F["a"]] / P[:, F["b"]]
    assert 1.0 <= ar.min() and ar.max() <= 3.0
    assert 1.0 <= P[:, F["den"]].min() and P[:, F["den"]].max() <= 1.2
    area = np.sum(math.pi * P[:, F["a"]] * P[:, F["b"]]) / 2.0
    assert 0.15 < area < 0.3
    assert min_gap(P, 2.0) >= 1.0 / 2048 - 1e-12


def test_couette_initial_profile():
    c = cases.couette_circle()
    ux, uy, p = c.fluid()
    xc = c.xc()
    assert np.allclose(uy[5, 1:-1], -0.5 + xc[1:-1])
    assert np.all(ux == 0) and np.all(p == 0)


def test_place_ellipses_keeps_ellipses_apart():
    """256 ellipses a = 0.04, aspect ratio U[1, 2.5] in the 1 x 2 channel (the largest
    suspension of the batch workload): no ellipse, grown by the clearance less a
    margin, contains a point of another's boundary sampled 4x finer than the
    placement's test; the bounding circles do overlap (a denser packing than the
    bounding-circle rule allows)."""
    import math
    import numpy as np
    from ellipsesinflows_gb300 import cases
    rng = np.random.default_rng(8)
    n, a, ly, clr = 256, 0.04, 2.0, 1.0 / 512
    ar = rng.uniform(1.0, 2.5, n)
    az = rng.uniform(0.0, math.pi, n)
    A, B = np.full(n, a), a / ar
    xs, ys = cases.place_ellipses(A, B, az, ly, clr, rng, clr)
    overlapping_discs = 0
    for k in range(n):
        for m in range(k):
            dy = ys[k] - ys[m]
            dy -= ly * round(dy / ly)
            if math.hypot(xs[k] - xs[m], dy) < 2 * a:
                overlapping_discs += 1
            else:
                continue
            ym = ys[k] - dy
            px, py = cases._boundary(A[k], B[k], az[k], xs[k], ys[k], k=288)
            qx, qy = cases._boundary(A[m], B[m], az[m], xs[m], ym, k=288)
            c = 0.5 * clr
            assert not cases._inside(px, py, A[m] + c, B[m] + c, az[m], xs[m], ym).any()
            assert not cases._inside(qx, qy, A[k] + c, B[k] + c, az[k], xs[k], ys[k]).any()
    assert overlapping_discs > 0
    assert np.all((xs > a) & (xs < 1 - a)) and np.all((ys >= 0) & (ys < ly))
