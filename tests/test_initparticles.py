"""Initial particle sets: the binned placement (eif_place_particles behind
initparticles.generate) reproduces the reference's own generator
(initparticles/RandomGenerator, built by oracle/ref/Makefile) byte for byte with
its parameters, and keeps its rule at a dense, larger size. CPU only (host code)."""
import os
import subprocess

import numpy as np
import pytest

from ellipsesinflows_gb300 import initparticles
from ellipsesinflows_gb300.capi import F
from oracle import build

HAVE_REF = build.build_ref() if os.path.isdir(os.path.join(build.REFERENCE_DIR, "src")) else False
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference sources not present")
GEN = os.path.join(os.path.dirname(build.__file__), "_ref", "random_generator")


@needs_ref
def test_generator_matches_reference(tmp_path):
    run = tmp_path / "run"
    run.mkdir()
    subprocess.check_call([GEN], cwd=run, stdout=subprocess.DEVNULL)   # writes into tmp_path
    rec = initparticles.generate()
    initparticles.write(str(tmp_path / "ours"), rec)
    names = sorted(f for f in os.listdir(tmp_path) if f.endswith(".npy"))
    assert len(names) == 10
    for name in names:
        assert (tmp_path / name).read_bytes() == (tmp_path / "ours" / name).read_bytes(), name


def test_dense_placement_keeps_the_rule():
    # 2048 ellipses, a = 0.012, aspect ratio 1.7 to 2.5, about 23 % area in 1 x 2
    rec = initparticles.generate(n=2048, lx=1.0, ly=2.0, a=(0.012, 0.012), ratio=(0.4, 0.6), seed=3)
    x, y, a, b = rec[:, F["x"]], rec[:, F["y"]], rec[:, F["a"]], rec[:, F["b"]]
    r = np.maximum(a, b)
    frac = np.sum(np.pi * a * b) / 2.0
    assert 0.2 < frac < 0.26
    assert np.all(x >= r) and np.all(x <= 1 - r) and np.all((y >= 0) & (y < 2))
    # bounding circles of the nearest periodic images do not overlap
    dy = y[:, None] - y[None, :]
    dy = np.minimum(np.abs(dy), 2.0 - np.abs(dy))
    d = np.hypot(x[:, None] - x[None, :], dy)
    np.fill_diagonal(d, np.inf)
    assert np.all(d >= r[:, None] + r[None, :])
