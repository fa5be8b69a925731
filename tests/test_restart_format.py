"""Checkpoint files in the reference's format (src/save.c:13-122): the package's
writer produces the reference save()'s files byte for byte for the same state, and
reads them back. CPU only."""
import os

import numpy as np
import pytest

from ellipsesinflows_gb300 import cases, restart
from oracle import build, ref

HAVE_REF = build.build_ref() if os.path.isdir(os.path.join(build.REFERENCE_DIR, "src")) else False
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference sources not present")


@needs_ref
def test_checkpoint_files_match_reference_save(tmp_path, monkeypatch):
    case = cases.poiseuille(itot=64, jtot=128, n=6, a=0.08, b=0.05, seed=5)
    s = ref.RefSolver(case.itot, case.jtot, case.ly, case.Re, case.Fr, case.extfrcy, case.safefactors)
    s.set_fluid(*case.fluid())
    s.set_particles(case.particles)
    for _ in range(2):
        s.step()
    step, time = 17, 0.1234567890123
    (tmp_path / "ref" / "output" / "save").mkdir(parents=True)
    monkeypatch.chdir(tmp_path / "ref")
    assert s.save(step, time) == 0
    ux, uy, p, _ = s.get_fluid()
    rec = s.get_particles()
    d = restart.write_state(str(tmp_path / "ours"), case.config(), ux, uy, p, rec, step, time)
    refdir = tmp_path / "ref" / "output" / "save" / ("step%010d" % step)
    names = sorted(os.listdir(refdir))
    assert names == sorted(os.listdir(d))
    for name in names:
        assert (refdir / name).read_bytes() == open(os.path.join(d, name), "rb").read(), name
    # and back: the fields without halo rows, the 9 particle fields, step and time
    gux, guy, gp, grec, gstep, gtime = restart.read_state(str(refdir))
    assert np.array_equal(gux[1:-1], ux[1:-1]) and np.array_equal(guy[1:-1], uy[1:-1])
    assert np.array_equal(gp[1:-1], p[1:-1])
    assert (gstep, gtime) == (step, time)
    from ellipsesinflows_gb300.capi import F
    for f in ("den", "a", "b", "x", "y", "az", "ux", "uy", "vz"):
        assert np.array_equal(grec[:, F[f]], rec[:, F[f]])
    s.close()
