"""The drop-in driver (ellipsesinflows_gb300/driver: the reference's main program with
the step through libeif_gb300.so, linked with the reference's own parameter, npy I/O,
logging, save and statistics code) builds against the reference sources and runs the
reference's initialisation from its environment variables and initparticles/ files up
to the GPU context. CPU only: without a GPU it stops at eif_create; the reference
sources are not present where the GPU is."""
import os
import subprocess

import pytest

from ellipsesinflows_gb300 import initparticles
from oracle import build

HERE = os.path.dirname(os.path.abspath(__file__))
DRIVER = os.path.join(os.path.dirname(HERE), "ellipsesinflows_gb300", "driver")
HAVE_REF = os.path.isdir(os.path.join(build.REFERENCE_DIR, "src"))
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference sources not present")


@needs_ref
def test_driver_builds_and_initialises(tmp_path):
    subprocess.check_call(["make", "-s", "-C", DRIVER, "REF=" + build.REFERENCE_DIR])
    exe = os.path.join(DRIVER, "_build", "eif_main_default")
    assert os.path.exists(exe)
    rec = initparticles.generate(n=4, ly=2.0, a=(0.05, 0.05), ratio=(0.5, 0.5), seed=2)
    initparticles.write(str(tmp_path / "initparticles"), rec)
    env = dict(os.environ, itot="64", jtot="128", ly="2.0", Re="100", timemax="0.01")
    r = subprocess.run([exe], cwd=tmp_path, env=env, capture_output=True, text=True, timeout=120)
    out = r.stdout + r.stderr
    assert "parameters are loaded" in out           # the reference's param_init ran
    if r.returncode != 0:
        # no GPU here: the driver stops at the context creation with the library's message
        assert "eif_create failed" in out, out
