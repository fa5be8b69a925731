"""The C ABI from a plain C host on the GPU: tests/c/eif_abi_run.c (C99, only
include/eif.h) is built with gcc against libeif_gb300.so, advances a case read from a
file, and its state after the steps equals bit for bit the same case advanced through
the Python binding, in both precision forms."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, build, cases
from ellipsesinflows_gb300.capi import NFIELDS

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STEPS = 5


@pytest.fixture(scope="module")
def c_host(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = build.build()
    exe = str(tmp_path_factory.mktemp("c_host") / "eif_abi_run")
    subprocess.run([cc, "-std=c99", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(HERE, "c", "eif_abi_run.c"), "-o", exe, "-L" + os.path.dirname(lib),
                    "-leif_gb300", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def write_case(path, case, precision, nsteps):
    ux, uy, p = (np.ascontiguousarray(a, dtype=np.float64) for a in case.fluid())
    rec = np.ascontiguousarray(case.particles, dtype=np.float64)
    hdr = np.array([case.itot, case.jtot, precision, nsteps, len(rec)], dtype=np.int32)
    par = np.array([case.ly, case.Re, case.Fr, case.extfrcy, *case.safefactors, *case.uy_wall], dtype=np.float64)
    with open(path, "wb") as f:
        for a in (hdr, par, ux, uy, p, rec):
            f.write(a.tobytes())


def read_result(path, case, n):
    it, jt = case.itot, case.jtot
    raw = open(path, "rb").read()
    step = int(np.frombuffer(raw, np.int32, 1)[0])
    vals = np.frombuffer(raw, np.float64, offset=4)
    time, vals = vals[0], vals[1:]
    sizes = [(jt + 2) * (it + 1), (jt + 2) * (it + 2), (jt + 2) * (it + 2), n * NFIELDS]
    out, k = [], 0
    for s in sizes:
        out.append(vals[k:k + s])
        k += s
    return step, time, out


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED], ids=["fp64", "mixed"])
def test_c_host_advances_like_the_python_binding(c_host, prec, tmp_path):
    case = cases.poiseuille(itot=128, jtot=256, n=8, a=0.05, b=0.025, seed=11)
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_case(src, case, prec, STEPS)
    run = subprocess.run([c_host, src, dst], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    step, time, (ux, uy, p, rec) = read_result(dst, case, len(case.particles))

    sim = Simulation.from_case(case, precision=prec)
    sim.advance(STEPS)
    pux, puy, pp, _ = sim.pull_fluid()
    assert (step, time) == sim.time_state()
    assert np.array_equal(ux, pux.ravel())
    assert np.array_equal(uy, puy.ravel())
    assert np.array_equal(p, pp.ravel())
    assert np.array_equal(rec, sim.pull_particles().ravel())
