"""The C ABI library without a GPU: it builds, loads, and exports every entry
point that include/eif.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "eif.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void \*|const char \*)\s*(eif_\w+)\s*\(", text, re.M)))


def test_library_builds_and_exports_declared_symbols():
    from ellipsesinflows_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_simulation_fails_loudly_without_library(monkeypatch):
    import ellipsesinflows_gb300 as pkg
    monkeypatch.setattr(pkg, "LIB_PATH", os.path.join(ROOT, "does-not-exist.so"))
    monkeypatch.setattr(pkg, "_lib", None)
    with pytest.raises(RuntimeError):
        pkg.library()


def test_create_rejects_invalid_configuration():
    """Argument checks run before any CUDA call."""
    from ellipsesinflows_gb300 import build, capi
    lib = capi.bind(ctypes.CDLL(build.build()), "eif_")
    ctx = ctypes.c_void_p()
    cfg = capi.make_config(2, 2)
    rc = lib.eif_create(ctypes.byref(cfg), ctypes.byref(ctx))
    assert rc == -1
    lib.eif_destroy(ctx)


def test_plain_c_host_builds_against_the_header(tmp_path):
    """tests/c/eif_abi_run.c, a C99 host that uses only include/eif.h, compiles without
    warnings and links against the library (it runs on the GPU in
    tests/test_gpu_c_host.py)."""
    import shutil
    import subprocess
    from ellipsesinflows_gb300 import build
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = build.build()
    exe = str(tmp_path / "eif_abi_run")
    subprocess.run([cc, "-std=c99", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "eif_abi_run.c"), "-o", exe, "-L" + os.path.dirname(lib),
                    "-leif_gb300", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    run = subprocess.run([exe], capture_output=True, text=True)
    assert run.returncode == 2 and "usage" in run.stderr
