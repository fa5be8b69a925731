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
