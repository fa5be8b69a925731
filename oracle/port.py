"""ctypes binding of the C restatement oracle (oracle/port/eif_port.c).

TEST INFRASTRUCTURE ONLY. It exposes the eif.h entry points with the prefix
``eifo_`` on host memory; ``PortSolver`` is the same binding class as the
product's, so a test drives both with identical calls.
"""
import ctypes
import os

from ellipsesinflows_gb300.capi import Solver, bind, make_config  # noqa: F401

from . import build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build.build_port()
        l = ctypes.CDLL(path)
        bind(l, "eifo_")
        for name in ("find_normal_t",):
            fn = getattr(l, "eifo_" + name)
            fn.argtypes = [ctypes.c_double] * 4
            fn.restype = ctypes.c_double
        for name in ("s_weight", "v_weight"):
            fn = getattr(l, "eifo_" + name)
            fn.argtypes = [ctypes.c_double] * 8
            fn.restype = ctypes.c_double
        _lib = l
    return _lib


class PortSolver(Solver):
    def __init__(self, cfg, threads=1):
        super().__init__(lib(), "eifo_", cfg)
        self.set_threads(threads)


def find_normal_t(a, b, x, y):
    return lib().eifo_find_normal_t(a, b, x, y)


def s_weight(h, a, b, px, py, paz, x, y):
    return lib().eifo_s_weight(h, a, b, px, py, paz, x, y)


def v_weight(h, a, b, px, py, paz, x, y):
    return lib().eifo_v_weight(h, a, b, px, py, paz, x, y)
