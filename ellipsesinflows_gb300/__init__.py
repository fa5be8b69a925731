"""EllipsesInFlows-GB300: the time-step hot path of EllipsesInFlows on one GB300.

The compute path is the CUDA library ``libeif_gb300.so`` (csrc/, built for
sm_103a by ``build.build()``) behind the C ABI of include/eif.h. This package
is the Python host side of that ABI: ``Simulation`` wraps one context, and
``cases`` builds the initial states of the benchmark configurations.

There is no CPU fallback: ``Simulation`` raises if the library cannot be
loaded.
"""
import ctypes
import os

from . import capi
from .capi import (Batch, EifError, F, FIELDS, NFIELDS, PREC_FP64, PREC_MIXED,  # noqa: F401
                   make_config)

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libeif_gb300.so")

_lib = None


def library():
    """Load (once) and return the in-tree CUDA library; raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libeif_gb300.so is not built: run ellipsesinflows_gb300.build.build()")
        lib = ctypes.CDLL(LIB_PATH)
        capi.bind(lib, "eif_")
        _lib = lib
    return _lib


class Simulation(capi.Solver):
    """One suspension advanced on the GPU through the eif.h C ABI."""

    def __init__(self, cfg):
        super().__init__(library(), "eif_", cfg)

    @classmethod
    def from_case(cls, case, precision=PREC_FP64, device=0):
        cfg = case.config(precision=precision, device=device)
        sim = cls(cfg)
        sim.push_fluid(*case.fluid())
        sim.push_particles(case.particles)
        return sim
