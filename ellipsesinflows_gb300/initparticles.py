"""Initial particle sets as the reference's generator makes them
(initparticles/RandomGenerator/src/main.c), with the placement binned.

``generate(n, lx, ly, a, ratio, seed)`` draws, with the C library's rand() after
srand(seed) exactly as the reference does (gen_random, main.c:20-22), the semi-axes
a ~ U[a0, a1], b = a * U[r0, r1] and the angles U[0, 2 pi) of all particles, then
places them by the reference's rejection rule (bounding circles and equivalent
circles of the nearest periodic image must not overlap) through
eif_place_particles, which tests only the ellipses within reach of a candidate
(host code; O(1) per candidate instead of O(N)). Densities are 1 and velocities 0.
``write(dirname, records)`` writes the generator's npy files (main.c:34-46).
With the generator's own parameters (256 ellipses, a = 0.05, b = a/2, lx = 1,
ly = 4, seed 1) the files are byte-identical to the reference's output.
"""
import ctypes
import ctypes.util
import math
import os

import numpy as np

from . import library
from .capi import EifError, F, NFIELDS
from .restart import write_npy

_libc = ctypes.CDLL(ctypes.util.find_library("c"))
_libc.rand.restype = ctypes.c_int
_libc.srand.argtypes = [ctypes.c_uint]
RAND_MAX = 2147483647


def _gen_random(mn, mx):
    # (max - min) * rand() / RAND_MAX + min, in the C evaluation order
    return (mx - mn) * float(_libc.rand()) / float(RAND_MAX) + mn


def generate(n=256, lx=1.0, ly=4.0, a=(0.05, 0.05), ratio=(0.5, 0.5), seed=1, max_tries=10 ** 9):
    """(n, NFIELDS) particle records"""
    _libc.srand(seed)
    as_ = np.empty(n)
    bs = np.empty(n)
    azs = np.empty(n)
    for k in range(n):
        as_[k] = _gen_random(a[0], a[1])
        bs[k] = as_[k] * _gen_random(ratio[0], ratio[1])
        azs[k] = _gen_random(0.0, 2.0 * math.pi)
    xs = np.empty(n)
    ys = np.empty(n)
    lib = library()
    fn = lib.eif_place_particles
    dp = ctypes.POINTER(ctypes.c_double)
    fn.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, dp, dp, dp, dp, dp, ctypes.c_longlong]
    fn.restype = ctypes.c_int
    p = [x.ctypes.data_as(dp) for x in (as_, bs, azs, xs, ys)]
    rc = fn(float(lx), float(ly), int(n), *p, int(max_tries))
    if rc != 0:
        raise EifError(rc, "particle placement failed (more than %d candidates)" % max_tries)
    rec = np.zeros((n, NFIELDS))
    rec[:, F["den"]] = 1.0
    rec[:, F["a"]], rec[:, F["b"]], rec[:, F["az"]] = as_, bs, azs
    rec[:, F["x"]], rec[:, F["y"]] = xs, ys
    return rec


def write(dirname, records):
    """the generator's output files (main.c:34-46) in dirname"""
    os.makedirs(dirname, exist_ok=True)
    rec = np.asarray(records).reshape(-1, NFIELDS)
    write_npy(os.path.join(dirname, "n_particles.npy"), np.int32(rec.shape[0]), "int32")
    for name, field in (("dens", "den"), ("as", "a"), ("bs", "b"), ("xs", "x"), ("ys", "y"), ("azs", "az"),
                        ("uxs", "ux"), ("uys", "uy"), ("vzs", "vz")):
        write_npy(os.path.join(dirname, "particle_%s.npy" % name), rec[:, F[field]], "float64")
