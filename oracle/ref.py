"""ctypes binding of the reference-built CPU oracle (oracle/_ref/libeifref*.so).

TEST INFRASTRUCTURE ONLY. The libraries are the reference solver's unmodified
sources plus single-rank MPI/FFTW shims and a step-driven driver
(oracle/ref/ref_driver.c). Particle records are 30 doubles in the order of the
reference's ``particle_t`` (include/suspensions.h:8-31).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "_ref")
NFIELDS = 30

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_libs = {}


def available(variant="default"):
    return os.path.exists(_libpath(variant))


def _libpath(variant):
    name = "libeifref.so" if variant == "default" else "libeifref_%s.so" % variant
    return os.path.join(LIBDIR, name)


def _lib(variant):
    if variant not in _libs:
        lib = ctypes.CDLL(_libpath(variant))
        vp = ctypes.c_void_p
        lib.ref_create.restype = vp
        lib.ref_create.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 7
        lib.ref_destroy.argtypes = [vp]
        for name in ("ref_set_fluid",):
            getattr(lib, name).argtypes = [vp, _dp, _dp, _dp]
        lib.ref_get_fluid.argtypes = [vp, _dp, _dp, _dp, _dp]
        lib.ref_get_src.argtypes = [vp] + [_dp] * 6
        lib.ref_set_src.argtypes = [vp, _dp, _dp]
        lib.ref_get_ibm_fields.argtypes = [vp, _dp, _dp]
        lib.ref_set_particles.argtypes = [vp, ctypes.c_int, _dp]
        lib.ref_get_particles.argtypes = [vp, _dp]
        lib.ref_get_dt.restype = ctypes.c_double
        lib.ref_get_dt.argtypes = [vp]
        lib.ref_set_dt.argtypes = [vp, ctypes.c_double]
        lib.ref_get_time.restype = ctypes.c_double
        lib.ref_get_time.argtypes = [vp]
        lib.ref_get_step.argtypes = [vp]
        lib.ref_get_grid.argtypes = [vp] + [_dp] * 6
        lib.ref_logging.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        lib.ref_save.argtypes = [vp, ctypes.c_int, ctypes.c_double]
        lib.ref_stats_collect.argtypes = [vp]
        lib.ref_stats_output.argtypes = [vp, ctypes.c_int, ctypes.c_double]
        lib.ref_decide_dt.restype = ctypes.c_double
        lib.ref_decide_dt.argtypes = [vp]
        lib.ref_integrate.argtypes = [vp]
        lib.ref_integrate_counted.argtypes = [vp, _ip]
        lib.ref_step.argtypes = [vp, ctypes.c_int, _ip]
        for name in ("ref_update_boundaries", "ref_reset_increments", "ref_exchange_momentum",
                     "ref_update_momentum_field", "ref_update_pressure", "ref_update_particles"):
            getattr(lib, name).argtypes = [vp]
        for name in ("ref_compute_inertia", "ref_update_velocity", "ref_compute_potential",
                     "ref_correct_velocity", "ref_collision"):
            getattr(lib, name).argtypes = [vp, ctypes.c_int]
        lib.ref_increment.restype = ctypes.c_double
        lib.ref_increment.argtypes = [vp, ctypes.c_int]
        lib.ref_find_normal_t.restype = ctypes.c_double
        lib.ref_find_normal_t.argtypes = [ctypes.c_double] * 4
        for name in ("ref_s_weight", "ref_v_weight"):
            getattr(lib, name).restype = ctypes.c_double
            getattr(lib, name).argtypes = [ctypes.c_double] * 8
        _libs[variant] = lib
    return _libs[variant]


def _ptr(a):
    return a.ctypes.data_as(_dp)


class RefSolver:
    """One reference solver state (param_t + fluid_t + suspensions_t) on the host."""

    def __init__(self, itot, jtot, ly, Re, Fr=np.finfo(np.float64).max, extfrcy=0.0,
                 safefactors=(0.75, 0.75, 0.95), variant="default"):
        self.lib = _lib(variant)
        self.itot, self.jtot = itot, jtot
        self.ctx = self.lib.ref_create(itot, jtot, ly, Re, Fr, extfrcy, *safefactors)
        self.n_particles = 0

    def close(self):
        if self.ctx:
            self.lib.ref_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        self.close()

    # ---- state ----
    def shapes(self):
        return (self.jtot + 2, self.itot + 1), (self.jtot + 2, self.itot + 2)

    def set_fluid(self, ux, uy, p):
        ux = np.ascontiguousarray(ux, dtype=np.float64)
        uy = np.ascontiguousarray(uy, dtype=np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64)
        sx, sy = self.shapes()
        assert ux.shape == sx and uy.shape == sy and p.shape == sy
        self.lib.ref_set_fluid(self.ctx, _ptr(ux), _ptr(uy), _ptr(p))

    def get_fluid(self):
        sx, sy = self.shapes()
        ux, uy, p, psi = np.empty(sx), np.empty(sy), np.empty(sy), np.empty(sy)
        self.lib.ref_get_fluid(self.ctx, _ptr(ux), _ptr(uy), _ptr(p), _ptr(psi))
        return ux, uy, p, psi

    def get_src(self):
        nx = (self.jtot, self.itot - 1)
        ny = (self.jtot, self.itot)
        arrs = [np.empty(nx) for _ in range(3)] + [np.empty(ny) for _ in range(3)]
        self.lib.ref_get_src(self.ctx, *[_ptr(a) for a in arrs])
        return arrs

    def set_src(self, uxa, uya):
        uxa = np.ascontiguousarray(uxa, dtype=np.float64)
        uya = np.ascontiguousarray(uya, dtype=np.float64)
        self.lib.ref_set_src(self.ctx, _ptr(uxa), _ptr(uya))

    def get_ibm_fields(self):
        _, sy = self.shapes()
        dux, duy = np.empty(sy), np.empty(sy)
        self.lib.ref_get_ibm_fields(self.ctx, _ptr(dux), _ptr(duy))
        return dux, duy

    def set_particles(self, records):
        records = np.ascontiguousarray(records, dtype=np.float64).reshape(-1, NFIELDS)
        self.n_particles = records.shape[0]
        rc = self.lib.ref_set_particles(self.ctx, self.n_particles, _ptr(records))
        assert rc == 0, "particle_t is not 30 packed doubles"

    def get_particles(self):
        out = np.zeros((max(self.n_particles, 1), NFIELDS))
        self.lib.ref_get_particles(self.ctx, _ptr(out))
        return out[: self.n_particles]

    def grid(self):
        it, jt = self.itot, self.jtot
        arrs = [np.empty(it + 1), np.empty(it + 2), np.empty(it), np.empty(it + 1), np.empty(jt + 1), np.empty(jt)]
        self.lib.ref_get_grid(self.ctx, *[_ptr(a) for a in arrs])
        return dict(zip(("xf", "xc", "dxf", "dxc", "yf", "yc"), arrs))

    @property
    def dt(self):
        return self.lib.ref_get_dt(self.ctx)

    @dt.setter
    def dt(self, v):
        self.lib.ref_set_dt(self.ctx, v)

    @property
    def time(self):
        return self.lib.ref_get_time(self.ctx)

    # ---- stepping ----
    def decide_dt(self):
        return self.lib.ref_decide_dt(self.ctx)

    def integrate(self):
        self.lib.ref_integrate(self.ctx)

    def integrate_counted(self):
        sub = (ctypes.c_int * 3)()
        self.lib.ref_integrate_counted(self.ctx, sub)
        return list(sub)

    def step(self, count_substeps=True):
        sub = (ctypes.c_int * 3)()
        self.lib.ref_step(self.ctx, 1 if count_substeps else 0, sub)
        return list(sub)

    def __getattr__(self, name):
        # stage functions: ref_<name>(ctx[, arg])
        fn = getattr(_lib_for(self), "ref_" + name)
        return lambda *args: fn(self.ctx, *args)


def _lib_for(solver):
    return solver.__dict__["lib"]


def find_normal_t(a, b, x, y, variant="default"):
    return _lib(variant).ref_find_normal_t(a, b, x, y)


def s_weight(h, a, b, px, py, paz, x, y, variant="default"):
    return _lib(variant).ref_s_weight(h, a, b, px, py, paz, x, y)


def v_weight(h, a, b, px, py, paz, x, y, variant="default"):
    return _lib(variant).ref_v_weight(h, a, b, px, py, paz, x, y)
