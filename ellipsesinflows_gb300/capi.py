"""ctypes binding of the C ABI declared in include/eif.h.

``Solver`` wraps one context. The same class binds any library that exports the
eif.h entry points under a given symbol prefix; the product library uses the
prefix ``eif_``.

Array conventions follow the reference solver (include/arrays/fluid.h):
``ux`` has shape (jtot+2, itot+1) and ``uy``, ``p``, ``psi`` have shape
(jtot+2, itot+2), each row-major with x contiguous; row 0 and row jtot+1 are
the periodic halo rows. Particle records have EIF_NFIELDS = 30 doubles in the
order of the reference's ``particle_t`` (include/suspensions.h:8-31).
"""
import ctypes

import numpy as np

NFIELDS = 30
PREC_FP64 = 0
PREC_MIXED = 1

ERRORS = {
    -1: "invalid argument",
    -2: "CUDA error",
    -3: "iteration cap reached",
    -4: "out of memory",
    -5: "call out of order",
    -6: "non-finite velocity",
    -7: "size beyond the fixed scratch",
}

# particle record fields (include/eif.h enum eif_particle_field)
FIELDS = ("den a b x y az dx dy daz ux uy vz dux duy dvz fux fuy tvz "
          "iux0 iux1 iuy0 iuy1 ivz0 ivz1 cfx0 cfx1 cfy0 cfy1 ctz0 ctz1").split()
F = {name: k for k, name in enumerate(FIELDS)}


class EifError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


class Config(ctypes.Structure):
    """eif_config_t (include/eif.h)."""

    _fields_ = [
        ("itot", ctypes.c_int),
        ("jtot", ctypes.c_int),
        ("ly", ctypes.c_double),
        ("Re", ctypes.c_double),
        ("Fr", ctypes.c_double),
        ("extfrcy", ctypes.c_double),
        ("safefactors", ctypes.c_double * 3),
        ("uy_wall", ctypes.c_double * 2),
        ("precision", ctypes.c_int),
        ("device", ctypes.c_int),
    ]


def make_config(itot, jtot, ly=1.0, Re=2334.0, Fr=np.finfo(np.float64).max, extfrcy=0.0,
                safefactors=(0.75, 0.75, 0.95), uy_wall=(0.0, 0.0), precision=PREC_FP64, device=0):
    cfg = Config()
    cfg.itot, cfg.jtot, cfg.ly = itot, jtot, ly
    cfg.Re, cfg.Fr, cfg.extfrcy = Re, Fr, extfrcy
    for k in range(3):
        cfg.safefactors[k] = safefactors[k]
    cfg.uy_wall[0], cfg.uy_wall[1] = uy_wall
    cfg.precision = precision
    cfg.device = device
    return cfg


ADJOINT_COUPLED, ADJOINT_FROZEN = 0, 1   # eif_adjoint_begin modes

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p


def bind(lib, prefix):
    """Declare argument types of every eif.h entry point present in ``lib``."""
    sigs = {
        "create": [ctypes.POINTER(Config), ctypes.POINTER(_vp)],
        "destroy": [_vp],
        "synchronize": [_vp],
        "push_fluid": [_vp, _dp, _dp, _dp],
        "pull_fluid": [_vp, _dp, _dp, _dp, _dp],
        "push_particles": [_vp, ctypes.c_int, _dp],
        "pull_particles": [_vp, ctypes.c_int, _dp],
        "pull_src": [_vp, _dp, _dp, _dp, _dp],
        "push_src": [_vp, _dp, _dp],
        "pull_ibm_fields": [_vp, _dp, _dp],
        "decide_dt": [_vp, _dp],
        "set_dt": [_vp, ctypes.c_double],
        "get_dt": [_vp, _dp],
        "integrate": [_vp, _ip],
        "advance": [_vp, ctypes.c_int],
        "advance_pull": [_vp, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _dp],
        "get_time": [_vp, _ip, _dp],
        "set_time": [_vp, ctypes.c_int, ctypes.c_double],
        "update_boundaries": [_vp],
        "reset_particle_increments": [_vp],
        "compute_inertia": [_vp, ctypes.c_int],
        "update_velocity": [_vp, ctypes.c_int],
        "exchange_momentum": [_vp],
        "update_momentum_field": [_vp],
        "compute_potential": [_vp, ctypes.c_int],
        "correct_velocity": [_vp, ctypes.c_int],
        "update_pressure": [_vp],
        "compute_collision_force": [_vp, ctypes.c_int],
        "increment_particles": [_vp, ctypes.c_int, _dp],
        "update_particles": [_vp],
        "divergence": [_vp, _dp, _dp],
        "momentum": [_vp, _dp],
        "energy": [_vp, _dp],
        "log_quantities": [_vp, _dp],
        "set_threads": [_vp, ctypes.c_int],
        "tiles": [_vp, _ip],
        "counters": [_vp, ctypes.POINTER(ctypes.c_longlong)],
        "memo_count": [_vp, ctypes.POINTER(ctypes.c_longlong)],
        "stats_reset": [_vp],
        "stats_collect": [_vp],
        "stats_pull": [_vp, _dp, _dp, _dp, _dp, _dp, _ip],
        "snapshot_take": [_vp],
        "snapshot_wait": [_vp, _dp, _dp, _dp, ctypes.c_int, _dp, _ip, _dp],
        "adjoint_begin": [_vp, ctypes.c_int, ctypes.c_int],
        "adjoint_seed_particles": [_vp, ctypes.c_int, _dp],
        "adjoint_pull_particles": [_vp, ctypes.c_int, _dp],
        "adjoint_wall_gradient": [_vp, _dp],
        "adjoint_substeps": [_vp, ctypes.c_int, _ip],
        "adjoint_forward": [_vp, ctypes.c_int],
        "adjoint_seed": [_vp, _dp, _dp, _dp],
        "adjoint_backward": [_vp],
        "adjoint_pull": [_vp, _dp, _dp, _dp],
        "adjoint_recorded": [_vp],
        "adjoint_end": [_vp],
    }
    for name, args in sigs.items():
        fn = getattr(lib, prefix + name, None)
        if fn is not None:
            fn.argtypes = args
            fn.restype = ctypes.c_int
    bsigs = {
        "batch_create": [ctypes.POINTER(_vp), ctypes.c_int, ctypes.POINTER(_vp)],
        "batch_advance": [_vp, ctypes.c_int],
        "batch_size": [_vp],
        "batch_destroy": [_vp],
    }
    for name, args in bsigs.items():
        fn = getattr(lib, prefix + name, None)
        if fn is not None:
            fn.argtypes = args
            fn.restype = ctypes.c_int
    bst = getattr(lib, prefix + "batch_stream", None)
    if bst is not None:
        bst.argtypes = [_vp]
        bst.restype = _vp
    ble = getattr(lib, prefix + "batch_last_error", None)
    if ble is not None:
        ble.argtypes = [_vp]
        ble.restype = ctypes.c_char_p
    le = getattr(lib, prefix + "last_error")
    le.argtypes = [_vp]
    le.restype = ctypes.c_char_p
    st = getattr(lib, prefix + "stream", None)
    if st is not None:
        st.argtypes = [_vp]
        st.restype = _vp
    return lib


def _ptr(a):
    return a.ctypes.data_as(_dp)


class Solver:
    """One solver context behind the eif.h C ABI."""

    def __init__(self, lib, prefix, cfg):
        self.lib, self.prefix, self.cfg = lib, prefix, cfg
        self.itot, self.jtot = cfg.itot, cfg.jtot
        self.n_particles = 0
        self.ctx = _vp()
        self._call("create", ctypes.byref(cfg), ctypes.byref(self.ctx))

    # ---- plumbing ----
    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def _call(self, name, *args):
        rc = self._fn(name)(*args)
        if rc != 0:
            msg = self._fn("last_error")(self.ctx) if self.ctx else b""
            raise EifError(rc, (msg or b"").decode(errors="replace"))
        return rc

    def close(self):
        if getattr(self, "ctx", None):
            self._fn("destroy")(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- shapes ----
    def shapes(self):
        return (self.jtot + 2, self.itot + 1), (self.jtot + 2, self.itot + 2)

    # ---- state transfer ----
    def push_fluid(self, ux, uy, p):
        sx, sy = self.shapes()
        ux = np.ascontiguousarray(ux, dtype=np.float64)
        uy = np.ascontiguousarray(uy, dtype=np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64)
        if ux.shape != sx or uy.shape != sy or p.shape != sy:
            raise ValueError("field shapes must be %s and %s" % (sx, sy))
        self._call("push_fluid", self.ctx, _ptr(ux), _ptr(uy), _ptr(p))

    def pull_fluid(self, out=None):
        """ux, uy, p, psi as haloed arrays; with out=(ux, uy, p, psi) (C-contiguous float64
        arrays of the right shapes, e.g. in pinned host memory) they are filled in place,
        and a None entry is skipped (not transferred)."""
        sx, sy = self.shapes()
        if out is None:
            out = (np.empty(sx), np.empty(sy), np.empty(sy), np.empty(sy))
        for a, shape in zip(out, (sx, sy, sy, sy)):
            if a is None:
                continue
            if a.shape != shape or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("output arrays must be C-contiguous float64 of shapes %s, %s" % (sx, sy))
        ux, uy, p, psi = out
        self._call("pull_fluid", self.ctx, *[None if a is None else _ptr(a) for a in (ux, uy, p, psi)])
        return ux, uy, p, psi

    def push_particles(self, records):
        records = np.ascontiguousarray(records, dtype=np.float64).reshape(-1, NFIELDS)
        self.n_particles = records.shape[0]
        buf = records if records.size else np.zeros(NFIELDS)
        self._call("push_particles", self.ctx, self.n_particles, _ptr(buf))

    def pull_particles(self, out=None):
        """(n, NFIELDS) particle records; with out (a C-contiguous float64 array of that
        shape) they are written in place."""
        if out is not None and self.n_particles > 0:
            if out.shape != (self.n_particles, NFIELDS) or out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"]:
                raise ValueError("output array must be C-contiguous float64 of shape (%d, %d)"
                                 % (self.n_particles, NFIELDS))
            self._call("pull_particles", self.ctx, self.n_particles, _ptr(out))
            return out
        out = np.zeros((max(self.n_particles, 1), NFIELDS))
        self._call("pull_particles", self.ctx, self.n_particles, _ptr(out))
        return out[: self.n_particles]

    def pull_src(self):
        nx = (self.jtot, self.itot - 1)
        ny = (self.jtot, self.itot)
        arrs = [np.empty(nx), np.empty(nx), np.empty(ny), np.empty(ny)]
        self._call("pull_src", self.ctx, *[_ptr(a) for a in arrs])
        return arrs

    def push_src(self, uxa, uya):
        uxa = np.ascontiguousarray(uxa, dtype=np.float64)
        uya = np.ascontiguousarray(uya, dtype=np.float64)
        self._call("push_src", self.ctx, _ptr(uxa), _ptr(uya))

    def pull_ibm_fields(self):
        _, sy = self.shapes()
        dux, duy = np.empty(sy), np.empty(sy)
        self._call("pull_ibm_fields", self.ctx, _ptr(dux), _ptr(duy))
        return dux, duy

    # ---- stepping ----
    def decide_dt(self):
        v = ctypes.c_double()
        self._call("decide_dt", self.ctx, ctypes.byref(v))
        return v.value

    @property
    def dt(self):
        v = ctypes.c_double()
        self._call("get_dt", self.ctx, ctypes.byref(v))
        return v.value

    @dt.setter
    def dt(self, value):
        self._call("set_dt", self.ctx, float(value))

    def integrate(self):
        sub = (ctypes.c_int * 3)()
        self._call("integrate", self.ctx, sub)
        return list(sub)

    def step(self):
        """decide_dt + integrate + counters, returning the sub-iteration counts."""
        self.decide_dt()
        sub = self.integrate()
        step, time = self.time_state()
        self._call("set_time", self.ctx, step + 1, time + self.dt)
        return sub

    def advance(self, nsteps):
        self._call("advance", self.ctx, int(nsteps))

    def advance_pull(self, nsteps, fluid, records=None):
        """advance(nsteps), then the fields into fluid = (ux, uy, p) (C-contiguous float64
        arrays of the haloed shapes, None entries skipped) and the particle records into
        records ((n, NFIELDS) or None), filled in place (eif_advance_pull: the fields'
        copy runs beside the last stage's particle work)."""
        sx, sy = self.shapes()
        for a, shape in zip(fluid, (sx, sy, sy)):
            if a is not None and (a.shape != shape or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]):
                raise ValueError("output arrays must be C-contiguous float64 of shapes %s, %s" % (sx, sy))
        n = 0
        if records is not None:
            if records.shape != (self.n_particles, NFIELDS) or records.dtype != np.float64 or \
                    not records.flags["C_CONTIGUOUS"]:
                raise ValueError("records must be C-contiguous float64 of shape (%d, %d)" % (self.n_particles, NFIELDS))
            n = self.n_particles
        rec = _ptr(records) if records is not None and n > 0 else None
        self._call("advance_pull", self.ctx, int(nsteps), *[None if a is None else _ptr(a) for a in fluid], n, rec)

    def time_state(self):
        s, t = ctypes.c_int(), ctypes.c_double()
        self._call("get_time", self.ctx, ctypes.byref(s), ctypes.byref(t))
        return s.value, t.value

    def set_time(self, step, time):
        self._call("set_time", self.ctx, int(step), float(time))

    def synchronize(self):
        fn = getattr(self.lib, self.prefix + "synchronize", None)
        if fn is not None:
            self._call("synchronize", self.ctx)

    def set_threads(self, n):
        self._call("set_threads", self.ctx, int(n))

    def divergence(self):
        mx, sm = ctypes.c_double(), ctypes.c_double()
        self._call("divergence", self.ctx, ctypes.byref(mx), ctypes.byref(sm))
        return mx.value, sm.value

    def momentum(self):
        m = (ctypes.c_double * 2)()
        self._call("momentum", self.ctx, m)
        return m[0], m[1]

    def energy(self):
        e = (ctypes.c_double * 2)()
        self._call("energy", self.ctx, e)
        return e[0], e[1]

    def log_quantities(self):
        """{divmax, divsum, momentum (x, y), energy (x, y)} in one call"""
        q = (ctypes.c_double * 6)()
        self._call("log_quantities", self.ctx, q)
        return {"divmax": q[0], "divsum": q[1], "momentum": (q[2], q[3]), "energy": (q[4], q[5])}

    # ---- stage-level entry points ----
    def update_boundaries(self):
        self._call("update_boundaries", self.ctx)

    def reset_particle_increments(self):
        self._call("reset_particle_increments", self.ctx)

    def compute_inertia(self, cnstep):
        self._call("compute_inertia", self.ctx, int(cnstep))

    def update_velocity(self, rkstep):
        self._call("update_velocity", self.ctx, int(rkstep))

    def exchange_momentum(self):
        self._call("exchange_momentum", self.ctx)

    def update_momentum_field(self):
        self._call("update_momentum_field", self.ctx)

    def compute_potential(self, rkstep):
        self._call("compute_potential", self.ctx, int(rkstep))

    def correct_velocity(self, rkstep):
        self._call("correct_velocity", self.ctx, int(rkstep))

    def update_pressure(self):
        self._call("update_pressure", self.ctx)

    def compute_collision_force(self, cnstep):
        self._call("compute_collision_force", self.ctx, int(cnstep))

    def increment_particles(self, rkstep):
        r = ctypes.c_double()
        self._call("increment_particles", self.ctx, int(rkstep), ctypes.byref(r))
        return r.value

    def update_particles(self):
        self._call("update_particles", self.ctx)

    def stats_reset(self):
        self._call("stats_reset", self.ctx)

    def stats_collect(self):
        self._call("stats_collect", self.ctx)

    def stats_pull(self):
        """(ux1, ux2, uy1, uy2, phi, num): the accumulated sums (eif_stats_pull)"""
        sx, sy = self.shapes()
        arrs = [np.zeros(sx), np.zeros(sx), np.zeros(sy), np.zeros(sy), np.zeros(sy)]
        num = ctypes.c_int()
        self._call("stats_pull", self.ctx, *[_ptr(a) for a in arrs], ctypes.byref(num))
        return tuple(arrs) + (num.value,)

    def snapshot_take(self):
        """start an asynchronous copy of the state (eif_snapshot_take)"""
        self._call("snapshot_take", self.ctx)
        self._snap_n = self.n_particles

    def snapshot_wait(self):
        """(ux, uy, p, records, step, time) of the last snapshot (eif_snapshot_wait)"""
        sx, sy = self.shapes()
        ux, uy, p = np.empty(sx), np.empty(sy), np.empty(sy)
        n = getattr(self, "_snap_n", self.n_particles)
        rec = np.zeros((max(n, 1), NFIELDS))
        step, time = ctypes.c_int(), ctypes.c_double()
        self._call("snapshot_wait", self.ctx, _ptr(ux), _ptr(uy), _ptr(p), n, _ptr(rec), ctypes.byref(step),
                   ctypes.byref(time))
        return ux, uy, p, rec[:n], step.value, time.value

    def counters(self):
        """{"substeps", "indicator_cells", "normal_foot_evals"} (eif_counters)"""
        v = (ctypes.c_longlong * 3)()
        self._call("counters", self.ctx, v)
        return {"substeps": v[0], "indicator_cells": v[1], "normal_foot_evals": v[2]}

    def memo_count(self):
        """indicator tasks whose weights were taken from the last sub-iteration loop's
        evaluation (eif_memo_count; counted while kernel timing is enabled)"""
        v = ctypes.c_longlong()
        self._call("memo_count", self.ctx, ctypes.byref(v))
        return v.value

    def tiles(self):
        """tile shapes chosen by the tuner: {"predictor_rows", "projection_rows",
        "thomas_threads", "tuned", "predictor_tensor_copies", "predictor_uniform_x"}"""
        t = (ctypes.c_int * 4)()
        self._call("tiles", self.ctx, t)
        return {"predictor_rows": t[0], "projection_rows": t[1], "thomas_threads": t[2], "tuned": bool(t[3] & 1),
                "predictor_tensor_copies": bool(t[3] & 2), "predictor_uniform_x": bool(t[3] & 4)}

    # ---- discrete adjoint (double-precision form) ----
    def adjoint_begin(self, max_steps, mode=ADJOINT_COUPLED):
        self._call("adjoint_begin", self.ctx, int(max_steps), int(mode))

    def adjoint_forward(self, record=True):
        self._call("adjoint_forward", self.ctx, 1 if record else 0)

    def adjoint_seed(self, ux_bar, uy_bar, p_bar=None):
        sx, sy = self.shapes()
        ux_bar = np.ascontiguousarray(ux_bar, dtype=np.float64)
        uy_bar = np.ascontiguousarray(uy_bar, dtype=np.float64)
        if ux_bar.shape != sx or uy_bar.shape != sy:
            raise ValueError("cotangent shapes must be %s and %s" % (sx, sy))
        pb = None
        if p_bar is not None:
            p_bar = np.ascontiguousarray(p_bar, dtype=np.float64)
            if p_bar.shape != sy:
                raise ValueError("pressure cotangent shape must be %s" % (sy,))
            pb = _ptr(p_bar)
        self._call("adjoint_seed", self.ctx, _ptr(ux_bar), _ptr(uy_bar), pb)

    def adjoint_backward(self):
        self._call("adjoint_backward", self.ctx)

    def adjoint_pull(self):
        sx, sy = self.shapes()
        ub, vb, pb = np.zeros(sx), np.zeros(sy), np.zeros(sy)
        self._call("adjoint_pull", self.ctx, _ptr(ub), _ptr(vb), _ptr(pb))
        return ub, vb, pb

    def adjoint_seed_particles(self, records_bar):
        rb = np.ascontiguousarray(records_bar, dtype=np.float64).reshape(-1, NFIELDS)
        if rb.shape[0] != self.n_particles:
            raise ValueError("expected %d particle records" % self.n_particles)
        buf = rb if rb.size else np.zeros(NFIELDS)
        self._call("adjoint_seed_particles", self.ctx, self.n_particles, _ptr(buf))

    def adjoint_pull_particles(self):
        out = np.zeros((max(self.n_particles, 1), NFIELDS))
        self._call("adjoint_pull_particles", self.ctx, self.n_particles, _ptr(out))
        return out[: self.n_particles]

    def adjoint_wall_gradient(self):
        g = np.zeros(2)
        self._call("adjoint_wall_gradient", self.ctx, _ptr(g))
        return g

    def adjoint_substeps(self, step):
        k = (ctypes.c_int * 3)()
        self._call("adjoint_substeps", self.ctx, int(step), k)
        return list(k)

    def adjoint_recorded(self):
        return self._fn("adjoint_recorded")(self.ctx)

    def adjoint_end(self):
        self._call("adjoint_end", self.ctx)


class Batch:
    """Several suspensions (Solver objects on one device) advanced together, one CUDA
    graph launch per step (eif_batch_* in include/eif.h). The solvers stay usable on
    their own; close the batch before them."""

    def __init__(self, solvers):
        if not solvers:
            raise ValueError("a batch needs at least one suspension")
        self.solvers = list(solvers)
        self.lib, self.prefix = self.solvers[0].lib, self.solvers[0].prefix
        arr = (_vp * len(self.solvers))(*[s.ctx for s in self.solvers])
        self.handle = _vp()
        rc = getattr(self.lib, self.prefix + "batch_create")(arr, len(self.solvers), ctypes.byref(self.handle))
        if rc != 0:
            raise EifError(rc, "batch_create")

    def advance(self, nsteps=1):
        rc = getattr(self.lib, self.prefix + "batch_advance")(self.handle, nsteps)
        if rc != 0:
            msg = getattr(self.lib, self.prefix + "batch_last_error")(self.handle) or b""
            raise EifError(rc, msg.decode(errors="replace"))

    def cells(self):
        return sum(s.itot * s.jtot for s in self.solvers)

    def stream(self):
        """The cudaStream_t (as an integer) the batch's step graphs run on."""
        return getattr(self.lib, self.prefix + "batch_stream")(self.handle)

    def close(self):
        if getattr(self, "handle", None):
            getattr(self.lib, self.prefix + "batch_destroy")(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
