"""Checkpoint and restart in the reference's format (src/save.c:13-122,
src/fileio.c:130-365; read back by src/param/init.c:215-235, src/fluid/init.c:33-85,
src/suspensions/init.c:27-36).

``save(sim, root)`` writes ``root/step%010d/`` with the same .npy files, byte for byte,
as the reference's save(): step, itot, jtot (int32), time, lx, ly, Re (float64), the
grid xf, xc, yf, yc, the fields ux (jtot, itot+1), uy and p (jtot, itot+2) without
the y halo rows, n_particles and the particle den, a, b, x, y, az, ux, uy, vz.
``AsyncSave`` takes the state with eif_snapshot_take and writes the files after the
steps that follow (the device->host copy overlaps with them). ``load(sim, dirname)``
pushes a saved state (the reference's restart: the RK source term is not saved and
not needed, beta_0 = 0) and sets step and time; a run continued from it gives the
same bits as one that did not stop.
"""
import os

import numpy as np

from .capi import F, NFIELDS

_PARTICLE_FILES = (("dens", "den"), ("as", "a"), ("bs", "b"), ("xs", "x"), ("ys", "y"), ("azs", "az"),
                   ("uxs", "ux"), ("uys", "uy"), ("vzs", "vz"))


def write_npy(path, data, descr):
    """.npy file with the header layout of the reference's writer (simple_npyio): no
    spaces in the dictionary, a trailing comma after every dimension, padded with
    spaces and a newline to a multiple of 64 bytes"""
    a = np.array(data, dtype={"int32": "<i4", "float64": "<f8"}[descr], order="C")   # keeps 0-d shapes
    shape = "(" + "".join("%d," % d for d in a.shape) + ")"
    head = "{'descr':'%s','fortran_order':False,'shape':%s}" % (descr, shape)
    total = 10 + len(head) + 1
    head += " " * ((-total) % 64) + "\n"
    with open(path, "wb") as f:
        f.write(b"\x93NUMPY\x01\x00" + len(head).to_bytes(2, "little") + head.encode("latin1"))
        f.write(a.tobytes())


def grid(itot, jtot, ly):
    """xf (itot+1), xc (itot+2) of set_coordinate (src/param/init.c:119-144, LX = 1) and
    yf (jtot+1), yc (jtot) as save_param computes them (src/save.c:29-36)"""
    dx = 1.0 / itot
    xf = np.array([1.0 * (i - 1) * dx for i in range(1, itot + 2)])
    xf[0], xf[itot] = 0.0, 1.0
    xc = np.empty(itot + 2)
    xc[0] = xf[0]
    xc[1:itot + 1] = 0.5 * (xf[:itot] + xf[1:itot + 1])
    xc[itot + 1] = xf[itot]
    dy = ly / jtot
    yf = np.array([1.0 * j * dy for j in range(jtot + 1)])
    yc = 0.5 * (yf[:jtot] + yf[1:])
    return xf, xc, yf, yc


def write_state(root, cfg, ux, uy, p, records, step, time):
    """the files of save() for a state given as host arrays (haloed layouts)"""
    d = os.path.join(root, "step%010d" % step)
    os.makedirs(d, exist_ok=True)
    itot, jtot, ly = cfg.itot, cfg.jtot, cfg.ly

    def w(name, data, descr):
        write_npy(os.path.join(d, name + ".npy"), data, descr)

    w("step", np.int32(step), "int32")
    w("itot", np.int32(itot), "int32")
    w("jtot", np.int32(jtot), "int32")
    w("time", np.float64(time), "float64")
    w("lx", np.float64(1.0), "float64")
    w("ly", np.float64(ly), "float64")
    w("Re", np.float64(cfg.Re), "float64")
    xf, xc, yf, yc = grid(itot, jtot, ly)
    w("xf", xf, "float64")
    w("xc", xc, "float64")
    w("yf", yf, "float64")
    w("yc", yc, "float64")
    w("ux", ux[1:jtot + 1], "float64")
    w("uy", uy[1:jtot + 1], "float64")
    w("p", p[1:jtot + 1], "float64")
    rec = np.asarray(records).reshape(-1, NFIELDS)
    w("n_particles", np.int32(rec.shape[0]), "int32")
    for fname, field in _PARTICLE_FILES:
        w("particle_" + fname, rec[:, F[field]], "float64")
    return d


def save(sim, root=os.path.join("output", "save")):
    """write the current state (synchronous); returns the directory"""
    step, time = sim.time_state()
    ux, uy, p, _ = sim.pull_fluid()
    return write_state(root, sim.cfg, ux, uy, p, sim.pull_particles(), step, time)


class AsyncSave:
    """take the state now, write it later: the transfer overlaps with the steps between"""

    def __init__(self, sim, root=os.path.join("output", "save")):
        self.sim, self.root = sim, root
        sim.snapshot_take()

    def finish(self):
        ux, uy, p, rec, step, time = self.sim.snapshot_wait()
        return write_state(self.root, self.sim.cfg, ux, uy, p, rec, step, time)


def read_state(dirname):
    """(ux, uy, p, records, step, time) from a saved directory, fields with halo rows"""

    def r(name):
        return np.load(os.path.join(dirname, name + ".npy"))

    itot, jtot = int(r("itot")), int(r("jtot"))
    ux = np.zeros((jtot + 2, itot + 1))
    uy = np.zeros((jtot + 2, itot + 2))
    p = np.zeros((jtot + 2, itot + 2))
    ux[1:jtot + 1], uy[1:jtot + 1], p[1:jtot + 1] = r("ux"), r("uy"), r("p")
    n = int(r("n_particles"))
    rec = np.zeros((n, NFIELDS))
    for fname, field in _PARTICLE_FILES:
        rec[:, F[field]] = r("particle_" + fname)
    return ux, uy, p, rec, int(r("step")), float(r("time"))


def load(sim, dirname):
    """push a saved state into ``sim`` (whose configuration must match) and set its step
    and time; returns (step, time)"""
    ux, uy, p, rec, step, time = read_state(dirname)
    if ux.shape != sim.shapes()[0]:
        raise ValueError("saved grid %s does not match the solver's %s" % (ux.shape, sim.shapes()[0]))
    sim.push_fluid(ux, uy, p)
    sim.push_particles(rec)
    sim.set_time(step, time)
    return step, time
