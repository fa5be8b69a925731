"""Time-averaged statistics (src/statistics/) with the accumulation on the device.

``Statistics(sim)`` resets the device accumulators (eif_stats_reset); ``collect()``
adds the current state (eif_stats_collect, statistics_collect of collect.c:84-95);
``output(root)`` writes ``root/step%010d/`` with the files of the reference's
statistics_output (output.c:8-78), byte for byte: num, step, itot, jtot (int32),
time, lx, ly, Re, xf, xc, yf, yc (float64) and the sums ux1, uy1, ux2, uy2, phi
without the y halo rows.
"""
import os

import numpy as np

from .restart import grid, write_npy


def write_stats(root, cfg, ux1, ux2, uy1, uy2, phi, num, step, time):
    d = os.path.join(root, "step%010d" % step)
    os.makedirs(d, exist_ok=True)
    itot, jtot, ly = cfg.itot, cfg.jtot, cfg.ly

    def w(name, data, descr):
        write_npy(os.path.join(d, name + ".npy"), data, descr)

    w("num", np.int32(num), "int32")
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
    w("ux1", ux1[1:jtot + 1], "float64")
    w("uy1", uy1[1:jtot + 1], "float64")
    w("ux2", ux2[1:jtot + 1], "float64")
    w("uy2", uy2[1:jtot + 1], "float64")
    w("phi", phi[1:jtot + 1], "float64")
    return d


class Statistics:
    def __init__(self, sim):
        self.sim = sim
        sim.stats_reset()

    def collect(self):
        self.sim.stats_collect()

    def output(self, root=os.path.join("output", "stat")):
        ux1, ux2, uy1, uy2, phi, num = self.sim.stats_pull()
        step, time = self.sim.time_state()
        return write_stats(root, self.sim.cfg, ux1, ux2, uy1, uy2, phi, num, step, time)
