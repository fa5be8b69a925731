"""Restatement of statistics_collect (src/statistics/collect.c:10-95), for tests.

TEST INFRASTRUCTURE ONLY. Accumulates into arrays of the reference's layouts
(include/arrays/statistics.h) from the haloed host fields and the particle
records, in the reference's loop order, with the C library's cos, sin and pow
(Python's math module) for the sharp indicator. Pinned against the reference's
own statistics_output files by tests/test_statistics_oracle.py.
"""
import math

import numpy as np

from ellipsesinflows_gb300.capi import F


class Accumulator:
    def __init__(self, itot, jtot, ly):
        self.itot, self.jtot, self.ly = itot, jtot, ly
        self.ux1 = np.zeros((jtot + 2, itot + 1))
        self.ux2 = np.zeros((jtot + 2, itot + 1))
        self.uy1 = np.zeros((jtot + 2, itot + 2))
        self.uy2 = np.zeros((jtot + 2, itot + 2))
        self.phi = np.zeros((jtot + 2, itot + 2))
        self.num = 0
        dx, dy = 1.0 / itot, ly / jtot
        xf = [1.0 * (i - 1) * dx for i in range(1, itot + 2)]
        xf[0], xf[itot] = 0.0, 1.0
        self.xc = [xf[0]] + [0.5 * (xf[i - 1] + xf[i]) for i in range(1, itot + 1)] + [xf[itot]]
        yf = [1.0 * j * dy for j in range(jtot + 1)]
        self.yc = [0.0] + [0.5 * (yf[j - 1] + yf[j]) for j in range(1, jtot + 1)]   # YC(j) at [j]

    def collect(self, ux, uy, records):
        it, jt = self.itot, self.jtot
        # collect.c:20-25 (i = 1..itot+1) and :37-42 (i = 0..itot+1), rows 1..jtot
        self.ux1[1:jt + 1] += ux[1:jt + 1]
        self.ux2[1:jt + 1] += ux[1:jt + 1] * ux[1:jt + 1]
        self.uy1[1:jt + 1] += uy[1:jt + 1]
        self.uy2[1:jt + 1] += uy[1:jt + 1] * uy[1:jt + 1]
        # collect.c:57-81: every cell against every particle image
        for r in np.asarray(records).reshape(-1, len(F)):
            pa, pb, px, py, paz = r[F["a"]], r[F["b"]], r[F["x"]], r[F["y"]], r[F["az"]]
            c, s = math.cos(-paz), math.sin(-paz)
            for periodic in (-1, 0, 1):
                py_ = py + self.ly * periodic
                for j in range(1, jt + 1):
                    y = self.yc[j]
                    for i in range(1, it + 1):
                        dx, dy = self.xc[i] - px, y - py_
                        x_, y_ = c * dx - s * dy, s * dx + c * dy
                        if 1.0 - math.pow(x_ / pa, 2.0) - math.pow(y_ / pb, 2.0) > 0.0:
                            self.phi[j, i] += 1.0
        self.num += 1
