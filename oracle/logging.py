"""Restatement of the reference's logging reductions (src/logging.c), for tests.

TEST INFRASTRUCTURE ONLY. Loops in the reference's order (j outer, i inner, one
accumulator each), on the haloed host arrays of the eif_push_fluid layouts, with
the grid metrics of src/param/init.c:105-167 for the uniform grid (LX = 1).
Pinned against the reference's own logging() output by tests/test_logging_oracle.py.
"""
import numpy as np


def metrics(itot):
    """DXF(1..itot), DXC(1..itot+1) as 1-based arrays (index 0 unused); set_coordinate
    (src/param/init.c:105-167) for the uniform grid with walls at 0 and 1"""
    dx = 1.0 / itot
    xf = np.array([1.0 * (i - 1) * dx for i in range(1, itot + 2)])
    xf[0], xf[itot] = 0.0, 1.0
    xc = np.empty(itot + 2)
    xc[0] = xf[0]
    xc[1:itot + 1] = 0.5 * (xf[:itot] + xf[1:itot + 1])
    xc[itot + 1] = xf[itot]
    dxf = np.zeros(itot + 2)
    dxc = np.zeros(itot + 2)
    for i in range(1, itot + 1):
        dxf[i] = xf[i] - xf[i - 1]          # DXF(i) = XF(i+1) - XF(i)
    for i in range(1, itot + 2):
        dxc[i] = xc[i] - xc[i - 1]          # DXC(i) = XC(i) - XC(i-1)
    return dxf, dxc


def log_quantities(ux, uy, itot, jtot, ly):
    """(divmax, divsum, (mom_x, mom_y), (energy_x, energy_y)): logging.c:40-172"""
    dxf, dxc = metrics(itot)
    dy = ly / jtot
    divmax, divsum = 0.0, 0.0
    for j in range(1, jtot + 1):              # logging.c:52-66
        for i in range(1, itot + 1):
            d = (ux[j, i] - ux[j, i - 1]) / dxf[i] + (uy[j + 1, i] - uy[j, i]) / dy
            divmax = max(divmax, abs(d))
            divsum += d
    mx = my = ex = ey = 0.0
    for j in range(1, jtot + 1):              # logging.c:100-105, 144-149
        for i in range(1, itot + 2):
            cs = dxc[i] * dy
            mx += ux[j, i - 1] * cs
            ex += 0.5 * ux[j, i - 1] ** 2 * cs
    for j in range(1, jtot + 1):              # logging.c:107-112, 151-156
        for i in range(1, itot + 1):
            cs = dxf[i] * dy
            my += uy[j, i] * cs
            ey += 0.5 * uy[j, i] ** 2 * cs
    return divmax, divsum, (mx, my), (ex, ey)
