"""Cross-check of the Poisson solve against cuFFT (the benchmark spec: cuFFT only as a
cross-check, never on the product path). The double-precision solve of L psi = q
(compute_potential.c:48-138: the divergence of a predicted velocity over gamma dt, the
5-point Laplacian with Neumann walls in x and periodic y) is compared with a spectral
solve on the GPU through torch.fft (cuFFT): the cosine transform in x formed from an FFT
of the even extension, the FFT in y, division by the operator's eigenvalues, and the
inverse transforms. Psi is compared with its mean removed (the constant mode is pinned
differently)."""
import math

import numpy as np
import pytest

from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, cases

pytestmark = pytest.mark.gpu

GAMMA = (45.0 - 25.0) / 60.0   # RK stage 2 (src/param/init.c:177-189)


def dct2(x, dim):
    """DCT-II along dim (sum_n x_n cos(pi k (2n+1) / 2N)) from an FFT of the even extension"""
    import torch
    n = x.shape[dim]
    y = torch.cat([x, torch.flip(x, [dim])], dim=dim)
    Y = torch.fft.fft(y, dim=dim)
    k = torch.arange(n, device=x.device, dtype=torch.float64)
    ph = torch.exp(-1j * math.pi * k / (2 * n))
    shape = [1] * x.dim()
    shape[dim] = n
    return 0.5 * torch.real(Y.narrow(dim, 0, n) * ph.reshape(shape))


def idct2(X, dim):
    """inverse of dct2 (a DCT-III with the 1/N scaling) through an FFT"""
    import torch
    n = X.shape[dim]
    k = torch.arange(n, device=X.device, dtype=torch.float64)
    shape = [1] * X.dim()
    shape[dim] = n
    Z = X.to(torch.complex128) * torch.exp(1j * math.pi * k / (2 * n)).reshape(shape)
    # even extension of the spectrum: Z_{2N-k} = conj(Z_k) with Z_N = 0
    zero = torch.zeros_like(Z.narrow(dim, 0, 1))
    rest = torch.conj(torch.flip(Z.narrow(dim, 1, n - 1), [dim]))
    full = torch.cat([Z, zero, rest], dim=dim)
    y = torch.fft.ifft(full, dim=dim)
    return 2.0 * torch.real(y.narrow(dim, 0, n))


def spectral_solve(q, dx, dy):
    """psi with L psi = q (Neumann x along dim 1, periodic y along dim 0), the (0, 0) mode zero"""
    import torch
    jt, it = q.shape
    Q = torch.fft.fft(dct2(q, 1), dim=0)
    kx = torch.arange(it, device=q.device, dtype=torch.float64)
    ky = torch.arange(jt, device=q.device, dtype=torch.float64)
    lx = -(4.0 / dx**2) * torch.sin(math.pi * kx / (2 * it)) ** 2
    ly = -(4.0 / dy**2) * torch.sin(math.pi * ky / jt) ** 2
    lam = ly[:, None] + lx[None, :]
    lam[0, 0] = 1.0
    P = Q / lam
    P[0, 0] = 0.0
    return idct2(torch.real(torch.fft.ifft(P, dim=0)), 1)


@pytest.mark.parametrize("prec,tol", [(PREC_FP64, 1e-11), (PREC_MIXED, 1e-10)], ids=["fp64", "mixed"])
@pytest.mark.parametrize("itot,jtot", [(128, 256), (512, 1024)])
def test_poisson_solve_matches_cufft(prec, tol, itot, jtot, gpu_lib):
    torch = pytest.importorskip("torch")
    case = cases.poiseuille(itot=itot, jtot=jtot, n=1, a=0.05, b=0.03, seed=7)
    case.particles = case.particles[:0]
    s = Simulation.from_case(case, precision=prec)
    rng = np.random.default_rng(3)
    ux, uy, p = (np.array(a) for a in case.fluid())
    ux[1:-1, 1:-1] = rng.standard_normal(ux[1:-1, 1:-1].shape)   # the walls stay at rest
    uy[1:-1, 1:-1] = rng.standard_normal(uy[1:-1, 1:-1].shape)
    for a in (ux, uy):   # periodic halo rows in y
        a[0], a[-1] = a[-2], a[1]
    s.push_fluid(ux, uy, p)
    dt = 1.0e-3
    s.dt = dt
    s.compute_potential(2)
    psi = s.pull_fluid()[3][1:-1, 1:-1]
    dx, dy = 1.0 / itot, case.ly / jtot
    div = (ux[1:-1, 1:] - ux[1:-1, :-1]) / dx + (uy[2:, 1:-1] - uy[1:-1, 1:-1]) / dy
    q = torch.tensor(div / (GAMMA * dt), dtype=torch.float64, device="cuda")
    ref = spectral_solve(q, dx, dy).cpu().numpy()
    a, b = psi - psi.mean(), ref - ref.mean()
    err = np.abs(a - b).max() / np.abs(b).max()
    print("%dx%d: max |psi - psi_cufft| / max |psi_cufft| = %.3g" % (itot, jtot, err))
    assert err < tol
