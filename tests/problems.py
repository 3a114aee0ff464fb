"""Problem builders shared by the tests (seeded; same shapes as the golden generator)."""

import numpy as np


def rfft_grid(n, a, b):
    dx = (b - a) / n
    x = np.arange(a, b, dx)
    kx = 2 * np.pi * np.fft.rfftfreq(n, d=dx)
    return x, kx


def fft_grid(n, a, b):
    dx = (b - a) / n
    x = np.arange(a, b, dx)
    kx = 2 * np.pi * np.fft.fftfreq(n, d=dx)
    return x, kx


def uux_nl(kx, c=-1.0):
    """c * rfft(irfft(u) * irfft(i kx u)) -- KS/Burgers (c=-1) and KdV (c=-6)."""
    def nl(u):
        return c * np.fft.rfft(np.fft.irfft(u) * np.fft.irfft(1j * kx * u))
    return nl


def nls_nl(u):
    v = np.fft.ifft(u)
    return np.fft.fft(1j * np.abs(v) ** 2 * v)


def ks(n, L):
    x, kx = rfft_grid(n, 0.0, L)
    return x, kx, kx**2 * (1 - kx**2), uux_nl(kx)


def ks_config1():
    x, kx, lin, nl = ks(1024, 32 * np.pi)
    u0 = np.fft.rfft(np.cos(x / 16) * (1 + np.sin(x / 16)))
    return kx, lin, nl, u0


def ks256_problem(golden):
    g = golden("adaptive")
    L = float(g["ks256_L"])
    x, kx, lin, nl = ks(256, L)
    return kx, lin, nl, g["ks256_u0"]


def kdv_soliton(x, ampl, x0, t):
    return 0.5 * ampl**2 / (np.cosh(ampl * (x - x0 - ampl**2 * t) / 2) ** 2)


def kdv_problem():
    x, kx = rfft_grid(256, -30, 30)
    u0 = np.fft.rfft(kdv_soliton(x, 1.0, -5.0, 0.0))
    lin = 1j * kx**3
    return kx, lin, uux_nl(kx, -6.0), u0


def nls256():
    x, kx = fft_grid(256, -20.0, 20.0)
    return kx, -0.5j * kx**2, nls_nl


def burgers(n, nu):
    x, kx = rfft_grid(n, 0.0, 2 * np.pi)
    return x, kx, -nu * kx**2, uux_nl(kx)


def cheb(n, a=-1.0, b=1.0):
    x = np.polynomial.chebyshev.chebpts2(n + 1)
    x = a + (b - a) * (x + 1) / 2.0
    c = np.r_[2, np.ones(n - 1), 2] * np.power(-1, np.arange(0, n + 1))
    X = np.tile(x.reshape(n + 1, 1), (1, n + 1))
    dX = X - X.T
    D = np.outer(c, 1.0 / c) / (dX + np.eye(n + 1))
    D = D - np.diag(D.sum(axis=1))
    return x, D


def allen_cahn(n, eps=0.01):
    x, D = cheb(n)
    lin = (eps * D.dot(D) + np.eye(n + 1))[1:-1, 1:-1]
    xi = x[1:-1]

    def nl(u):
        return np.asarray(xi - np.power(u + xi, 3), dtype=np.complex128).ravel()
    return x, lin, nl


def nls4096():
    """The NLS soliton configuration's grid and operator: n = 4096 on [-50, 50)."""
    x, kx = fft_grid(4096, -50.0, 50.0)
    return kx, -0.5j * kx**2, nls_nl
