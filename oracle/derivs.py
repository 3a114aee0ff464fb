"""NumPy FP64 restatement of rkstiff's grid builders and spectral derivatives (CPU oracle;
test infrastructure only -- the device helpers live in rkstiff_gb300.grids /
rkstiff_gb300.derivatives).

Each function names the reference lines it follows (paths relative to the whalenpt/rkstiff
project root).  Parity pin: ``tests/test_oracle_golden.py`` checks these against vectors
written by the reference itself (``tests/golden/derivs.npz``).
"""

from __future__ import annotations

import numpy as np


def fourier_grid(n: int, a: float, b: float, real_grid: bool):
    """construct_x_kx_rfft / construct_x_kx_fft (rkstiff/grids.py:40-131): x = arange(a, b,
    dx) filled as a + j*((a + dx) - a); kx = 2 pi * (k * (1 / (n dx))) with k the rfftfreq or
    fftfreq integers."""
    dx = (b - a) / n
    delta = (a + dx) - a
    x = a + np.arange(n) * delta
    val = 1.0 / (n * dx)
    if real_grid:
        k = np.arange(0, n // 2 + 1)
    else:
        k = np.concatenate([np.arange(0, (n - 1) // 2 + 1), np.arange(-(n // 2), 0)])
    return x, 2 * np.pi * (k * val)


def cheb_grid(n: int, a: float, b: float):
    """construct_x_dx_cheb (rkstiff/grids.py:134-219): the n + 1 points cos(linspace(-pi, 0))
    mapped to [a, b] and the matrix c_i/c_j / (x_i - x_j) with the negative-sum diagonal
    (Trefethen, Spectral Methods in MATLAB, cheb.m)."""
    t = np.arange(n + 1) * (np.pi / n) - np.pi
    t[-1] = 0.0
    x = a + (b - a) * (np.cos(t) + 1) / 2.0
    c = np.where((np.arange(n + 1) == 0) | (np.arange(n + 1) == n), 2.0, 1.0) * (-1.0) ** np.arange(n + 1)
    D = np.zeros((n + 1, n + 1))
    for i in range(n + 1):
        for j in range(n + 1):
            if i != j:
                D[i, j] = (c[i] / c[j]) / (x[i] - x[j])
        D[i, i] = -(np.sum(D[i]))
    return x, D


def _ikx_pow(kx, order):
    return (1j ** (order % 4)) * kx.astype(np.float64) ** order


def dx_rfft(kx, u, order=1):
    """dx_rfft (rkstiff/derivatives.py:47-124): irfft((i kx)^order rfft(u), n=len(u))."""
    return np.fft.irfft(_ikx_pow(kx, order) * np.fft.rfft(u), n=u.shape[-1])


def dx_fft(kx, u, order=1):
    """dx_fft (rkstiff/derivatives.py:126-180): ifft((i kx)^order fft(u))."""
    return np.fft.ifft(_ikx_pow(kx, order) * np.fft.fft(u))


def dx_cheb(D, u, order=1):
    """dx_cheb (rkstiff/derivatives.py:182-253): D^order u with D^order formed first."""
    P = D
    for _ in range(order - 1):
        P = P @ D
    return P @ u
