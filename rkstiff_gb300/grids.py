"""Grid builders used to set up problems (the same grids as rkstiff/grids.py:40-219).

By default they return NumPy arrays, as the reference does.  With ``device=`` (a CUDA
device) the Fourier and Chebyshev grids are computed on the GPU by the library's kernels
(``rk_fourier_grid`` / ``rk_cheb_grid``) and returned as CUDA float64 tensors, so that set-up
need not leave the device; the Fourier grids are then bitwise the NumPy ones.
"""

from __future__ import annotations

from typing import Tuple

import numpy as np


def _device_fourier(n, a, b, real_grid, device):
    import torch

    from . import _native as nat
    from .engine import _dev, stream_handle

    dev = _dev(device)
    dx = (b - a) / n
    x = torch.empty(n, dtype=torch.float64, device=dev)
    kx = torch.empty(n // 2 + 1 if real_grid else n, dtype=torch.float64, device=dev)
    lib = nat.load()
    with torch.cuda.device(dev):
        nat.check(lib.rk_fourier_grid(1 if real_grid else 0, n, float(a), float(dx), x.data_ptr(), kx.data_ptr(),
                                      stream_handle(dev)), "rk_fourier_grid")
    return x, kx


def _device_cheb(n, a, b, with_matrix, device):
    import torch

    from . import _native as nat
    from .engine import _dev, stream_handle

    dev = _dev(device)
    x = torch.empty(n + 1, dtype=torch.float64, device=dev)
    D = torch.empty((n + 1, n + 1), dtype=torch.float64, device=dev) if with_matrix else None
    lib = nat.load()
    with torch.cuda.device(dev):
        nat.check(lib.rk_cheb_grid(n, float(a), float(b), x.data_ptr(), D.data_ptr() if D is not None else None,
                                   stream_handle(dev)), "rk_cheb_grid")
    return x, D


def _check_even(n):
    if not isinstance(n, (int, np.integer)):
        raise TypeError("n must be an integer.")
    if n <= 2 or (n % 2) != 0:
        raise ValueError("n must be an even integer greater than 2.")


def construct_x_kx_rfft(n: int, a: float = 0.0, b: float = 2 * np.pi, device=None):
    """Uniform grid on [a, b) and its real-FFT wavenumbers (length n/2 + 1)."""
    _check_even(n)
    if device is not None:
        return _device_fourier(int(n), a, b, True, device)
    dx = (b - a) / n
    x = np.arange(a, b, dx)
    return x, 2 * np.pi * np.fft.rfftfreq(n, d=dx)


def construct_x_kx_fft(n: int, a: float = 0.0, b: float = 2 * np.pi, device=None):
    """Uniform grid on [a, b) and its complex-FFT wavenumbers (length n)."""
    _check_even(n)
    if device is not None:
        return _device_fourier(int(n), a, b, False, device)
    dx = (b - a) / n
    x = np.arange(a, b, dx)
    return x, 2 * np.pi * np.fft.fftfreq(n, d=dx)


def construct_x_cheb(n: int, a: float = -1.0, b: float = 1.0, device=None):
    """n + 1 Chebyshev extreme points mapped to [a, b]."""
    if not isinstance(n, (int, np.integer)):
        raise TypeError("n must be an integer.")
    if n < 2:
        raise ValueError("n must be >= 2.")
    if device is not None:
        return _device_cheb(int(n), a, b, False, device)[0]
    x = np.polynomial.chebyshev.chebpts2(n + 1)
    return a + (b - a) * (x + 1) / 2.0


def construct_x_dx_cheb(n: int, a: float = -1, b: float = 1, device=None):
    """Chebyshev points and the (n+1) x (n+1) first-derivative matrix: the published
    construction of L. N. Trefethen, Spectral Methods in MATLAB (SIAM, 2000), program
    cheb.m -- off-diagonal entries c_i/c_j (-1)^(i+j) / (x_i - x_j) with c = 2 at the ends,
    the diagonal by the negative-sum trick (each row sums to zero).  The same matrix as the
    reference's construct_x_dx_cheb (rkstiff/grids.py:178-219)."""
    if device is not None:
        if not isinstance(n, (int, np.integer)):
            raise TypeError("n must be an integer.")
        if n < 2:
            raise ValueError("n must be >= 2.")
        return _device_cheb(int(n), a, b, True, device)
    x = construct_x_cheb(n, a, b)
    c = np.r_[2, np.ones(n - 1), 2] * np.power(-1, np.arange(0, n + 1))
    X = np.tile(x.reshape(n + 1, 1), (1, n + 1))
    dX = X - X.T
    D = np.outer(c, 1.0 / c) / (dX + np.eye(n + 1))
    D = D - np.diag(D.sum(axis=1))
    return x, D


def construct_r_kr_hankel(nr: int, rmax: float) -> Tuple[np.ndarray, np.ndarray, np.ndarray, float]:
    """Radial and spectral grids of the quasi-discrete Hankel transform of order zero
    (rkstiff/grids.py:222-264): with j_1 .. j_{nr+1} the first zeros of J0,
    r_i = j_i rmax / j_{nr+1} and kr_i = j_i / rmax.  Returns (r, kr, zeros, j_{nr+1})."""
    from scipy import special

    if nr < 4:
        raise ValueError("nr must be >= 4.")
    if rmax <= 0:
        raise ValueError("rmax must be positive.")
    z = special.jn_zeros(0, nr + 1)
    zeros, jn = z[:-1], float(z[-1])
    return zeros * rmax / jn, zeros / rmax, zeros, jn


def mirror_grid(r: np.ndarray, u=None, axis: int = -1):
    """Reflect a radial grid [0, rmax] (and values on it) to [-rmax, rmax]
    (rkstiff/grids.py:267-321): the grid as -flip(r) followed by r; values flipped along
    ``axis`` (-1: 1-D, 0: rows, 1: columns) and stacked in front."""
    r = np.asarray(r)
    rnew = np.concatenate([-r[::-1], r])
    if u is None:
        return rnew, None
    u = np.asarray(u)
    if axis == -1:  # rows flipped, stacked along the last axis of a 2-D array
        return rnew, np.hstack([u[::-1], u])
    if axis == 0:
        return rnew, np.vstack([u[::-1], u])
    if axis == 1:
        return rnew, np.hstack([u[:, ::-1], u])
    raise ValueError("axis must be -1, 0, or 1.")
