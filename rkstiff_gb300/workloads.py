"""Seeded synthetic instance sets: the NLS soliton problem, the viscous Burgers ensemble
and a Kuramoto-Sivashinsky ensemble, as lists of (lin_op, nl_func, u0_hat).

These stand in for real data when the learned step-size controller is trained and
evaluated; the problems follow rkstiff/models.py (burgers_ops, nls_ops) and the KS
operator of the reference's README.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np

from . import grids, models

Instance = Tuple[np.ndarray, models.BuiltinNL, np.ndarray]


def nls_solitons(count: int, seed: int, n: int = 4096) -> List[Instance]:
    """Cubic NLS on [-50, 50) (complex fft grid of n points): u0 = sum of three solitons
    A_j sech(A_j (x - x_j)) exp(i v_j x), A_j ~ U[0.5, 2], x_j ~ U[-30, 30], v_j ~ U[-1, 1]."""
    rng = np.random.default_rng(seed)
    _, kx = grids.construct_x_kx_fft(n, -50.0, 50.0)
    x = -50.0 + np.arange(n) * (100.0 / n)
    lin, nl = models.nls_ops(kx)
    out = []
    for _ in range(count):
        A = rng.uniform(0.5, 2.0, 3)
        x0 = rng.uniform(-30.0, 30.0, 3)
        v = rng.uniform(-1.0, 1.0, 3)
        u = sum(A[j] / np.cosh(A[j] * (x - x0[j])) * np.exp(1j * v[j] * x) for j in range(3))
        out.append((lin, nl, np.fft.fft(u)))
    return out


def burgers_ensemble(count: int, seed: int, n: int = 512, nu_range: Sequence[float] = (1e-3, 1e-1)) -> List[Instance]:
    """Viscous Burgers on [0, 2 pi) (real grid of n points): nu log-uniform over nu_range,
    u0 = sum_{k=1..6} a_k sin(k x) with a_k ~ N(0, 1/k)."""
    rng = np.random.default_rng(seed)
    _, kx = grids.construct_x_kx_rfft(n, 0.0, 2 * np.pi)
    x = np.arange(n) * (2 * np.pi / n)
    k = np.arange(1, 7)
    out = []
    for _ in range(count):
        nu = float(np.exp(rng.uniform(np.log(nu_range[0]), np.log(nu_range[1]))))
        lin, nl = models.burgers_ops(kx, nu)
        a = rng.standard_normal(6) / k
        out.append((lin, nl, np.fft.rfft(np.sum(a[:, None] * np.sin(k[:, None] * x[None, :]), axis=0))))
    return out


def ks_ensemble(count: int, seed: int, n_choices: Sequence[int] = (256, 512, 1024, 2048),
                L_range: Sequence[float] = (22.0, 120.0)) -> List[Instance]:
    """Kuramoto-Sivashinsky instances of mixed grid sizes: n uniform over n_choices,
    L ~ U[L_range], u0 = sum_{k=1..8} a_k cos(2 pi k x / L + phi_k), a_k ~ N(0,1) exp(-k/4)."""
    rng = np.random.default_rng(seed)
    k = np.arange(1, 9)
    out = []
    for _ in range(count):
        n = int(rng.choice(np.asarray(n_choices)))
        L = float(rng.uniform(*L_range))
        _, kx = grids.construct_x_kx_rfft(n, 0.0, L)
        x = np.arange(n) * (L / n)
        lin, nl = models.ks_ops(kx)
        a = rng.standard_normal(8) * np.exp(-k / 4.0)
        ph = rng.uniform(0.0, 2 * np.pi, 8)
        u = np.sum(a[:, None] * np.cos(2 * np.pi * k[:, None] * x[None, :] / L + ph[:, None]), axis=0)
        out.append((lin, nl, np.fft.rfft(u)))
    return out


def cheb_points_matrix(n: int, a: float = -1.0, b: float = 1.0):
    """n + 1 Chebyshev extreme points on [a, b] and the differentiation matrix
    (rkstiff/grids.py:134-219)."""
    x = np.polynomial.chebyshev.chebpts2(n + 1)
    x = a + (b - a) * (x + 1) / 2.0
    c = np.r_[2, np.ones(n - 1), 2] * np.power(-1, np.arange(0, n + 1))
    X = np.tile(x.reshape(n + 1, 1), (1, n + 1))
    dX = X - X.T
    D = np.outer(c, 1.0 / c) / (dX + np.eye(n + 1))
    return x, D - np.diag(D.sum(axis=1))


def allen_cahn_batch(count: int, seed: int, n: int = 129, epsilon: float = 0.01):
    """Allen-Cahn on the n + 1 Chebyshev points of [-1, 1] (n - 1 interior points, 128 for
    n = 129) with u(+-1) = +-1: (lin_op, nl_func, w0[count, n-1]) where
    u0 = 0.53 x + 0.47 sin(-1.5 pi x) + 0.1 N(0, 1) smoothed by a 5-point moving average on
    the interior, and w0 = u0 - x (the lifted state of models.allen_cahn_ops)."""
    x, D = cheb_points_matrix(n)
    lin, nl = models.allen_cahn_ops(x, D, epsilon)
    xi = x[1:-1]
    rng = np.random.default_rng(seed)
    base = 0.53 * xi + 0.47 * np.sin(-1.5 * np.pi * xi)
    noise = 0.1 * rng.standard_normal((count, xi.size))
    k = np.ones(5) / 5.0
    smooth = np.stack([np.convolve(r, k, mode="same") for r in noise])
    return lin, nl, base[None, :] + smooth - xi[None, :]
