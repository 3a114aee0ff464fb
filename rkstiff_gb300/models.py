"""Model equations whose nonlinearities run as fused device kernels.

Each ``*_ops`` helper returns ``(lin_op, nl_func)`` like rkstiff/models.py does, but
``nl_func`` is a :class:`BuiltinNL`: a callable that also tells the solvers which fused
kernel to run.  Calling it directly evaluates the same map with torch (on the device of a
tensor argument), which is also what the host-driven path for user callables uses.
"""

from __future__ import annotations

from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native as nat


class BuiltinNL:
    """A nonlinearity with a fused device implementation.

    kind  : RK_NL_UUX  -> c * rfft(irfft(u) * irfft(i kx u))   (real grid, n points)
            RK_NL_NLS  -> fft(i c |ifft(u)|^2 ifft(u))          (complex grid, n points)
            RK_NL_ALLEN_CAHN -> x - (u + x)^3 on the points x     (dense operators)
            RK_NL_NONE -> 0
    """

    def __init__(self, kind: int, coef: float, n: int, kx: Optional[np.ndarray] = None, name: str = "",
                 shift: Optional[np.ndarray] = None):
        self.kind = int(kind)
        self.coef = float(coef)
        self.n = int(n)
        self.kx = None if kx is None else np.asarray(kx, dtype=np.float64)
        self.shift = None if shift is None else np.asarray(shift, dtype=np.float64)
        self.name = name or {nat.RK_NL_UUX: "uux", nat.RK_NL_NLS: "nls", nat.RK_NL_NONE: "zero",
                             nat.RK_NL_ALLEN_CAHN: "allen_cahn"}[self.kind]
        self._kx_t = {}

    @property
    def modes(self) -> int:
        return self.n // 2 + 1 if self.kind == nat.RK_NL_UUX else self.n

    def _kx(self, device, dtype):
        key = (str(device), dtype)
        if key not in self._kx_t:
            self._kx_t[key] = torch.as_tensor(self.kx, dtype=dtype, device=device)
        return self._kx_t[key]

    def torch_eval(self, u: torch.Tensor) -> torch.Tensor:
        if self.kind == nat.RK_NL_UUX:
            rdt = torch.float64 if u.dtype == torch.complex128 else torch.float32
            kx = self._kx(u.device, rdt)
            a = torch.fft.irfft(u, n=self.n)
            b = torch.fft.irfft(1j * kx * u, n=self.n)
            return self.coef * torch.fft.rfft(a * b)
        if self.kind == nat.RK_NL_NLS:
            v = torch.fft.ifft(u)
            return torch.fft.fft(1j * self.coef * (v.abs() ** 2) * v)
        if self.kind == nat.RK_NL_ALLEN_CAHN:
            x = torch.as_tensor(self.shift, dtype=u.real.dtype if u.is_complex() else u.dtype, device=u.device)
            return (x - (u + x) ** 3).to(u.dtype)
        return torch.zeros_like(u)

    def __call__(self, u):
        if isinstance(u, torch.Tensor):
            return self.torch_eval(u)
        t = torch.from_numpy(np.asarray(u, dtype=np.complex128))
        return self.torch_eval(t).numpy()

    def __repr__(self):
        return f"BuiltinNL({self.name}, coef={self.coef}, n={self.n})"


def allen_cahn_ops(x: np.ndarray, d_cheb_matrix: np.ndarray, epsilon: float = 0.01) -> Tuple[np.ndarray, BuiltinNL]:
    """Allen-Cahn on Chebyshev points (rkstiff/models.py:202-247): L = epsilon D^2 + I without
    the boundary rows and columns, N(w) = x - (w + x)^3 on the interior points (the state w is
    u - x, which vanishes at both ends for u(+-1) = +-1)."""
    x = np.asarray(x, dtype=np.float64)
    D = np.asarray(d_cheb_matrix, dtype=np.float64)
    lin = (epsilon * D.dot(D) + np.eye(*D.shape))[1:-1, 1:-1]
    xi = x[1:-1]
    return lin, BuiltinNL(nat.RK_NL_ALLEN_CAHN, 1.0, len(xi), None, "allen_cahn", shift=xi)


def _n_from_rfft_kx(kx) -> int:
    return 2 * (len(kx) - 1)


def ks_ops(kx: np.ndarray) -> Tuple[np.ndarray, BuiltinNL]:
    """Kuramoto-Sivashinsky: L = kx^2 (1 - kx^2), N = -rfft(u u_x) (README quickstart)."""
    kx = np.asarray(kx, dtype=np.float64)
    return kx**2 * (1 - kx**2), BuiltinNL(nat.RK_NL_UUX, -1.0, _n_from_rfft_kx(kx), kx, "ks")


def kdv_ops(kx: np.ndarray) -> Tuple[np.ndarray, BuiltinNL]:
    """KdV: L = i kx^3, N = -6 rfft(u u_x) (rkstiff/models.py:113-145)."""
    kx = np.asarray(kx, dtype=np.float64)
    return 1j * kx**3, BuiltinNL(nat.RK_NL_UUX, -6.0, _n_from_rfft_kx(kx), kx, "kdv")


def burgers_ops(kx: np.ndarray, mu: float) -> Tuple[np.ndarray, BuiltinNL]:
    """Viscous Burgers: L = -mu kx^2, N = -rfft(u u_x) (rkstiff/models.py:153-194)."""
    kx = np.asarray(kx, dtype=np.float64)
    return -mu * kx**2, BuiltinNL(nat.RK_NL_UUX, -1.0, _n_from_rfft_kx(kx), kx, "burgers")


def nls_ops(kx: np.ndarray, coef: float = 1.0) -> Tuple[np.ndarray, BuiltinNL]:
    """Cubic NLS on a complex grid: L = -(i/2) kx^2, N = fft(i c |u|^2 u)."""
    kx = np.asarray(kx, dtype=np.float64)
    return -0.5j * kx**2, BuiltinNL(nat.RK_NL_NLS, coef, len(kx), None, "nls")


def kdv_soliton(x: np.ndarray, ampl: float = 0.5, x0: float = 0.0, t: float = 0.0) -> np.ndarray:
    """Exact KdV soliton (rkstiff/models.py:32-73)."""
    return 0.5 * ampl**2 / (np.cosh(ampl * (x - x0 - ampl**2 * t) / 2) ** 2)


def kdv_multi_soliton(x: np.ndarray, ampl: Sequence[float], x0: Sequence[float], t: float = 0.0) -> np.ndarray:
    """Sum of KdV solitons (rkstiff/models.py:76-110)."""
    if len(x0) != len(ampl):
        raise ValueError("Lengths of ampl and x0 must match.")
    a = np.asarray(ampl, dtype=float).reshape(1, -1)
    c = np.asarray(x0, dtype=float).reshape(1, -1)
    xx = np.asarray(x).reshape(-1, 1)
    return np.sum(0.5 * a**2 / (np.cosh(a * (xx - c - a**2 * t) / 2) ** 2), axis=1)


# ---------------------------------------------------------------------------------------
# multi-dimensional cubic NLS (the reference's NLS demo, demos/nls.ipynb): the state is the
# flattened spectrum of a 2-D field, lin_op the flattened (diagonal) dispersion, and the
# nonlinearity a device-side torch callable (the solvers' callable path) that reshapes,
# transforms back, forms i gamma |F|^2 F and transforms forward.
# ---------------------------------------------------------------------------------------
def _pow2(n: int) -> bool:
    return n >= 1 and (n & (n - 1)) == 0


class SpectralNL:
    """A nonlinearity ``g -> fwd(i gamma |F|^2 F)`` with ``F = inv(g)`` on a flattened
    spectrum.  On a CUDA tensor it runs the library's kernels (``_device``: line FFTs with
    the product fused between them, ``rk_nls_lines``, and the Hankel product ``rk_dht``)
    when the transform lengths are powers of two, torch's FFTs otherwise; NumPy input is
    evaluated on the host and returned as NumPy."""

    def __init__(self, shape, inv, fwd, gamma: float, name: str, ht=None):
        self.shape, self._inv, self._fwd = tuple(shape), inv, fwd
        self.gamma, self.name = float(gamma), name
        self._ht = ht

    def _lines(self, mode, n, lines, es, ls, x, out):
        from . import _native as nat
        from .engine import twiddles

        prec = nat.RK_FP64 if x.dtype == torch.complex128 else nat.RK_FP32
        lib = nat.load()
        nat.check(lib.rk_nls_lines(prec, mode, n, lines, es, ls, self.gamma, x.data_ptr(), out.data_ptr(),
                                   twiddles(x.device, prec).data_ptr(), torch.cuda.current_stream(x.device).cuda_stream),
                  "rk_nls_lines")
        return out

    def _device(self, g):
        """The nonlinearity on the library's kernels, or None when a length is unsupported."""
        if g.dtype not in (torch.complex128, torch.complex64):
            return None
        if self.name == "nls_2d":
            nx, ny = self.shape
            if not (_pow2(nx) and _pow2(ny) and nx > 1 and ny > 1):
                return None
            G = g.reshape(nx, ny).contiguous()  # may be a view of the caller's tensor: read only
            W = torch.empty_like(G)
            out = torch.empty_like(G)
            with torch.cuda.device(g.device):
                self._lines(0, ny, nx, 1, ny, G, W)   # ifft along axis 1 (rows)
                self._lines(2, nx, ny, ny, 1, W, W)   # fft(i gamma |v|^2 v), v = ifft, along axis 0
                self._lines(1, ny, nx, 1, ny, W, out)  # fft along axis 1
            return out.reshape(-1)
        if self.name in ("nls_radial", "nls_radial_time") and self._ht is not None:
            nt = self.shape[1] if self.name == "nls_radial_time" else 1
            if not _pow2(nt):
                return None
            nr = self.shape[0]
            X = self._ht.iht(g.reshape(nr, nt) if nt > 1 else g.reshape(nr).contiguous())
            with torch.cuda.device(g.device):
                self._lines(2, nt, nr, 1, nt, X, X)
            return self._ht.ht(X).reshape(-1)
        return None

    def __call__(self, g):
        if not isinstance(g, torch.Tensor):
            return self(torch.from_numpy(np.asarray(g, dtype=np.complex128))).numpy()
        if g.is_cuda:
            out = self._device(g)
            if out is not None:
                return out
        F = self._inv(g.reshape(self.shape))
        a2 = F.real * F.real + F.imag * F.imag
        return self._fwd((1j * self.gamma) * (a2 * F)).reshape(-1)

    def __repr__(self):
        return f"SpectralNL({self.name}, shape={self.shape}, gamma={self.gamma})"


def nls_radial_ops(ht, gamma: float = 2.0) -> Tuple[np.ndarray, SpectralNL]:
    """Radially symmetric NLS on a Hankel grid (demos/nls.ipynb cells 6-12):
    L = -i kr^2, N(g) = i gamma ht(|f|^2 f) with f = iht(g); ``ht`` a
    ``transforms.HankelTransform`` (its transform runs as a GEMM on the device)."""
    return -1j * ht.kr**2, SpectralNL((ht.nr,), ht.iht, ht.ht, gamma, "nls_radial", ht=ht)


def nls_radial_time_ops(ht, omega: np.ndarray, sigma: float = 0.5,
                        gamma: float = 2.0) -> Tuple[np.ndarray, SpectralNL]:
    """(r, t) NLS with a Hankel transform over r (axis 0) and an FFT over t (axis 1)
    (demos/nls.ipynb cells 14-20): L = -i kr^2 + i sigma omega^2 flattened row-major over
    (nr, nt), N(g) = i gamma fft_t(ht(|F|^2 F)) with F = ifft_t(iht(g))."""
    omega = np.asarray(omega, dtype=np.float64)
    KR, OM = np.meshgrid(ht.kr, omega, indexing="ij")
    L = (-1j * KR**2 + 1j * sigma * OM**2).reshape(-1)

    def inv(G):
        return torch.fft.ifft(ht.iht(G), dim=1)

    def fwd(F):
        return torch.fft.fft(ht.ht(F), dim=1)
    return L, SpectralNL((ht.nr, len(omega)), inv, fwd, gamma, "nls_radial_time", ht=ht)


def nls_2d_ops(kx: np.ndarray, ky: np.ndarray, gamma: float = 2.0) -> Tuple[np.ndarray, SpectralNL]:
    """2-D NLS on complex FFT grids (demos/nls.ipynb cells 27-29): L = -i (kx^2 + ky^2)
    flattened row-major over (nx, ny), N(g) = i gamma fft2(|F|^2 F) with F = ifft2(g)."""
    kx = np.asarray(kx, dtype=np.float64)
    ky = np.asarray(ky, dtype=np.float64)
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    L = (-1j * (KX**2 + KY**2)).reshape(-1)
    return L, SpectralNL((len(kx), len(ky)), torch.fft.ifft2, torch.fft.fft2, gamma, "nls_2d")
