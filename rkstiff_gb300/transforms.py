"""Quasi-discrete Hankel transform of order zero (the interface of rkstiff/transforms.py:43-240),
usable on host arrays and on device tensors.

On the grids of ``grids.construct_r_kr_hankel`` the transform is one real matrix
Y_ij = 2 J0(j_i j_j / j_{N+1}) / (j_{N+1} J1(j_j)^2) (J0, J1 Bessel functions of the first
kind, j_i the zeros of J0): ``ht(f) = S Y f`` and ``iht(g) = Y g / S`` with
S = rmax^2 / j_{N+1}.  For a CUDA tensor the product runs in the library's tiled kernel
(``rk_dht``) over axis 0 (the radial axis), the real and imaginary parts of a complex tensor
as one real matrix of 2x the columns; the matrix is built once in FP64 on the host and
cached per device and dtype.  Host arrays use NumPy, as the reference does.
"""

from __future__ import annotations

from typing import Dict, Tuple

import numpy as np
import torch

from .grids import construct_r_kr_hankel


class HankelTransform:
    """Discrete Hankel transform on ``nr`` radial points in (0, rmax] (rkstiff/transforms.py:43)."""

    def __init__(self, nr: int, rmax: float = 1.0):
        self._dev: Dict[Tuple[str, torch.dtype], torch.Tensor] = {}
        self._set(nr, rmax)

    def _set(self, nr: int, rmax: float) -> None:
        from scipy import special

        self._nr, self._rmax = nr, rmax
        self.r, self.kr, self._zeros, self._jN = construct_r_kr_hankel(nr, rmax)
        j1 = special.j1(self._zeros)
        self._Y = 2.0 * special.j0(np.outer(self._zeros, self._zeros) / self._jN) / (self._jN * j1**2)
        self._dev = {}

    def _scalefactor(self) -> float:
        return self._rmax**2 / self._jN

    def hankel_matrix(self) -> np.ndarray:
        """The transform matrix Y (a copy)."""
        return self._Y.copy()

    def bessel_zeros(self) -> np.ndarray:
        """The first ``nr`` zeros of J0 (a copy)."""
        return self._zeros.copy()

    @property
    def nr(self) -> int:
        return self._nr

    @nr.setter
    def nr(self, nr: int) -> None:
        if not isinstance(nr, int) or nr < 4:
            raise ValueError("nr must be an integer >= 4.")
        self._set(nr, self._rmax)

    @property
    def rmax(self) -> float:
        return self._rmax

    @rmax.setter
    def rmax(self, rmax: float) -> None:
        if rmax <= 0:
            raise ValueError("rmax must be positive.")
        self._set(self._nr, rmax)

    # -- transforms ---------------------------------------------------------------------
    def _matrix(self, like: torch.Tensor) -> torch.Tensor:
        rdt = like.real.dtype if like.is_complex() else like.dtype
        key = (str(like.device), rdt)
        if key not in self._dev:
            self._dev[key] = torch.as_tensor(self._Y, dtype=torch.float64).to(device=like.device, dtype=rdt).contiguous()
        return self._dev[key]

    def _apply(self, f: torch.Tensor, divide: bool) -> torch.Tensor:
        if f.shape[0] != self._nr:
            raise ValueError(f"the radial axis has {f.shape[0]} points, the transform {self._nr}")
        if not f.is_cuda:
            M = torch.as_tensor(self._Y / self._scalefactor() if divide else self._scalefactor() * self._Y,
                                dtype=f.real.dtype if f.is_complex() else f.dtype)
            if not f.is_complex():
                return M @ f
            fr = torch.view_as_real(f.contiguous()).reshape(f.shape[0], -1)
            return torch.view_as_complex((M @ fr).reshape(*f.shape, 2).contiguous())
        from . import _native as nat

        if f.dtype not in (torch.float64, torch.float32, torch.complex128, torch.complex64):
            f = f.to(torch.float64)
        f = f.contiguous()
        prec = nat.RK_FP64 if f.dtype in (torch.float64, torch.complex128) else nat.RK_FP32
        w = (f.numel() // self._nr) * (2 if f.is_complex() else 1)
        out = torch.empty_like(f)
        lib = nat.load()
        with torch.cuda.device(f.device):
            nat.check(lib.rk_dht(prec, 1 if divide else 0, self._nr, w, self._matrix(f).data_ptr(),
                                 float(self._scalefactor()), f.data_ptr(), out.data_ptr(),
                                 torch.cuda.current_stream(f.device).cuda_stream), "rk_dht")
        return out

    def ht(self, f):
        """Forward transform over axis 0: S Y f (rkstiff/transforms.py:178-208)."""
        if isinstance(f, torch.Tensor):
            return self._apply(f, False)
        return self._scalefactor() * self._Y.dot(f)

    def iht(self, g):
        """Inverse transform over axis 0: Y g / S (rkstiff/transforms.py:210-240)."""
        if isinstance(g, torch.Tensor):
            return self._apply(g, True)
        return self._Y.dot(g) / self._scalefactor()
