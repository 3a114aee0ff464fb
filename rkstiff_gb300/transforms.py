"""Quasi-discrete Hankel transform of order zero (the interface of rkstiff/transforms.py:43-240),
usable on host arrays and on device tensors.

On the grids of ``grids.construct_r_kr_hankel`` the transform is one real matrix
Y_ij = 2 J0(j_i j_j / j_{N+1}) / (j_{N+1} J1(j_j)^2) (J0, J1 Bessel functions of the first
kind, j_i the zeros of J0): ``ht(f) = S Y f`` and ``iht(g) = Y g / S`` with
S = rmax^2 / j_{N+1}.  For a torch tensor the product is a GEMM on the tensor's device over
axis 0 (the radial axis), the real and imaginary parts of a complex tensor as one real
matrix of 2x the columns; the matrix is built once in FP64 on the host and cached per
device and dtype.
"""

from __future__ import annotations

from typing import Dict, Tuple

import numpy as np
import torch

from .grids import construct_r_kr_hankel


class HankelTransform:
    """Discrete Hankel transform on ``nr`` radial points in (0, rmax] (rkstiff/transforms.py:43)."""

    def __init__(self, nr: int, rmax: float = 1.0):
        self._dev: Dict[Tuple[str, torch.dtype], Tuple[torch.Tensor, torch.Tensor]] = {}
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
    def _matrices(self, like: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
        rdt = like.real.dtype if like.is_complex() else like.dtype
        key = (str(like.device), rdt)
        if key not in self._dev:
            s = self._scalefactor()
            fwd = torch.as_tensor(s * self._Y, dtype=torch.float64).to(device=like.device, dtype=rdt)
            inv = torch.as_tensor(self._Y / s, dtype=torch.float64).to(device=like.device, dtype=rdt)
            self._dev[key] = (fwd.contiguous(), inv.contiguous())
        return self._dev[key]

    @staticmethod
    def _apply(M: torch.Tensor, f: torch.Tensor) -> torch.Tensor:
        if not f.is_complex():
            return M @ f
        shape = f.shape
        fr = torch.view_as_real(f.contiguous()).reshape(shape[0], -1)  # [nr, 2 * rest]
        out = (M @ fr).reshape(*shape, 2)
        return torch.view_as_complex(out.contiguous())

    def ht(self, f):
        """Forward transform over axis 0: S Y f (rkstiff/transforms.py:178-208)."""
        if isinstance(f, torch.Tensor):
            return self._apply(self._matrices(f)[0], f)
        return self._scalefactor() * self._Y.dot(f)

    def iht(self, g):
        """Inverse transform over axis 0: Y g / S (rkstiff/transforms.py:210-240)."""
        if isinstance(g, torch.Tensor):
            return self._apply(self._matrices(g)[1], g)
        return self._Y.dot(g) / self._scalefactor()
