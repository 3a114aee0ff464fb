"""ETD configuration, psi functions and the ETD solver shells (rkstiff/etd.py:46-278)."""

from __future__ import annotations

from typing import Callable, Optional, Union

import numpy as np

from .solveras import BaseSolverAS, SolverConfig
from .solvercs import BaseSolverCS


class ETDConfig:
    """psi-function evaluation settings (rkstiff/etd.py:81-131): ``modecutoff`` switches
    between the direct formula and the contour mean, ``contour_points`` / ``contour_radius``
    define the contour."""

    def __init__(self, modecutoff: float = 0.01, contour_points: int = 32, contour_radius: float = 1.0) -> None:
        self._modecutoff = 0.01
        self._contour_points = 32
        self._contour_radius = 1.0
        self.modecutoff = modecutoff
        self.contour_points = contour_points
        self.contour_radius = contour_radius

    @property
    def modecutoff(self) -> float:
        return self._modecutoff

    @modecutoff.setter
    def modecutoff(self, value: float) -> None:
        if (value > 1.0) or (value <= 0):
            raise ValueError(f"modecutoff must be between 0.0 and 1.0 but is {value}")
        self._modecutoff = value

    @property
    def contour_points(self) -> int:
        return self._contour_points

    @contour_points.setter
    def contour_points(self, value: int) -> None:
        if not isinstance(value, int):
            raise TypeError(f"contour_points must be an integer but is {value}")
        if value <= 1:
            raise ValueError(f"contour_points must be an integer greater than 1 but is {value}")
        self._contour_points = value

    @property
    def contour_radius(self) -> float:
        return self._contour_radius

    @contour_radius.setter
    def contour_radius(self, value: float) -> None:
        if value <= 0:
            raise ValueError(f"contour_radius must greater than 0 but is {value}")
        self._contour_radius = value


def psi1(z):
    """(e^z - 1)/z, elementwise."""
    return (np.exp(z) - 1) / z


def psi2(z):
    """2 (e^z - 1 - z)/z^2, elementwise."""
    return 2 * (np.exp(z) - 1 - z) / z**2


def psi3(z):
    """6 (e^z - 1 - z - z^2/2)/z^3, elementwise."""
    return 6 * (np.exp(z) - 1 - z - z**2 / 2) / z**3


class ETDAS(BaseSolverAS):
    """Adaptive ETD solver shell: adds ``etd_config`` and the coefficient cache key."""

    def __init__(self, lin_op, nl_func: Callable, config: Optional[SolverConfig] = None,
                 etd_config: Optional[ETDConfig] = None, loglevel: Union[str, int] = "WARNING",
                 device_options=None) -> None:
        super().__init__(lin_op, nl_func, config, loglevel=loglevel, device_options=device_options)
        self.etd_config = etd_config if etd_config is not None else ETDConfig()
        self._h_coeff = None


class ETDCS(BaseSolverCS):
    """Constant-step ETD solver shell."""

    def __init__(self, lin_op, nl_func: Callable, etd_config: Optional[ETDConfig] = None,
                 loglevel: Union[str, int] = "WARNING", device_options=None) -> None:
        super().__init__(lin_op, nl_func, loglevel=loglevel, device_options=device_options)
        self.etd_config = etd_config if etd_config is not None else ETDConfig()
        self._h_coeff = None
