"""IF4: Fourth-order integrating-factor Runge-Kutta, constant step (rkstiff/if4.py:202-275), run on the device."""

from __future__ import annotations

from typing import Callable, Optional, Union

from .solvercs import BaseSolverCS


class IF4(BaseSolverCS):
    """Fourth-order integrating-factor Runge-Kutta, constant step."""

    _method_name = "IF4"

    def __init__(self, lin_op, nl_func: Callable, loglevel: Union[str, int] = "WARNING",
                 device_options=None) -> None:
        super().__init__(lin_op, nl_func, loglevel=loglevel, device_options=device_options)
