"""IF34: Fourth-order integrating-factor Runge-Kutta with a third-order embedding (rkstiff/if34.py:260-338), run on the device."""

from __future__ import annotations

from typing import Callable, Optional, Union

from .solver import check_diagonalizable
from .solveras import BaseSolverAS, SolverConfig


class IF34(BaseSolverAS):
    """Fourth-order integrating-factor Runge-Kutta with a third-order embedding.  ``_q()`` = 4 (the controller exponent is 1/q)."""

    _method_name = "IF34"

    def __init__(self, lin_op, nl_func: Callable, config: Optional[SolverConfig] = None, diagonalize: bool = False,
                 loglevel: Union[str, int] = "WARNING",
                 device_options=None) -> None:
        super().__init__(lin_op, nl_func, config, loglevel=loglevel, device_options=device_options)
        self.diagonalize = bool(diagonalize)
        if self.diagonalize and not self._diag:
            check_diagonalizable(lin_op, self.logger)
        self._accept = False

    def _q(self) -> int:
        return 4
