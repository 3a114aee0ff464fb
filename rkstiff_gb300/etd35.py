"""ETD35: Fifth-order ETD Runge-Kutta with a third-order embedding (rkstiff/etd35.py:723-889), run on the device."""

from __future__ import annotations

from typing import Callable, Optional, Union

from .etd import ETDAS, ETDConfig, SolverConfig
from .solver import check_diagonalizable


class ETD35(ETDAS):
    """Fifth-order ETD Runge-Kutta with a third-order embedding.  ``_q()`` = 4 (the controller exponent is 1/q)."""

    _method_name = "ETD35"

    def __init__(self, lin_op, nl_func: Callable, config: Optional[SolverConfig] = None, etd_config: Optional[ETDConfig] = None, diagonalize: bool = False,
                 loglevel: Union[str, int] = "WARNING",
                 device_options=None) -> None:
        super().__init__(lin_op, nl_func, config, etd_config, loglevel=loglevel, device_options=device_options)
        self.diagonalize = bool(diagonalize)
        if self.diagonalize and not self._diag:
            check_diagonalizable(lin_op, self.logger)
        self._accept = False

    def _q(self) -> int:
        return 4
