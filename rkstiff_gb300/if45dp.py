"""IF45DP: Dormand-Prince 5(4) integrating-factor method (diagonal operators only) (rkstiff/if45dp.py:8-249), run on the device."""

from __future__ import annotations

from typing import Callable, Optional, Union

from .solver import _shape
from .solveras import BaseSolverAS, SolverConfig


class IF45DP(BaseSolverAS):
    """Dormand-Prince 5(4) integrating-factor method (diagonal operators only).  ``_q()`` = 5 (the controller exponent is 1/q)."""

    _method_name = "IF45DP"

    def __init__(self, lin_op, nl_func: Callable, config: Optional[SolverConfig] = None,
                 loglevel: Union[str, int] = "WARNING",
                 device_options=None) -> None:
        super().__init__(lin_op, nl_func, config, loglevel=loglevel, device_options=device_options)
        if len(_shape(lin_op)) > 1:
            raise ValueError("IF45DP only handles 1D linear operators (diagonal systems): try IF34,ETD34, or ETD35")
        self._accept = False

    def _q(self) -> int:
        return 5
