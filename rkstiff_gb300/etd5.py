"""ETD5: Fifth-order ETD Runge-Kutta, constant step (rkstiff/etd5.py), run on the device."""

from __future__ import annotations

from typing import Callable, Optional, Union

from .etd import ETDCS, ETDConfig


class ETD5(ETDCS):
    """Fifth-order ETD Runge-Kutta, constant step."""

    _method_name = "ETD5"

    def __init__(self, lin_op, nl_func: Callable, etd_config: Optional[ETDConfig] = None,
                 loglevel: Union[str, int] = "WARNING",
                 device_options=None) -> None:
        super().__init__(lin_op, nl_func, etd_config, loglevel=loglevel, device_options=device_options)
