"""ETD4: Fourth-order Krogstad ETD Runge-Kutta, constant step (rkstiff/etd4.py:311-422), run on the device."""

from __future__ import annotations

from typing import Callable, Optional, Union

from .etd import ETDCS, ETDConfig


class ETD4(ETDCS):
    """Fourth-order Krogstad ETD Runge-Kutta, constant step."""

    _method_name = "ETD4"

    def __init__(self, lin_op, nl_func: Callable, etd_config: Optional[ETDConfig] = None,
                 loglevel: Union[str, int] = "WARNING",
                 device_options=None) -> None:
        super().__init__(lin_op, nl_func, etd_config, loglevel=loglevel, device_options=device_options)
