"""BaseSolver: operator/nonlinearity holder, logger and snapshot lists
(the interface of rkstiff/solver.py:30-213)."""

from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Callable, Optional, Union

import numpy as np
import torch

from .device import DeviceOptions
from .util.loghelper import get_level_name, get_solver_logger, set_log_level


def _shape(a):
    if isinstance(a, torch.Tensor):
        return tuple(a.shape)
    return np.shape(a)


def check_diagonalizable(lin_op, logger) -> None:
    """The diagonalized strategies' checks on a 2-D lin_op, made when the solver is built
    (etd35.py:412-418, etd34.py:235-243, if34.py:157-163): ValueError when cond(lin_op) >
    1e16, a warning above 1000."""
    a = lin_op.detach().cpu().numpy() if isinstance(lin_op, torch.Tensor) else np.asarray(lin_op)
    cond = np.linalg.cond(a)
    if cond > 1e16:
        raise ValueError("cannot diagonalize a non-invertible linear operator L")
    if cond > 1000:
        logger.warning(f"Linear matrix array has a large condition number of {cond:.2f}, method may be unstable")


class BaseSolver(ABC):
    """Stores ``lin_op`` / ``nl_func``, validates the operator shape (1-D diagonal or
    square 2-D, rkstiff/solver.py:129-135) and keeps the ``t`` / ``u`` snapshot lists."""

    def __init__(self, lin_op, nl_func: Callable, loglevel: Union[str, int] = "WARNING",
                 device_options: Optional[DeviceOptions] = None) -> None:
        self.lin_op = lin_op
        self.nl_func = nl_func
        self.logger = get_solver_logger(self.__class__, loglevel)
        self.logger.info("Initialized %s solver", self.__class__.__name__)
        self.t, self.u = [], []
        dims = _shape(lin_op)
        if len(dims) not in (1, 2):
            raise ValueError("lin_op must be 1D or 2D")
        if len(dims) == 2 and dims[0] != dims[1]:
            raise ValueError("lin_op must be a square matrix")
        self._diag = len(dims) == 1
        self.device_options = device_options if device_options is not None else DeviceOptions()
        self.logger.debug("Linear operator shape: %s, diagonal: %s", dims, self._diag)

    @property
    @abstractmethod
    def solver_type(self):
        """SolverType.CONSTANT_STEP or SolverType.ADAPTIVE_STEP."""

    def set_loglevel(self, loglevel: Union[str, int]) -> None:
        set_log_level(self.logger, loglevel)
        self.logger.info("Log level changed to %s", get_level_name(self.logger.level))

    @abstractmethod
    def reset(self) -> None:
        """Clear the snapshot lists and the stepping state."""

    @abstractmethod
    def _reset(self) -> None:
        """Clear method-specific state."""
