"""Constant-step solver base (the interface of rkstiff/solvercs.py:31-279), executed on
the device."""

from __future__ import annotations

from typing import Callable, Union

from .solver import BaseSolver
from .util.solver_type import SolverType


class BaseSolverCS(BaseSolver):
    """``step(u, h) -> u`` and ``evolve(u, t0, tf, h, store_data=True, store_freq=1)``."""

    _method_name = ""

    def __init__(self, lin_op, nl_func: Callable, loglevel: Union[str, int] = "WARNING", device_options=None):
        super().__init__(lin_op, nl_func, loglevel, device_options)
        self._backend = None

    @property
    def solver_type(self) -> SolverType:
        return SolverType.CONSTANT_STEP

    def _engine(self):
        if self._backend is None:
            from ._backend import DiagBackend
            from ._callable import CallableBackend, EigenBackend
            from .models import BuiltinNL
            if not self._diag:
                self._backend = EigenBackend(self, self._method_name)
            elif isinstance(self.nl_func, BuiltinNL):
                self._backend = DiagBackend(self, self._method_name)
            else:
                self._backend = CallableBackend(self, self._method_name)
        return self._backend

    def reset(self) -> None:
        self.logger.debug("Resetting constant-step solver state")
        self.t, self.u = [], []
        self._reset()

    def _reset(self) -> None:
        if self._backend is not None:
            self._backend.reset()

    def step(self, u, h: float):
        """One step of size h: rkstiff/solvercs.py:163-186."""
        assert h >= 0.0
        unew, _ = self._engine().step(u, h)
        return unew

    def evolve(self, u, t0: float, tf: float, h: float, store_data: bool = True, store_freq: int = 1):
        """Fixed-step integration until t >= tf: rkstiff/solvercs.py:191-279."""
        self.reset()
        self.logger.info("Starting constant-step evolution from t=%s to t=%s", t0, tf)
        if store_data:
            self.t.append(t0)
            self.u.append(u)
        if t0 + h > tf:
            raise ValueError("Step size h must be <= (tf - t0); reduce h or extend tf.")
        ufinal, _ = self._engine().evolve(u, t0, tf, h, store_data, store_freq)
        return ufinal

    @property
    def stats(self) -> dict:
        return self._engine().counters
