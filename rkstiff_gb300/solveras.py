"""Adaptive-step solver base: SolverConfig and BaseSolverAS (the interface of
rkstiff/solveras.py:27-650), executed on the device.

The retry loop, the masked error norm, the reject/accept step-size rules and the evolve
loop all run inside the persistent kernel; this class validates arguments, maps the
per-instance status back to the reference's exceptions and fills ``t`` / ``u``.
"""

from __future__ import annotations

from typing import Callable, Optional, Tuple, Union

from . import _native as nat
from .solver import BaseSolver
from .util.solver_type import SolverType


class SolverConfig:
    """Adaptive step-size settings with the reference defaults and validators
    (rkstiff/solveras.py:71-169)."""

    def __init__(self, epsilon: float = 1e-4, incr_f: float = 1.25, decr_f: float = 0.85, safety_f: float = 0.8,
                 adapt_cutoff: float = 0.01, minh: float = 1e-16) -> None:
        self._epsilon = self._incr_f = self._decr_f = self._safety_f = self._adapt_cutoff = self._minh = None
        self.epsilon = epsilon
        self.incr_f = incr_f
        self.decr_f = decr_f
        self.safety_f = safety_f
        self.adapt_cutoff = adapt_cutoff
        self.minh = minh

    @property
    def epsilon(self) -> float:
        return self._epsilon

    @epsilon.setter
    def epsilon(self, value: float) -> None:
        if value <= 0:
            raise ValueError(f"epsilon must be positive but is {value}")
        self._epsilon = float(value)

    @property
    def incr_f(self) -> float:
        return self._incr_f

    @incr_f.setter
    def incr_f(self, value: float) -> None:
        if value <= 1.0:
            raise ValueError(f"incr_f must be > 1.0 but is {value}")
        self._incr_f = float(value)

    @property
    def decr_f(self) -> float:
        return self._decr_f

    @decr_f.setter
    def decr_f(self, value: float) -> None:
        if value >= 1.0:
            raise ValueError(f"decr_f must be < 1.0 but is {value}")
        self._decr_f = float(value)

    @property
    def safety_f(self) -> float:
        return self._safety_f

    @safety_f.setter
    def safety_f(self, value: float) -> None:
        if value > 1.0:
            raise ValueError(f"safety_f must be <= 1.0 but is {value}")
        self._safety_f = float(value)

    @property
    def adapt_cutoff(self) -> float:
        return self._adapt_cutoff

    @adapt_cutoff.setter
    def adapt_cutoff(self, value: float) -> None:
        if value >= 1.0:
            raise ValueError(f"adapt_cutoff must be < 1.0 but is {value}")
        self._adapt_cutoff = float(value)

    @property
    def minh(self) -> float:
        return self._minh

    @minh.setter
    def minh(self, value: float) -> None:
        if value <= 0:
            raise ValueError(f"minh must be positive but is {value}")
        self._minh = float(value)


class BaseSolverAS(BaseSolver):
    """Adaptive-step solver: ``step(u, h_suggest) -> (u, h, h_suggest)`` and
    ``evolve(u, t0, tf, h_init=None, store_data=True, store_freq=1)``."""

    class SolverError(RuntimeError):
        """Base exception for solver-related runtime errors."""

    class MaxLoopsExceeded(SolverError):
        """Raised when too many attempts are made to find a valid adaptive step."""

    class MinimumStepReached(SolverError):
        """Raised when the adaptive step size falls below the minimum allowed value."""

    MAX_LOOPS = 50
    MAX_S = 4.0
    MIN_S = 0.25

    _method_name = ""

    def __init__(self, lin_op, nl_func: Callable, config: Optional[SolverConfig] = None,
                 loglevel: Union[str, int] = "WARNING", device_options=None) -> None:
        super().__init__(lin_op, nl_func, loglevel, device_options)
        # a fresh SolverConfig per solver: the reference's shared default instance
        # (solveras.py:266) would leak mutations between solvers
        self.config = config if config is not None else SolverConfig()
        self.logger.debug("Adaptive configuration: epsilon=%s, incr_f=%s, decr_f=%s, safety_f=%s",
                          self.config.epsilon, self.config.incr_f, self.config.decr_f, self.config.safety_f)
        self._accept = False
        self._backend = None

    @property
    def solver_type(self) -> SolverType:
        return SolverType.ADAPTIVE_STEP

    def _engine(self):
        if self._backend is None:
            from ._backend import DenseBackend, DiagBackend
            from ._callable import CallableBackend, EigenBackend
            from .models import BuiltinNL
            if not self._diag:
                # FP32 ETD35 with the built-in Allen-Cahn nonlinearity: the tensor-core stages;
                # any other dense problem: the eigenbasis stepping in the chosen precision
                if DenseBackend.takes(self):
                    self._backend = DenseBackend(self, self._method_name)
                else:
                    self._backend = EigenBackend(self, self._method_name)
            elif isinstance(self.nl_func, BuiltinNL):
                self._backend = DiagBackend(self, self._method_name)
            else:
                self._backend = CallableBackend(self, self._method_name)
        return self._backend

    def reset(self) -> None:
        self.logger.debug("Resetting adaptive solver state")
        self.t, self.u = [], []
        self._accept = False
        self._reset()

    def _reset(self) -> None:
        if self._backend is not None:
            self._backend.reset()

    def _raise_for(self, status: int) -> None:
        if status == nat.RK_ST_MAX_LOOPS:
            msg = ("Solver failed: adaptive step made too many attempts to find a step size with an acceptible "
                   "amount of error.")
            self.logger.error(msg)
            raise self.MaxLoopsExceeded(msg)
        if status == nat.RK_ST_MIN_STEP:
            msg = "Solver failed: adaptive step reached minimum step size"
            self.logger.error(msg)
            raise self.MinimumStepReached(msg)

    def step(self, u, h_suggest: float) -> Tuple[object, float, float]:
        """One accepted adaptive step (retries on the device): rkstiff/solveras.py:336-410."""
        h = h_suggest
        assert h >= 0.0
        be = self._engine()
        unew, status = be.step(u, h)
        self._accept = bool(be.st["accept"][0])
        self._raise_for(status)
        return unew, float(be.st["h_used"][0]), float(be.st["h_suggest"][0])

    def evolve(self, u, t0: float, tf: float, h_init: Optional[float] = None, store_data: bool = True,
               store_freq: int = 1):
        """Integrate from t0 to tf on the device: rkstiff/solveras.py:556-650."""
        self.reset()
        self.logger.info("Starting evolution from t=%s to t=%s", t0, tf)
        if store_data:
            self.t.append(t0)
            self.u.append(u)
        if h_init is None:
            h_init = (tf - t0) / 100.0
        h = h_init
        if t0 + h > tf:
            h = tf - t0
        be = self._engine()
        ufinal, status = be.evolve(u, t0, tf, h, store_data, store_freq)
        self._accept = bool(be.st["accept"][0])
        self._raise_for(status)
        self.logger.info("Evolution complete after %d steps", int(be.st["steps"][0]))
        return ufinal

    @property
    def stats(self) -> dict:
        """Device counters of the last evolve/step: steps, attempts, rejects, nl_evals,
        coeff_updates."""
        return self._engine().counters
