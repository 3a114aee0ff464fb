"""Batched ensembles: thousands of independent instances, each with its own grid size,
operator and adaptive step, advanced by one persistent kernel launch.

The reference runs one solver object per problem; an ensemble is the same algorithm per
instance (rkstiff/solveras.py:556-650 with the method's stage program), with the
instances sharing one launch.  All instances use the same method and the same kind of
built-in nonlinearity (its constant and wavenumbers may differ per instance).
"""

from __future__ import annotations

from typing import Optional, Sequence

import numpy as np
import torch

from . import _native as nat
from .engine import DiagEnsemble, EvolveBoundError
from .models import BuiltinNL

STATUS_NAMES = {nat.RK_ST_DONE: "done", nat.RK_ST_MAX_LOOPS: "max_loops", nat.RK_ST_MIN_STEP: "min_step",
                nat.RK_ST_RUNNING: "running", nat.RK_ST_ITER_CAP: "iter_cap", nat.RK_ST_SNAP_FULL: "snap_full",
                nat.RK_ST_STEP_DONE: "step_done", nat.RK_ST_BAD_SIZE: "bad_size"}


class Ensemble:
    """Independent instances of u_t = L_i u + N_i(u) advanced together on one GPU.

    Parameters
    ----------
    method : 'IF34' | 'ETD35' | 'ETD34' | 'IF45DP' | 'ETD4' | 'ETD5' | 'IF4'
    lin_ops : per-instance 1-D operators
    nl_funcs : per-instance :class:`BuiltinNL` (same kind and constant for all)
    config, etd_config : SolverConfig / ETDConfig shared by all instances
    precision : 'fp32' (default) or 'fp64'
    schedule : 'history' (default: after each evolve, every grid-size class is queued
        longest-first by that evolve's attempt counts) or 'size' (index order)
    """

    def __init__(self, method: str, lin_ops: Sequence, nl_funcs: Sequence[BuiltinNL], config=None, etd_config=None,
                 precision: str = "fp32", device=None, threads: int = 0, schedule: str = "history"):
        if schedule not in ("history", "size"):
            raise ValueError("schedule must be 'history' or 'size'")
        if len(nl_funcs) != len(lin_ops):
            raise ValueError("one nonlinearity per instance is required")
        kinds = {(nl.kind, nl.coef) for nl in nl_funcs}
        if len(kinds) != 1:
            raise ValueError("all instances of an ensemble must share the nonlinearity kind and constant")
        if not all(isinstance(nl, BuiltinNL) for nl in nl_funcs):
            raise TypeError("ensembles run built-in nonlinearities (rkstiff_gb300.models)")
        nl0 = nl_funcs[0]
        kxs = [nl.kx for nl in nl_funcs] if nl0.kind == nat.RK_NL_UUX else None
        self.method = method
        self.adaptive = method in ("IF34", "ETD35", "ETD34", "IF45DP")
        self.engine = DiagEnsemble(method, lin_ops, nl0.kind, nl0.coef, kxs, [nl.n for nl in nl_funcs],
                                   precision=precision, config=config, etd_config=etd_config, device=device,
                                   threads=threads)
        self.engine.schedule = schedule
        self.state = None
        self._lin_ops = list(lin_ops)
        self._kxs = kxs

    def autotune(self, u0s: Sequence, span: float, **kw) -> dict:
        """Pick threads and scratch placement per grid-size class by timing candidates on
        a sample of each class over ``span`` of simulated time (see rkstiff_gb300.autotune)."""
        from . import autotune
        return autotune.tune(self.engine, u0s, self._lin_ops, self._kxs, span, **kw)

    @property
    def n_inst(self) -> int:
        return self.engine.n_inst

    @property
    def modes(self) -> np.ndarray:
        return self.engine.ms.copy()

    def pack(self, u0s: Sequence) -> torch.Tensor:
        """Concatenated device copy of the initial spectra (working dtype)."""
        return self.engine.pack_u(u0s)

    def evolve_packed(self, u_dev: torch.Tensor, t0: float, tf: float, h_init: Optional[float] = None,
                      max_steps: int = 200_000, max_launches: int = 50) -> np.ndarray:
        """Advance the packed state in place from t0 to tf; returns the state records.

        ``h_init`` defaults to (tf - t0)/100 and is clamped to the span, as the
        reference's evolve does (solveras.py:614-621); constant-step methods need it."""
        if h_init is None:
            if not self.adaptive:
                raise ValueError("constant-step methods need h_init")
            h_init = (tf - t0) / 100.0
        h = h_init
        if self.adaptive and t0 + h > tf:
            h = tf - t0
        if not self.adaptive and t0 + h > tf:
            raise ValueError("Step size h must be <= (tf - t0); reduce h or extend tf.")
        try:
            self.state = self.engine.evolve(u_dev, t0, tf, h, max_steps=max_steps, max_launches=max_launches)
        except EvolveBoundError as ex:
            self.state = ex.state
            raise
        self._schedule_from(self.state)
        return self.state

    def _schedule_from(self, st: np.ndarray) -> None:
        if self.engine.schedule == "history":
            self.engine.reorder_by_cost(st["attempts"])

    def evolve_graph(self, u_dev: torch.Tensor, u0_dev: torch.Tensor, t0: float, tf: float,
                     h_init: Optional[float] = None, max_steps: int = 200_000, max_launches: int = 50) -> np.ndarray:
        """evolve_packed from u0_dev into u_dev with the launch replayed from a captured CUDA
        graph (the copy of the initial state, the state reset and every class kernel);
        instances the launch bound paused are resumed with ordinary launches."""
        if h_init is None:
            if not self.adaptive:
                raise ValueError("constant-step methods need h_init")
            h_init = (tf - t0) / 100.0
        h = tf - t0 if (self.adaptive and t0 + h_init > tf) else h_init
        eng = self.engine
        eng.graph_launch(u_dev, u0_dev, t0, tf, h, max_steps=max_steps)
        st = eng.get_state()
        paused = (nat.RK_ST_SNAP_FULL, nat.RK_ST_ITER_CAP)
        for _ in range(max_launches - 1):
            resume = np.isin(st["status"], paused)
            if not np.any(resume):
                break
            st["snap_count"] = 0
            st["status"] = np.where(resume, nat.RK_ST_RUNNING, st["status"])
            eng.put_state(st)
            eng.launch(u_dev, nat.RK_RUN_EVOLVE, max_steps=max_steps)
            st = eng.get_state()
        else:
            if np.any(np.isin(st["status"], paused)):
                self.state = st
                raise EvolveBoundError(f"evolve did not reach tf within {max_launches} launches", st)
        self.state = st
        self._schedule_from(st)
        return st

    def evolve(self, u0s: Sequence, t0: float, tf: float, h_init: Optional[float] = None, **bounds):
        """Evolve all instances; returns the list of final spectra (device tensors).
        ``max_steps`` (accepted steps per launch) and ``max_launches`` bound the run."""
        u = self.pack(u0s)
        self.evolve_packed(u, t0, tf, h_init, **bounds)
        return self.engine.unpack_u(u)

    def stats(self) -> dict:
        """Per-instance counters and outcome of the last evolve."""
        st = self.state
        if st is None:
            raise RuntimeError("no evolve has run yet")
        return {
            "status": st["status"].copy(),
            "t": st["t"].copy(),
            "steps": st["steps"].copy(),
            "attempts": st["attempts"].copy(),
            "rejects": st["rejects"].copy(),
            "nl_evals": st["nl_evals"].copy(),
            "coeff_updates": st["coeff_updates"].copy(),
            "modes": self.engine.ms.copy(),
        }

    def mode_steps(self) -> int:
        """sum_i m_i x accepted_steps_i of the last evolve (the throughput numerator)."""
        st = self.state
        return int(np.sum(self.engine.ms * st["steps"]))
