"""Execution backend of the solver classes: the fused device path for a diagonal
operator with a built-in nonlinearity."""

from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .engine import DiagEnsemble, snapshot_views
from .models import BuiltinNL


def _to_output(t: torch.Tensor, like):
    if isinstance(like, torch.Tensor):
        return t.clone()
    return t.detach().cpu().numpy().copy()


class DiagBackend:
    """One-instance ensemble kept alive across calls, so the coefficient cache and the
    controller state (accept flag, h of the cached coefficients) persist like the
    attributes of a reference solver object."""

    def __init__(self, solver, method: str):
        nl = solver.nl_func
        if not isinstance(nl, BuiltinNL):
            raise NotImplementedError(
                "nl_func must be a built-in nonlinearity from rkstiff_gb300.models (fused device kernel); "
                "arbitrary callables are not supported on this path")
        opts = solver.device_options
        self.solver = solver
        self.ens = DiagEnsemble(method, [solver.lin_op], nl.kind, nl.coef, None if nl.kx is None else [nl.kx],
                                [nl.n], precision=opts.precision, config=getattr(solver, "config", None),
                                etd_config=getattr(solver, "etd_config", None), device=opts.device,
                                threads=opts.threads)
        self.snap_cap = max(1, int(opts.snap_cap))
        self.reset()

    def reset(self):
        self.st = self.ens.fresh_state(0.0, np.inf, 0.0)

    def _sync_config(self):
        self.ens.set_config(getattr(self.solver, "config", None), getattr(self.solver, "etd_config", None))

    def evolve(self, u, t0, tf, h, store_data, store_freq):
        """Device evolve; appends snapshots to solver.t / solver.u; returns (u_final, status)."""
        self._sync_config()
        s = self.solver
        u_dev = self.ens.pack_u([u])

        def on_snaps(st, snap_u, snap_t):
            ts, us = snapshot_views(self.ens, st, snap_u, snap_t, 0)
            for tt, uu in zip(ts, us):
                s.t.append(float(tt))
                s.u.append(_to_output(uu, u))

        freq = int(store_freq) if store_data else 0
        if store_data and freq <= 0:
            raise ValueError("store_freq must be a positive integer")
        opts = s.device_options
        if freq > 0 and (opts.stream_snapshots or opts.snapshot_file):
            writer = None
            if opts.snapshot_file:
                from .snapshots import NpzSnapshotWriter

                writer = NpzSnapshotWriter(opts.snapshot_file)
                # the initial state the solver recorded goes to the file as well
                writer.append(s.t[-1], s.u.pop())
            as_tensor = isinstance(u, torch.Tensor)

            def sink(inst, tt, step, uu):
                s.t.append(tt)
                if writer is not None:
                    writer.append(tt, uu)
                else:
                    s.u.append(torch.from_numpy(uu).to(u.device) if as_tensor else uu)

            try:
                st = self.ens.evolve_stream(u_dev, t0, tf, h, freq, sink)
            finally:
                if writer is not None:
                    writer.close()
            self.st = st
            return _to_output(u_dev, u), int(st["status"][0])
        st = self.ens.evolve(u_dev, t0, tf, h, store_freq=freq, snap_cap=self.snap_cap, on_snapshots=on_snaps)
        self.st = st
        return _to_output(u_dev, u), int(st["status"][0])

    def step(self, u, h):
        self._sync_config()
        u_dev = self.ens.pack_u([u])
        st = self.st
        st["t"] = 0.0
        st["tf"] = np.inf
        st["h"] = h
        st["status"] = nat.RK_ST_RUNNING
        st["snap_count"] = 0
        self.ens.put_state(st)
        self.ens.launch(u_dev, nat.RK_RUN_STEP)
        self.st = self.ens.get_state()
        return _to_output(u_dev, u), int(self.st["status"][0])

    @property
    def counters(self):
        st = self.st
        return {k: int(st[k][0]) for k in ("steps", "attempts", "rejects", "nl_evals", "coeff_updates")}


class DenseBackend:
    """One-instance dense ensemble (rkstiff_gb300.dense, per-instance controller) behind a
    solver object with a 2-D lin_op: ETD35, ETD34 or IF34 stepped in the eigenbasis with FP32
    states and 3xTF32 tensor-core basis changes, under the reference's controller."""

    @staticmethod
    def takes(solver) -> bool:
        """ETD35, ETD34 or IF34, FP32, the built-in Allen-Cahn nonlinearity, n <= 128."""
        from .models import BuiltinNL

        nl = solver.nl_func
        return (solver._method_name in ("ETD35", "ETD34", "IF34") and solver.device_options.precision == "fp32"
                and isinstance(nl, BuiltinNL) and nl.kind == nat.RK_NL_ALLEN_CAHN
                and tuple(solver.lin_op.shape)[0] <= nat.RK_DENSE_NMAX)

    def __init__(self, solver, method: str):
        from .dense import DenseEnsemble

        if method not in ("ETD35", "ETD34", "IF34"):
            raise NotImplementedError(f"{method}: the dense (2-D lin_op) tensor-core path implements ETD35, ETD34, IF34")
        opts = solver.device_options
        self.solver = solver
        # diagonalize=True: the error vector in the eigenbasis, as the reference's
        # diagonalized forms return it (etd35.py:495, etd34.py:303, if34.py:195); otherwise in
        # physical space (etd35.py:719, etd34.py:435, if34.py:253)
        basis = "eigen" if getattr(solver, "diagonalize", False) else "physical"
        self.ens = DenseEnsemble(solver.lin_op, solver.nl_func, 1, config=getattr(solver, "config", None),
                                 etd_config=getattr(solver, "etd_config", None), device=opts.device,
                                 err_basis=basis, method=method)
        self.reset()

    def reset(self):
        self.st = {"accept": np.zeros(1, np.int32), "h_used": np.zeros(1), "h_suggest": np.zeros(1),
                   "steps": np.zeros(1, np.int64), "attempts": np.zeros(1, np.int64), "rejects": np.zeros(1, np.int64),
                   "nl_evals": np.zeros(1, np.int64), "coeff_updates": np.zeros(1, np.int64)}
        self._dstate = None

    def _sync_config(self):
        self.ens.config = getattr(self.solver, "config", None) or self.ens.config
        self.ens.etd_config = getattr(self.solver, "etd_config", None) or self.ens.etd_config

    def _record(self, dst, h_used):
        for k in ("steps", "attempts", "rejects", "nl_evals", "coeff_updates", "accept"):
            self.st[k][0] = dst[k][0]
        self.st["h_used"][0] = h_used
        self.st["h_suggest"][0] = dst["h_suggest"][0]

    @staticmethod
    def _out(u_dev, like):
        v = u_dev[0].detach()
        if isinstance(like, torch.Tensor):
            return v.clone()
        return v.cpu().numpy().astype(np.float64).astype(np.complex128)

    def evolve(self, u, t0, tf, h, store_data, store_freq):
        self._sync_config()
        s = self.solver
        ens = self.ens
        u_dev = ens.pack_u(np.asarray(u)[None, :] if not isinstance(u, torch.Tensor) else u.reshape(1, -1))
        if store_data and int(store_freq) <= 0:
            raise ValueError("store_freq must be a positive integer")
        st = ens.fresh_state(t0, tf, h)
        ens.put_state(st)
        if not store_data:
            dst = ens.run(u_dev, 10_000_000)
        else:
            freq = int(store_freq)
            steps = 0
            while True:
                dst = ens.run(u_dev, 1)
                if int(dst["steps"][0]) > steps:
                    steps = int(dst["steps"][0])
                    if steps % freq == 0:
                        s.t.append(float(dst["t"][0]))
                        s.u.append(self._out(u_dev, u))
                if int(dst["status"][0]) != nat.RK_ST_RUNNING:
                    break
        self._dstate = dst
        self._record(dst, 0.0)
        return self._out(u_dev, u), int(dst["status"][0])

    def step(self, u, h):
        """One accepted step with retries (solveras.py:379-410)."""
        self._sync_config()
        ens = self.ens
        u_dev = ens.pack_u(np.asarray(u)[None, :] if not isinstance(u, torch.Tensor) else u.reshape(1, -1))
        ens.put_state(ens.fresh_state(0.0, np.inf, h))
        while True:
            dst = ens.run(u_dev, 1)
            if int(dst["steps"][0]) >= 1 or int(dst["status"][0]) != nat.RK_ST_RUNNING:
                break
        self._dstate = dst
        self._record(dst, float(dst["t"][0]))  # t started at 0
        return self._out(u_dev, u), int(dst["status"][0])

    @property
    def counters(self):
        return {k: int(self.st[k][0]) for k in ("steps", "attempts", "rejects", "nl_evals", "coeff_updates")}
