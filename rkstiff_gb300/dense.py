"""Dense (non-diagonal) operators on the tensor cores: ETD35 (and, with the per-instance
controller, ETD34 and IF34) for a batch of instances that share one n x n lin_op (n <= 128),
e.g. the Allen-Cahn Chebyshev operator.

The operator is diagonalised once on the host in FP64 (lin_op = S diag(eig) S^-1, real
spectrum; rkstiff/etd35.py:412-420 does the same for its diagonalized form).  Two device
paths, both whole evolve loops on the GPU:

* ``controller="instance"`` (default, ``rk_dense_eig_evolve``): every instance under the
  reference's accept/reject rule with its own h, as a loop of single-instance solvers would
  run; stages in the eigenbasis with per-instance diagonal coefficients, the basis changes
  S k and S^-1 N as 3xTF32 tcgen05 GEMMs, one persistent launch;
* ``controller="lockstep"`` (``rk_dense_evolve``): one h for the batch (an attempt is
  accepted when every instance passes), FP64 psi-matrices rebuilt when h changes, one
  K-concatenated 3xTF32 GEMM per stage.

A one-instance batch follows the reference's controller on either path.
"""

from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np
import torch

from . import _native as nat
from .etd import ETDConfig
from .models import BuiltinNL
from .solveras import SolverConfig


class DenseEnsemble:
    """ETD35, ETD34 or IF34 with a dense ``lin_op`` for ``n_inst`` instances on one device
    (FP32 states, FP64 operator factors, 3xTF32 stage products)."""

    def __init__(self, lin_op, nl_func: BuiltinNL, n_inst: int, config: Optional[SolverConfig] = None,
                 etd_config: Optional[ETDConfig] = None, device=None, method: str = "ETD35",
                 err_basis: str = "physical", controller: str = "instance"):
        """``err_basis``: "physical" forms the embedded error vector in physical space, as the
        reference's non-diagonal ETD35 does (etd35.py:719); "eigen" forms it in the eigenbasis
        (S^-1 applied) with the mask taken from the physical state, as the reference's
        diagonalized ETD35 returns it (etd35.py:495).

        ``controller``: "lockstep" (one h for the batch, ``rk_dense_evolve``: psi-matrices and
        one K-concatenated GEMM per stage) or "instance" (every instance under the reference's
        controller with its own h, ``rk_dense_eig_evolve``: the stages in the eigenbasis with
        per-instance diagonal coefficients, the basis changes as GEMMs).

        ``method``: "ETD35" on either controller; "ETD34" and "IF34" (first same as last:
        N1 of an accepted attempt is its N5) with the instance controller."""
        if err_basis not in ("physical", "eigen"):
            raise ValueError("err_basis must be 'physical' or 'eigen'")
        if controller not in ("lockstep", "instance"):
            raise ValueError("controller must be 'lockstep' or 'instance'")
        self.controller = controller
        self.err_eigen = 1 if err_basis == "eigen" else 0
        methods = ("ETD35", "ETD34", "IF34") if controller == "instance" else ("ETD35",)
        if method not in methods:
            raise NotImplementedError(f"the dense tensor-core path with the {controller} controller "
                                      f"implements {', '.join(methods)}")
        self.method = method
        if not isinstance(nl_func, BuiltinNL) or nl_func.kind != nat.RK_NL_ALLEN_CAHN:
            raise TypeError("the dense path runs the Allen-Cahn nonlinearity (rkstiff_gb300.models.allen_cahn_ops)")
        lin = np.asarray(lin_op)
        if lin.ndim != 2 or lin.shape[0] != lin.shape[1]:
            raise ValueError("lin_op must be a square matrix")
        if np.iscomplexobj(lin):
            if np.max(np.abs(lin.imag)) > 0:
                raise NotImplementedError("the dense path needs a real lin_op")
            lin = lin.real
        lin = lin.astype(np.float64)
        n = lin.shape[0]
        if n > nat.RK_DENSE_NMAX or n != nl_func.n:
            raise ValueError(f"lin_op is {n} x {n}; the dense path takes n <= {nat.RK_DENSE_NMAX} "
                             "matching the nonlinearity")
        w, S = np.linalg.eig(lin)
        if np.iscomplexobj(w):
            if np.max(np.abs(w.imag)) > 1e-12 * max(1.0, np.max(np.abs(w))):
                raise NotImplementedError("the dense path needs an operator with a real spectrum")
            w, S = w.real, S.real
        if not self.err_eigen:
            # eigenvalues in descending order: the stiff modes of every h fill whole 32-row
            # chunks, which balances the per-instance kernel's coefficient rebuilds.  The
            # eigenbasis error vector keeps NumPy's order: the reference masks it by the
            # physical state's index (etd35.py:495 into solveras.py:412-455), so the order
            # of the eigenvectors decides which components count.
            order = np.argsort(-w, kind="stable")
            w, S = w[order], S[:, order]
        Sinv = np.linalg.inv(S)
        self.lib = nat.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.n = n
        self.n_inst = int(n_inst)
        self.config = config or SolverConfig()
        self.etd_config = etd_config or ETDConfig()
        self.cond_S = float(np.linalg.cond(S))
        dev = self.device
        self.eig = torch.as_tensor(w, dtype=torch.float64, device=dev).contiguous()
        self.S = torch.as_tensor(S, dtype=torch.float64, device=dev).contiguous()
        self.Sinv = torch.as_tensor(Sinv, dtype=torch.float64, device=dev).contiguous()
        self.shift = torch.as_tensor(nl_func.shift, dtype=torch.float64, device=dev).contiguous()
        per_instance = controller == "instance"
        nbytes = int(self.lib.rk_dense_eig_work_bytes(self.n_inst) if per_instance
                     else self.lib.rk_dense_work_bytes(self.n_inst))
        # torch's caching allocator returns 512-byte aligned blocks: over-allocate and align
        self._work_buf = torch.empty(nbytes + 1024, dtype=torch.uint8, device=dev)
        base = self._work_buf.data_ptr()
        self.work_ptr = (base + 1023) & ~1023
        self.state_dtype = nat.STATE_DTYPE if per_instance else nat.DENSE_STATE_DTYPE
        self.state_dev = torch.zeros(self.state_dtype.itemsize * (self.n_inst if per_instance else 1),
                                     dtype=torch.uint8, device=dev)
        self.state = None
        self._first = True

    # -- state ------------------------------------------------------------------------
    def fresh_state(self, t0: float, tf: float, h: float) -> np.ndarray:
        """Records of a run from t0 (one for the lockstep batch, one per instance otherwise)."""
        st = np.zeros(self.n_inst if self.controller == "instance" else 1, dtype=self.state_dtype)
        st["t"], st["tf"], st["h"], st["h_coeff"] = t0, tf, h, np.nan
        st["status"] = nat.RK_ST_RUNNING
        if self.controller == "lockstep":
            st["n1_fresh"] = 1
        return st

    def put_state(self, st: np.ndarray) -> None:
        """Install records; the next run starts from the states in ``u``."""
        self.state_dev.copy_(torch.from_numpy(np.ascontiguousarray(st).view(np.uint8).copy()))
        self._first = True

    def get_state(self) -> np.ndarray:
        return self.state_dev.cpu().numpy().view(self.state_dtype).copy()

    def pack_u(self, u0s) -> torch.Tensor:
        """(n_inst, n) FP32 device states from host arrays or tensors."""
        if isinstance(u0s, torch.Tensor):
            u = u0s.to(device=self.device, dtype=torch.float32)
        else:
            arr = np.asarray(u0s)
            if np.iscomplexobj(arr):
                arr = arr.real
            u = torch.as_tensor(np.ascontiguousarray(arr, dtype=np.float32), device=self.device)
        u = u.reshape(self.n_inst, self.n).contiguous()
        return u

    # -- run --------------------------------------------------------------------------
    def run(self, u: torch.Tensor, max_attempts: int) -> np.ndarray:
        """Continue the current state for at most ``max_attempts`` attempts (per instance with
        the instance controller); u in place."""
        if u.dtype != torch.float32 or u.device != self.device or not u.is_contiguous() or u.numel() != self.n_inst * self.n:
            raise ValueError("u must be a contiguous FP32 (n_inst, n) tensor on the ensemble's device")
        per_instance = self.controller == "instance"
        b = nat.RkDenseEigBatch() if per_instance else nat.RkDenseBatch()
        b.method = {"ETD35": nat.RK_ETD35, "ETD34": nat.RK_ETD34, "IF34": nat.RK_IF34}[self.method]
        b.n = self.n
        b.n_inst = self.n_inst
        b.nl_kind = nat.RK_NL_ALLEN_CAHN
        b.err_eigen = self.err_eigen
        b.eig, b.S, b.Sinv, b.shift = (t.data_ptr() for t in (self.eig, self.S, self.Sinv, self.shift))
        b.u = u.data_ptr()
        b.work = self.work_ptr
        b.state = self.state_dev.data_ptr()
        c = self.config
        b.ctl = nat.RkController(c.epsilon, c.incr_f, c.decr_f, c.safety_f, c.adapt_cutoff, c.minh)
        e = self.etd_config
        b.etd = nat.RkEtdConfig(e.modecutoff, e.contour_radius, e.contour_points, 0)
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device)
            if per_instance:
                b.first = 1 if self._first else 0
                b.max_attempts = int(min(max_attempts, 2**31 - 1))
                nat.check(self.lib.rk_dense_eig_evolve(ctypes.byref(b), stream.cuda_stream), "rk_dense_eig_evolve")
                self._first = False
            else:
                b.max_attempts = int(max_attempts)
                nat.check(self.lib.rk_dense_evolve(ctypes.byref(b), stream.cuda_stream), "rk_dense_evolve")
        self.state = self.get_state()
        if per_instance and np.any(self.state["status"] == nat.RK_ST_WAIT_TIMEOUT):
            raise nat.NativeError("rk_dense_eig_evolve: a device wait timed out")
        return self.state

    def evolve(self, u0s, t0: float, tf: float, h_init: Optional[float] = None,
               max_attempts: int = 1_000_000) -> torch.Tensor:
        """All instances from t0 to tf; returns the (n_inst, n) FP32 final states."""
        if h_init is None:
            h_init = (tf - t0) / 100.0  # solveras.py:614-621
        h = tf - t0 if t0 + h_init > tf else h_init
        u = self.pack_u(u0s)
        self.put_state(self.fresh_state(t0, tf, h))
        st = self.run(u, max_attempts)
        if np.any(st["status"] == nat.RK_ST_RUNNING):
            raise RuntimeError(f"dense evolve did not reach tf within {max_attempts} attempts")
        return u

    def stats(self) -> dict:
        """Counters of the last run: scalars for the lockstep batch; for the instance
        controller the per-instance arrays plus their totals (``*_total``)."""
        st = self.state
        if st is None:
            raise RuntimeError("no evolve has run yet")
        keys = ("t", "h", "status", "steps", "attempts", "rejects", "nl_evals", "coeff_updates")
        if self.controller == "lockstep":
            return {k: st[k][0].item() for k in keys}
        out = {k: st[k].copy() for k in keys}
        for k in ("steps", "attempts", "rejects", "nl_evals", "coeff_updates"):
            out[k + "_total"] = int(st[k].sum())
        return out


def _main(argv=None) -> None:
    """python -m rkstiff_gb300.dense [--instances 8192] [--tf 70]: the Allen-Cahn batch of
    rkstiff_gb300.workloads on this GPU, timed (used for profiling the dense kernels)."""
    import argparse
    import json
    import time

    from . import workloads

    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=8192)
    ap.add_argument("--tf", type=float, default=70.0)
    ap.add_argument("--epsilon", type=float, default=1e-4)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--controller", choices=["lockstep", "instance"], default="instance")
    ap.add_argument("--method", choices=["ETD35", "ETD34", "IF34"], default="ETD35")
    args = ap.parse_args(argv)
    lin, nl, w0 = workloads.allen_cahn_batch(args.instances, args.seed)
    ens = DenseEnsemble(lin, nl, args.instances, config=SolverConfig(epsilon=args.epsilon),
                        controller=args.controller, method=args.method)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ens.evolve(w0, 0.0, args.tf)
    torch.cuda.synchronize()
    st = ens.stats()
    if args.controller == "instance":
        st = {k: v for k, v in st.items() if k.endswith("_total")}
        st["status_max"] = int(ens.state["status"].max())
    st["seconds"] = time.perf_counter() - t0
    print(json.dumps(st))


if __name__ == "__main__":
    _main()
