"""Execution backends for a user-supplied nonlinearity: on a diagonal operator
(``CallableBackend``) and on a dense one stepped in its eigenbasis (``EigenBackend``).

The reference takes any callable ``nl_func`` (rkstiff/solver.py:104-115).  Here it must be a
device-side torch callable: it receives the stage vector as a 1-D complex tensor on the
solver's device (complex128 for FP64, complex64 for FP32) and returns one of the same shape.
Between its calls the stepping runs on the device: coefficients by ``rk_coeffs`` when h
changes, every stage combination of the method's ``_update_stages`` by one ``rk_combine``
pass, the embedded error test by ``rk_error_s``.  The accept/reject rule
(solveras.py:457-554) runs on the host on the one scalar s read back per attempt.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _native as nat

# coefficient indices (include/rkstiff_gb300.h layouts; csrc/rk_coeffs.cuh)
(E14, E12, E34, E35_E, A21, A31, A32, A41, A43, A51, A52, A54, A61, A62, A63, A65, A71, A73, A74, A75,
 A76) = range(21)
(E34_E, E34_E2, B21, B31, B32, B41, B43, B51, B52, B54) = range(10)
(IF_E, IF_E2) = range(2)
(DP_E15, DP_E310, DP_E45, DP_E89, DP_E, D21, D31, D32, D41, D42, D43, D51, D52, D53, D54, D61, D62, D63, D64, D65,
 D71, D73, D74, D75, R1, R3, R4, R5) = range(28)

Q = {"ETD35": 4, "ETD34": 4, "IF34": 4, "IF45DP": 5}
FSAL = {"IF34", "ETD34", "IF45DP", "ETD4", "ETD5", "IF4"}
MAX_LOOPS, MAX_S, MIN_S = 50, 4.0, 0.25


class CallableBackend:
    """One solver's device stepping loop around a torch nonlinearity (diagonal lin_op)."""

    def __init__(self, solver, method: str, lin=None):
        """``lin``: the diagonal the coefficients are built from (default: solver.lin_op)."""
        nl = solver.nl_func
        if not callable(nl):
            raise TypeError("nl_func must be callable")
        opts = solver.device_options
        self.solver = solver
        self.method_name = method
        self.method = nat.METHOD_IDS[method]
        self.lib = nat.load()
        self.device = torch.device(opts.device) if opts.device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self.prec = nat.RK_FP64 if opts.precision == "fp64" else nat.RK_FP32
        lin = np.asarray(solver.lin_op if lin is None else lin)
        if lin.ndim != 1:
            raise NotImplementedError("the callable-nonlinearity path takes a diagonal (1-D) lin_op")
        self.m = int(lin.shape[0])
        self.coef_complex = 1 if np.iscomplexobj(lin) else 0
        self.cdtype = torch.complex128 if self.prec == nat.RK_FP64 else torch.complex64
        rdtype = torch.float64 if self.prec == nat.RK_FP64 else torch.float32
        self.lin_dev = torch.as_tensor(lin.astype(np.complex128), device=self.device).contiguous()
        ncoef = int(self.lib.rk_num_coeffs(self.method))
        self.C = torch.zeros(ncoef * self.m, dtype=self.cdtype if self.coef_complex else rdtype, device=self.device)
        self._cptr = [self.C[c * self.m:(c + 1) * self.m].data_ptr() for c in range(ncoef)]
        self.s_dev = torch.zeros(1, dtype=torch.float64, device=self.device)
        self.adaptive = method in Q
        self._contour_at_zero = False  # the eigenbasis backend may take the reference's matrix contour
        self.reset()

    # -- bookkeeping ------------------------------------------------------------------
    def reset(self):
        self.hc = None
        self.st = {k: np.zeros(1, np.int64) for k in ("steps", "attempts", "rejects", "nl_evals", "coeff_updates")}
        self.st.update({"accept": np.zeros(1, np.int32), "h_used": np.zeros(1), "h_suggest": np.zeros(1)})

    @property
    def counters(self):
        return {k: int(self.st[k][0]) for k in ("steps", "attempts", "rejects", "nl_evals", "coeff_updates")}

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _coeffs(self, h):
        if h == self.hc:  # exact compare, etd35.py:851
            return
        e = getattr(self.solver, "etd_config", None)
        zero = 1 if self._contour_at_zero else 0
        etd = nat.RkEtdConfig(e.modecutoff, e.contour_radius, e.contour_points, zero) if e is not None else \
            nat.RkEtdConfig(0.01, 1.0, 32, zero)
        nat.check(self.lib.rk_coeffs(self.method, self.prec, self.coef_complex, self.m, self.lin_dev.data_ptr(), h,
                                     ctypes.byref(etd), self.C.data_ptr(), self._stream()), "rk_coeffs")
        self.hc = h
        self.st["coeff_updates"][0] += 1

    def _N(self, v):
        self.st["nl_evals"][0] += 1
        r = self.solver.nl_func(v)
        if not isinstance(r, torch.Tensor):
            raise TypeError("nl_func must return a torch tensor on the solver's device (device-side callable)")
        if r.device != self.device or r.shape != v.shape:
            raise ValueError("nl_func must return a tensor of the input's shape on the same device")
        return r.to(self.cdtype).contiguous()

    def _comb(self, terms):
        """sum of w * C[c] * v over (c, w, v); c None: w * v."""
        arr = (nat.RkTerm * len(terms))()
        for i, (c, w, v) in enumerate(terms):
            arr[i].coef = None if c is None else self._cptr[c]
            arr[i].v = v.data_ptr()
            arr[i].w = float(w)
        out = torch.empty(self.m, dtype=self.cdtype, device=self.device)
        nat.check(self.lib.rk_combine(self.prec, self.coef_complex, self.m, arr, len(terms), out.data_ptr(),
                                      self._stream()), "rk_combine")
        return out

    # -- stage programs (_update_stages of each method) ---------------------------------
    def _stages(self, u, N1, h):
        """Returns (unew, err or None, carry or None)."""
        m, N, cb = self.method_name, self._N, self._comb
        if m in ("ETD35", "ETD5"):  # etd35.py:320-345, etd5.py:236-260
            N2 = N(cb([(E14, 1, u), (A21, 1, N1)]))
            N3 = N(cb([(E14, 1, u), (A31, 1, N1), (A32, 1, N2)]))
            N4 = N(cb([(E12, 1, u), (A41, 1, N1), (A43, 1, N3)]))
            N5 = N(cb([(E34, 1, u), (A51, 1, N1), (A52, 1, N2), (A52, -1, N3), (A54, 1, N4)]))
            N6 = N(cb([(E35_E, 1, u), (A61, 1, N1), (A62, 1, N2), (A62, -1.5, N4), (A63, 1, N3), (A65, 1, N5)]))
            unew = cb([(E35_E, 1, u), (A71, 1, N1), (A73, 1, N3), (A74, 1, N4), (A75, 1, N5), (A76, 1, N6)])
            if m == "ETD5":
                return unew, None, N(unew)
            err = cb([(A75, -1, N1), (A75, 4, N3), (A75, -6, N4), (A75, 4, N5), (A75, -1, N6)])
            return unew, err, None
        if m in ("ETD34", "ETD4"):  # etd34.py:182-190, etd4.py:167-174
            N2 = N(cb([(E34_E2, 1, u), (B21, 1, N1)]))
            N3 = N(cb([(E34_E2, 1, u), (B31, 1, N1), (B32, 1, N2)]))
            N4 = N(cb([(E34_E, 1, u), (B41, 1, N1), (B43, 1, N3)]))
            unew = cb([(E34_E, 1, u), (B51, 1, N1), (B52, 1, N2), (B52, 1, N3), (B54, 1, N4)])
            N5 = N(unew)
            if m == "ETD4":
                return unew, None, N5
            return unew, cb([(B54, 1, N4), (B54, -1, N5)]), N5
        if m in ("IF34", "IF4"):  # if34.py:120-130, if4.py:112-121
            N2 = N(cb([(IF_E2, 1, u), (IF_E2, h / 2.0, N1)]))
            N3 = N(cb([(IF_E2, 1, u), (None, h / 2.0, N2)]))
            N4 = N(cb([(IF_E, 1, u), (IF_E2, h, N3)]))
            unew = cb([(IF_E, 1, u), (IF_E, h / 6.0, N1), (IF_E2, h / 3.0, N2), (IF_E2, h / 3.0, N3),
                       (None, h / 6.0, N4)])
            N5 = N(unew)
            if m == "IF4":
                return unew, None, N5
            return unew, cb([(None, h / 6.0, N4), (None, -h / 6.0, N5)]), N5
        # IF45DP, if45dp.py:140-179 (a76, r6, r7 are scalars)
        N2 = N(cb([(DP_E15, 1, u), (D21, 1, N1)]))
        N3 = N(cb([(DP_E310, 1, u), (D31, 1, N1), (D32, 1, N2)]))
        N4 = N(cb([(DP_E45, 1, u), (D41, 1, N1), (D42, 1, N2), (D43, 1, N3)]))
        N5 = N(cb([(DP_E89, 1, u), (D51, 1, N1), (D52, 1, N2), (D53, 1, N3), (D54, 1, N4)]))
        N6 = N(cb([(DP_E, 1, u), (D61, 1, N1), (D62, 1, N2), (D63, 1, N3), (D64, 1, N4), (D65, 1, N5)]))
        unew = cb([(DP_E, 1, u), (D71, 1, N1), (D73, 1, N3), (D74, 1, N4), (D75, 1, N5), (None, 11 * h / 84.0, N6)])
        N7 = N(unew)
        err = cb([(R1, 1, N1), (R3, 1, N3), (R4, 1, N4), (R5, 1, N5), (None, 22 * h / 525.0, N6),
                  (None, -h / 40.0, N7)])
        return unew, err, N7

    def _s(self, unew, err):
        c = self.solver.config
        ctl = nat.RkController(c.epsilon, c.incr_f, c.decr_f, c.safety_f, c.adapt_cutoff, c.minh)
        nat.check(self.lib.rk_error_s(self.prec, self.m, unew.data_ptr(), err.data_ptr(), ctypes.byref(ctl),
                                      Q[self.method_name], self.s_dev.data_ptr(), self._stream()), "rk_error_s")
        return float(self.s_dev.item())

    def _to_dev(self, u):
        if isinstance(u, torch.Tensor):
            return u.to(device=self.device, dtype=self.cdtype).reshape(-1).contiguous()
        return torch.as_tensor(np.asarray(u, dtype=np.complex128).ravel(), device=self.device).to(self.cdtype)

    @staticmethod
    def _out(t, like):
        if isinstance(like, torch.Tensor):
            return t.clone()
        return t.detach().cpu().numpy().astype(np.complex128)

    # -- adaptive ---------------------------------------------------------------------
    def _adaptive_step(self, u, h, N1, accept_prev):
        """The retry loop of solveras.py:379-410.  Returns (unew, h_used, h_suggest, N1 for
        the next step or None, status)."""
        cfg = self.solver.config
        numloops = 0
        while True:
            self._coeffs(h)
            if N1 is None:
                N1 = self._N(u)
            unew, err, carry = self._stages(u, N1, h)
            self.st["attempts"][0] += 1
            s = self._s(unew, err)
            if math.isinf(s) or math.isnan(s) or s < 1.0:
                self.st["rejects"][0] += 1
                self.st["accept"][0] = 0
                h = MIN_S * h if (math.isinf(s) or math.isnan(s)) else min(max(s, MIN_S), cfg.decr_f) * h
                numloops += 1
                if numloops > MAX_LOOPS:
                    return u, h, h, N1, nat.RK_ST_MAX_LOOPS
                if h < cfg.minh:
                    return u, h, h, N1, nat.RK_ST_MIN_STEP
                continue
            self.st["accept"][0] = 1
            s = min(s, MAX_S)
            hs = s * h if s > cfg.incr_f else h
            nxt = carry if self.method_name in FSAL else None  # ETD35 recomputes N(u) after an accept
            return unew, h, hs, nxt, nat.RK_ST_RUNNING

    def evolve(self, u, t0, tf, h, store_data, store_freq):
        s = self.solver
        v = self._to_dev(u)
        freq = int(store_freq) if store_data else 0
        if store_data and freq <= 0:
            raise ValueError("store_freq must be a positive integer")
        t, steps, N1 = t0, 0, None
        status = nat.RK_ST_DONE
        if self.adaptive:
            while t < tf:
                v, h_used, hs, N1, st = self._adaptive_step(v, h, N1, None)
                if st != nat.RK_ST_RUNNING:
                    status = st
                    break
                t += h_used
                steps += 1
                self.st["steps"][0] += 1
                self.st["h_used"][0], self.st["h_suggest"][0] = h_used, hs
                h = tf - t if t + hs > tf else hs
                if freq and steps % freq == 0:
                    s.t.append(t)
                    s.u.append(self._out(v, u))
                if t < tf and t + h == t:
                    status = nat.RK_ST_MIN_STEP
                    break
        else:
            while t < tf:
                self._coeffs(h)
                if N1 is None:
                    N1 = self._N(v)
                v, _, N1 = self._stages(v, N1, h)
                self.st["attempts"][0] += 1
                t += h
                steps += 1
                self.st["steps"][0] += 1
                if freq and steps % freq == 0:
                    s.t.append(t)
                    s.u.append(self._out(v, u))
        return self._out(v, u), status

    def step(self, u, h):
        """One step (adaptive: one accepted step with retries); N1 = N(u) at the start of
        every call."""
        v = self._to_dev(u)
        if self.adaptive:
            v, h_used, hs, _, status = self._adaptive_step(v, h, None, None)
            if status == nat.RK_ST_RUNNING:
                self.st["steps"][0] += 1
                self.st["h_used"][0], self.st["h_suggest"][0] = h_used, hs
            return self._out(v, u), status
        self._coeffs(h)
        v, _, _ = self._stages(v, self._N(v), h)
        self.st["attempts"][0] += 1
        self.st["steps"][0] += 1
        return self._out(v, u), nat.RK_ST_RUNNING


class EigenBackend(CallableBackend):
    """A dense (2-D) lin_op with any method and nonlinearity, stepped in the eigenbasis of
    lin_op = S diag(eig) S^-1 (eig and S^-1 once on the host in FP64, as the reference's
    diagonalized strategies do: etd35.py:348-495, etd34.py:194-304, if34.py:137-199).

    The state is v = S^-1 u; the coefficients are the diagonal ones of h eig (``rk_coeffs``),
    each stage combination one ``rk_combine`` pass, each nonlinearity S^-1 N(S k) with the two
    basis changes as ``rk_cgemv``.  The error test takes the physical state unew = S k and
    either the eigenbasis error vector (``diagonalize=True``, the reference's diagonalized
    result, etd35.py:495) or the physical one S err (``diagonalize=False``).  The second is the
    reference's non-diagonal strategy (etd35.py:498-720, etd34.py:307-436, if34.py:202-254,
    etd4.py:178-309, etd5.py:264-483, if4.py:125-199) in exact arithmetic: its psi-matrices
    are S diag(psi(h eig)) S^-1, which this form applies without forming them (the reference
    forms them by expm and a contour mean of resolvents)."""

    def __init__(self, solver, method: str):
        lin = solver.lin_op
        lin = lin.detach().cpu().numpy() if isinstance(lin, torch.Tensor) else np.asarray(lin)
        if lin.ndim != 2 or lin.shape[0] != lin.shape[1]:
            raise ValueError("a 2-D lin_op must be square")
        diagonalize = bool(getattr(solver, "diagonalize", False))
        eig, S = np.linalg.eig(lin)
        Sinv = np.linalg.inv(S)
        self.cond_S = float(np.linalg.cond(S))
        if not np.isfinite(self.cond_S) or self.cond_S > 1e12:
            raise NotImplementedError(
                f"lin_op's eigenvector matrix has condition number {self.cond_S:.3e}: the device path steps "
                "in the eigenbasis and needs a diagonalizable operator")
        super().__init__(solver, method, lin=eig)
        self.n = int(lin.shape[0])
        self.S = torch.as_tensor(np.ascontiguousarray(S, dtype=np.complex128), device=self.device).to(self.cdtype)
        self.Sinv = torch.as_tensor(np.ascontiguousarray(Sinv, dtype=np.complex128), device=self.device).to(
            self.cdtype)
        self.err_physical = not diagonalize
        dense_psi = getattr(solver.device_options, "dense_psi", "exact")
        if dense_psi not in ("exact", "contour"):
            raise ValueError("dense_psi must be 'exact' or 'contour'")
        # the reference's non-diagonal psi-matrices (a zero-centred contour of resolvents);
        # the diagonalized strategy uses the diagonal rule, as the reference's does
        self._contour_at_zero = dense_psi == "contour" and not diagonalize

    def _mv(self, M, x):
        y = torch.empty(self.n, dtype=self.cdtype, device=self.device)
        nat.check(self.lib.rk_cgemv(self.prec, self.n, M.data_ptr(), x.data_ptr(), y.data_ptr(), self._stream()),
                  "rk_cgemv")
        return y

    def _N(self, v):
        return self._mv(self.Sinv, super()._N(self._mv(self.S, v)))

    def _s(self, unew, err):
        return super()._s(self._mv(self.S, unew), self._mv(self.S, err) if self.err_physical else err)

    def _to_dev(self, u):
        return self._mv(self.Sinv, super()._to_dev(u))

    def _out(self, t, like):
        return CallableBackend._out(self._mv(self.S, t), like)
