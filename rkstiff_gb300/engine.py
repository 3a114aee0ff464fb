"""Device engine: packs a batch of diagonal-operator instances into device arrays and
drives the persistent evolve kernel (``rk_evolve`` of the C ABI).

One ``DiagEnsemble`` holds, on one CUDA device:

* the operators (complex128, concatenated by mode offset) and wavenumbers (float64),
* the per-instance scratch ("slab": the coefficient block, u/unew and the stage arrays),
* the per-instance controller state records (``STATE_DTYPE``),
* the processing order (largest grid first; within a grid size, longest first by the
  previous evolve's attempt counts, so the tail of a persistent launch is short).

The solver classes use a one-instance ensemble; ``rkstiff_gb300.ensemble`` exposes the
batched form directly.
"""

from __future__ import annotations

import ctypes
import math
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as nat

_TWIDDLES = {}


def _dev(device) -> torch.device:
    if device is None:
        if not torch.cuda.is_available():
            raise RuntimeError("rkstiff_gb300 needs a CUDA device; none is available")
        return torch.device("cuda", torch.cuda.current_device())
    d = torch.device(device)
    if d.type != "cuda":
        raise ValueError(f"rkstiff_gb300 runs on CUDA devices only, got {d}")
    if d.index is None:
        d = torch.device("cuda", torch.cuda.current_device())
    return d


def stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def twiddles(device: torch.device, precision: int) -> torch.Tensor:
    """exp(-2 pi i k / RK_TW_N) tables, built once per device by rk_fill_twiddles."""
    key = (device.index, precision)
    if key not in _TWIDDLES:
        lib = nat.load()
        tw64 = torch.empty(nat.RK_TW_N, dtype=torch.complex128, device=device)
        tw32 = torch.empty(nat.RK_TW_N, dtype=torch.complex64, device=device)
        with torch.cuda.device(device):
            nat.check(lib.rk_fill_twiddles(tw64.data_ptr(), tw32.data_ptr(), stream_handle(device)),
                      "rk_fill_twiddles")
        _TWIDDLES[(device.index, nat.RK_FP64)] = tw64
        _TWIDDLES[(device.index, nat.RK_FP32)] = tw32
    return _TWIDDLES[key]


def precision_id(precision) -> int:
    p = str(precision).lower()
    if p in ("fp64", "float64", "double", "complex128"):
        return nat.RK_FP64
    if p in ("fp32", "float32", "float", "complex64"):
        return nat.RK_FP32
    raise ValueError(f"precision must be 'fp64' or 'fp32', got {precision!r}")


def complex_dtype(prec: int) -> torch.dtype:
    return torch.complex128 if prec == nat.RK_FP64 else torch.complex64


def _as_numpy_1d(a, dtype=None) -> np.ndarray:
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    a = np.asarray(a)
    if dtype is not None:
        a = a.astype(dtype, copy=False)
    return np.ascontiguousarray(a).ravel()


class DiagEnsemble:
    """Independent instances u_t = L u + N(u) with diagonal L and one built-in N kind.

    Parameters
    ----------
    method : str         one of IF34, ETD35, ETD34, IF45DP, ETD4, ETD5, IF4
    lin_ops : sequence   per-instance 1-D operators (length m_i)
    nl_kind, nl_coef     built-in nonlinearity (RK_NL_*) and its constant
    kxs : sequence|None  per-instance wavenumbers (RK_NL_UUX)
    ns : sequence        per-instance grid sizes (powers of two)
    """

    def __init__(self, method: str, lin_ops: Sequence, nl_kind: int, nl_coef: float, kxs: Optional[Sequence],
                 ns: Sequence[int], precision="fp64", config=None, etd_config=None, device=None, threads: int = 0,
                 complex_operator: Optional[bool] = None):
        self.lib = nat.load()
        self.device = _dev(device)
        self.method_name = method
        self.method = nat.METHOD_IDS[method]
        self.prec = precision_id(precision)
        self.nl_kind = int(nl_kind)
        self.nl_coef = float(nl_coef)
        self.threads = int(threads)
        ns = [int(n) for n in ns]
        n_inst = len(ns)
        if len(lin_ops) != n_inst:
            raise ValueError("one operator per instance is required")
        limit = 4096 if self.prec == nat.RK_FP64 else 8192
        for n in ns:
            if n < 4 or n & (n - 1) or n > limit:
                raise ValueError(f"grid size {n} must be a power of two in [4, {limit}] for this precision")
        ms = [(n // 2 + 1) if self.nl_kind == nat.RK_NL_UUX else n for n in ns]
        lins = []
        for L, m in zip(lin_ops, ms):
            a = _as_numpy_1d(L)
            if a.shape[0] != m:
                raise ValueError(f"operator has {a.shape[0]} modes, expected {m}")
            lins.append(a)
        if complex_operator is None:
            complex_operator = any(np.iscomplexobj(a) for a in lins)
        self.coef_complex = 1 if complex_operator else 0
        self.ns = np.array(ns, dtype=np.int32)
        self.ms = np.array(ms, dtype=np.int64)
        self.n_inst = n_inst
        self.mode_off = np.zeros(n_inst, dtype=np.int64)
        if n_inst > 1:
            self.mode_off[1:] = np.cumsum(self.ms)[:-1]
        self.total_m = int(self.ms.sum())
        dev = self.device
        lin_all = np.concatenate([a.astype(np.complex128) for a in lins])
        self.lin_dev = torch.from_numpy(lin_all).to(dev)
        if self.nl_kind == nat.RK_NL_UUX:
            if kxs is None or len(kxs) != n_inst:
                raise ValueError("the u*u_x nonlinearity needs one wavenumber array per instance")
            kx_all = np.concatenate([_as_numpy_1d(k, np.float64) for k in kxs])
            if kx_all.shape[0] != self.total_m:
                raise ValueError("wavenumber arrays must have m_i = n_i/2 + 1 entries")
            self.kx_dev = torch.from_numpy(kx_all).to(dev)
        else:
            self.kx_dev = None
        self.n_dev = torch.from_numpy(self.ns).to(dev)
        self.off_dev = torch.from_numpy(self.mode_off).to(dev)
        # largest grids first; instances of equal n form one class (one kernel each)
        order = np.argsort(-self.ns, kind="stable").astype(np.int32)
        self._size_order = order
        self.order_dev = torch.from_numpy(order).to(dev)
        # "history": after each evolve the queue of every class is reordered longest-first
        # by that evolve's attempt counts (reorder_by_cost); "size": index order within a class
        self.schedule = "history"
        sorted_n = self.ns[order]
        bounds = [0] + [i for i in range(1, n_inst) if sorted_n[i] != sorted_n[i - 1]] + [n_inst]
        self.class_n = np.ascontiguousarray([int(sorted_n[b]) for b in bounds[:-1]], dtype=np.int32)
        self.class_start = np.ascontiguousarray(bounds, dtype=np.int64)
        self.class_threads = None  # per-class threads (np.int32) or None: library default
        self.class_place = None    # per-class placement (np.int32) or None: library default
        self.class_groups = None   # per-class instance groups per block (np.int32) or None
        self.coef_blocks = 1
        self.ladder = 0
        self._alloc_slab()
        self.state_dev = torch.zeros(n_inst * nat.STATE_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        self.queue = torch.zeros(max(1, len(self.class_n)), dtype=torch.int32, device=dev)
        self.tw = twiddles(dev, self.prec)
        self.cdtype = complex_dtype(self.prec)
        self.set_config(config, etd_config)
        self.launches = 0          # rk_evolve calls issued by this ensemble
        self.kernel_launches = 0   # evolve-kernel launches (one per non-empty grid-size class)
        self.record_events = False  # when True, (start, end) CUDA events bracket each launch
        self.events = []
        self.attempt_log = None     # float32 device tensor [n_inst, log_cap, RK_LOG_FIELDS] or None
        self.log_cap = 0
        self.mlp = None             # packed learned-controller buffer (uint8 device tensor) or None
        self.mlp_target = 1.25

    def _alloc_slab(self) -> None:
        sizes = [int(self.lib.rk_slab_bytes_blocks(self.method, self.prec, self.coef_complex, int(m),
                                                   int(self.coef_blocks))) for m in self.ms]
        offs = np.zeros(self.n_inst, dtype=np.int64)
        acc = 0
        for i, sz in enumerate(sizes):
            offs[i] = acc
            acc += (sz + 255) // 256 * 256
        self.slab_bytes = acc
        self.slab = torch.empty(max(acc, 256), dtype=torch.uint8, device=self.device)
        self.slab_off_dev = torch.from_numpy(offs).to(self.device)

    def set_coef_cache(self, blocks: int, ladder: bool = False) -> None:
        """Keep ``blocks`` coefficient blocks per instance keyed by their exact h (1: the
        reference's single-entry cache) and, with ``ladder``, put the learned controller's
        step sizes on the 2^(1/16) ladder (rk_batch.coef_blocks / ladder); a change of
        ``blocks`` reallocates the scratch, so the next launch rebuilds the coefficients."""
        blocks = int(blocks)
        if not 1 <= blocks <= 4:
            raise ValueError("blocks must be in 1..4")
        if blocks != self.coef_blocks:
            self.coef_blocks = blocks
            self._alloc_slab()
        self.ladder = 1 if ladder else 0

    # -- configuration ----------------------------------------------------------------
    def set_config(self, config=None, etd_config=None):
        c = config
        self.ctl = nat.RkController(
            epsilon=getattr(c, "epsilon", 1e-4), incr_f=getattr(c, "incr_f", 1.25),
            decr_f=getattr(c, "decr_f", 0.85), safety_f=getattr(c, "safety_f", 0.8),
            adapt_cutoff=getattr(c, "adapt_cutoff", 0.01), minh=getattr(c, "minh", 1e-16))
        e = etd_config
        self.etd = nat.RkEtdConfig(modecutoff=getattr(e, "modecutoff", 0.01),
                                   contour_radius=getattr(e, "contour_radius", 1.0),
                                   contour_points=int(getattr(e, "contour_points", 32)), contour_at_zero=0)

    # -- state records ----------------------------------------------------------------
    def fresh_state(self, t0, tf, h) -> np.ndarray:
        st = np.zeros(self.n_inst, dtype=nat.STATE_DTYPE)
        st["t"] = t0
        st["tf"] = tf
        st["h"] = h
        st["h_coeff"] = np.nan
        st["h_used"] = np.nan
        st["h_suggest"] = np.nan
        st["s_last"] = np.nan
        st["status"] = nat.RK_ST_RUNNING
        return st

    def reorder_by_cost(self, cost) -> None:
        """Reorder the work queue of every grid-size class longest-first by ``cost`` (one
        value per instance, e.g. the attempts of the previous evolve): a persistent launch
        then starts the longest instances first and ends on short ones, which shortens the
        tail where a class's last instances run while its other blocks have exited.  Each
        instance's arithmetic does not depend on the order, so results are unchanged."""
        cost = np.asarray(cost)
        if cost.shape != (self.n_inst,):
            raise ValueError("one cost per instance is required")
        order = self._size_order.copy()
        for c in range(len(self.class_n)):
            a, b = int(self.class_start[c]), int(self.class_start[c + 1])
            idx = order[a:b]
            order[a:b] = idx[np.argsort(-cost[idx], kind="stable")]
        self.order_dev.copy_(torch.from_numpy(order))

    def reset_order(self) -> None:
        self.order_dev.copy_(torch.from_numpy(self._size_order))

    def put_state(self, st: np.ndarray) -> None:
        self.state_dev.copy_(torch.from_numpy(np.ascontiguousarray(st).view(np.uint8)))

    def get_state(self) -> np.ndarray:
        return self.state_dev.cpu().numpy().view(nat.STATE_DTYPE).copy()

    # -- state vectors ----------------------------------------------------------------
    def pack_u(self, us: Sequence) -> torch.Tensor:
        """Concatenate per-instance spectra into one device tensor of the working dtype."""
        parts = []
        for u, m in zip(us, self.ms):
            if isinstance(u, torch.Tensor):
                t = u.to(device=self.device, dtype=self.cdtype).reshape(-1)
            else:
                t = torch.from_numpy(np.ascontiguousarray(np.asarray(u, dtype=np.complex128)).ravel()).to(
                    device=self.device, dtype=self.cdtype)
            if t.shape[0] != m:
                raise ValueError(f"state has {t.shape[0]} modes, expected {int(m)}")
            parts.append(t)
        return torch.cat(parts) if len(parts) > 1 else parts[0].clone()

    def unpack_u(self, u_dev: torch.Tensor) -> List[torch.Tensor]:
        return [u_dev[int(o):int(o) + int(m)] for o, m in zip(self.mode_off, self.ms)]

    # -- launch -----------------------------------------------------------------------
    def launch(self, u_dev: torch.Tensor, run_mode: int, store_freq: int = 0, snap_cap: int = 0,
               snap_u: Optional[torch.Tensor] = None, snap_t: Optional[torch.Tensor] = None,
               max_steps: int = 200_000, ring=None) -> None:
        if u_dev.dtype != self.cdtype or u_dev.device != self.device or not u_dev.is_contiguous():
            raise ValueError("state tensor must be a contiguous device tensor of the working dtype")
        b = nat.RkBatch()
        b.method = self.method
        b.precision = self.prec
        b.coef_complex = self.coef_complex
        b.nl_kind = self.nl_kind
        b.nl_coef = self.nl_coef
        b.n_inst = self.n_inst
        b.n_max = int(self.ns.max())
        b.n = self.n_dev.data_ptr()
        b.mode_off = self.off_dev.data_ptr()
        b.order = self.order_dev.data_ptr()
        b.lin_op = self.lin_dev.data_ptr()
        b.kx = self.kx_dev.data_ptr() if self.kx_dev is not None else None
        b.u = u_dev.data_ptr()
        b.state = self.state_dev.data_ptr()
        b.slab = self.slab.data_ptr()
        b.slab_off = self.slab_off_dev.data_ptr()
        b.twiddle = self.tw.data_ptr()
        b.queue = self.queue.data_ptr()
        b.store_freq = int(store_freq)
        b.snap_cap = int(snap_cap)
        b.snap_u = snap_u.data_ptr() if snap_u is not None else None
        b.snap_t = snap_t.data_ptr() if snap_t is not None else None
        b.max_steps = int(max_steps)
        b.run_mode = int(run_mode)
        b.threads = self.threads
        b.ctl = self.ctl
        b.etd = self.etd
        b.n_classes = len(self.class_n)
        b.placement = nat.RK_PLACE_AUTO
        b.class_n = self.class_n.ctypes.data
        b.class_start = self.class_start.ctypes.data
        b.class_threads = self.class_threads.ctypes.data if self.class_threads is not None else None
        b.class_place = self.class_place.ctypes.data if self.class_place is not None else None
        b.class_groups = self.class_groups.ctypes.data if self.class_groups is not None else None
        b.attempt_log = self.attempt_log.data_ptr() if self.attempt_log is not None else None
        b.log_cap = int(self.log_cap) if self.attempt_log is not None else 0
        b.mlp = self.mlp.data_ptr() if self.mlp is not None else None
        b.mlp_target = float(self.mlp_target)
        if ring is not None:
            ring.fill_batch(b)
        b.coef_blocks = int(self.coef_blocks)
        b.ladder = int(self.ladder)
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device)
            if self.record_events:
                ev0 = torch.cuda.Event(enable_timing=True)
                ev1 = torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
            nat.check(self.lib.rk_evolve(ctypes.byref(b), stream.cuda_stream), "rk_evolve")
            if self.record_events:
                ev1.record(stream)
                self.events.append((ev0, ev1))
        self.launches += 1
        self.kernel_launches += int(np.count_nonzero(np.diff(self.class_start)))

    def graph_launch(self, u_dev: torch.Tensor, u_src: torch.Tensor, t0, tf, h, max_steps: int = 200_000) -> None:
        """One evolve launch from (u_src, t0, h) as a replay of a captured CUDA graph:
        [u_dev <- u_src, state <- fresh state, rk_evolve (all class kernels)].  The graph is
        captured on the first call for these buffers and parameters and replayed after."""
        key = (u_dev.data_ptr(), u_src.data_ptr(), float(t0), float(tf), float(h), int(max_steps),
               tuple(int(v) for v in (self.class_threads if self.class_threads is not None else ())),
               tuple(int(v) for v in (self.class_groups if self.class_groups is not None else ())),
               tuple(int(v) for v in (self.class_place if self.class_place is not None else ())),
               None if self.mlp is None else self.mlp.data_ptr(), float(self.mlp_target),
               int(self.coef_blocks), int(self.ladder), self.slab.data_ptr(),
               None if self.attempt_log is None else self.attempt_log.data_ptr())
        if getattr(self, "_graph_key", None) != key:
            fresh = torch.from_numpy(np.ascontiguousarray(self.fresh_state(t0, tf, h)).view(np.uint8)).to(self.device)
            # one ordinary launch first: creates the side streams and sets kernel attributes
            u_dev.copy_(u_src)
            self.state_dev.copy_(fresh)
            self.launch(u_dev, nat.RK_RUN_EVOLVE, max_steps=max_steps)
            torch.cuda.synchronize(self.device)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.device(self.device):
                with torch.cuda.graph(g, capture_error_mode="relaxed"):
                    u_dev.copy_(u_src)
                    self.state_dev.copy_(fresh)
                    self.launch(u_dev, nat.RK_RUN_EVOLVE, max_steps=max_steps)
            self.launches -= 1  # the capture pass launched nothing
            self.kernel_launches -= int(np.count_nonzero(np.diff(self.class_start)))
            self._graph, self._graph_fresh, self._graph_key = g, fresh, key
        if self.record_events:
            stream = torch.cuda.current_stream(self.device)
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            self._graph.replay()
            ev1.record(stream)
            self.events.append((ev0, ev1))
        else:
            self._graph.replay()
        self.launches += 1
        self.kernel_launches += int(np.count_nonzero(np.diff(self.class_start)))

    def evolve(self, u_dev: torch.Tensor, t0, tf, h, store_freq: int = 0, snap_cap: int = 0,
               max_steps: int = 200_000, max_launches: int = 50, on_snapshots=None) -> np.ndarray:
        """Run every instance from (t0, h) to tf, relaunching while any instance paused
        (full snapshot buffer, or the per-launch bound of ``max_steps`` accepted steps,
        which keeps every launch finite).  ``on_snapshots(state, snap_u, snap_t)``
        receives each launch's snapshots.  Returns the final state records."""
        st = self.fresh_state(t0, tf, h)
        self.put_state(st)
        snap_u = snap_t = None
        if store_freq > 0:
            snap_cap = max(1, int(snap_cap))
            snap_u = torch.empty(snap_cap * self.total_m, dtype=self.cdtype, device=self.device)
            snap_t = torch.empty(snap_cap * self.n_inst, dtype=torch.float64, device=self.device)
        paused = (nat.RK_ST_SNAP_FULL, nat.RK_ST_ITER_CAP)
        for _ in range(max_launches):
            self.launch(u_dev, nat.RK_RUN_EVOLVE, store_freq, snap_cap, snap_u, snap_t, max_steps)
            st = self.get_state()
            if on_snapshots is not None and store_freq > 0:
                on_snapshots(st, snap_u, snap_t)
            resume = np.isin(st["status"], paused)
            if not np.any(resume):
                return st
            # resume the paused instances; finished or failed ones are skipped by the kernel
            st["snap_count"] = 0
            st["status"] = np.where(resume, nat.RK_ST_RUNNING, st["status"])
            self.put_state(st)
        raise EvolveBoundError(f"evolve did not reach tf within {max_launches} launches of {max_steps} steps",
                               self.get_state())


    def evolve_stream(self, u_dev: torch.Tensor, t0, tf, h, store_freq: int, sink, ring=None, slots: int = 64,
                      max_steps: int = 200_000, max_launches: int = 50) -> np.ndarray:
        """``evolve`` with the snapshots streamed: every ``store_freq`` accepted steps the
        kernel writes the state into a pinned, mapped host ring (``snapshots.SnapshotRing``,
        created here unless given) and the host hands each one to ``sink(inst, t, step,
        u)`` (u a NumPy copy) while the launch runs; a launch ends only at tf, on failure or
        at the ``max_steps`` bound.  Returns the final state records."""
        from .snapshots import SnapshotRing, SnapshotStreamOverrun

        if store_freq <= 0:
            raise ValueError("store_freq must be a positive integer")
        own = ring is None
        if own:
            ring = SnapshotRing(slots, int(self.ms.max()), self.prec)
        try:
            ring.reset()
            st = self.fresh_state(t0, tf, h)
            self.put_state(st)
            for _ in range(max_launches):
                self.launch(u_dev, nat.RK_RUN_EVOLVE, store_freq, 0, None, None, max_steps, ring=ring)
                ev = torch.cuda.Event()
                ev.record(torch.cuda.current_stream(self.device))
                ring.drain(ev.query, self.ms, sink)
                st = self.get_state()
                if np.any(st["status"] == nat.RK_ST_SNAP_FULL):
                    raise SnapshotStreamOverrun("a snapshot writer timed out waiting for the host")
                resume = st["status"] == nat.RK_ST_ITER_CAP
                if not np.any(resume):
                    return st
                st["snap_count"] = 0
                st["status"] = np.where(resume, nat.RK_ST_RUNNING, st["status"])
                self.put_state(st)
            raise EvolveBoundError(f"evolve did not reach tf within {max_launches} launches of {max_steps} steps",
                                   self.get_state())
        finally:
            if own:
                ring.close()


class EvolveBoundError(RuntimeError):
    """An evolve stopped by its launch bound; ``state`` holds the records reached so far
    (paused instances carry RK_ST_ITER_CAP or RK_ST_SNAP_FULL)."""

    def __init__(self, msg: str, state: np.ndarray):
        super().__init__(msg)
        self.state = state


def snapshot_views(ens: DiagEnsemble, st: np.ndarray, snap_u: torch.Tensor, snap_t: torch.Tensor, inst: int):
    """(times, states) written for instance ``inst`` by the last launch."""
    cnt = int(st["snap_count"][inst])
    cap = snap_t.shape[0] // ens.n_inst
    m = int(ens.ms[inst])
    base = cap * int(ens.mode_off[inst])
    ts = snap_t[inst * cap: inst * cap + cnt].cpu().numpy()
    us = [snap_u[base + k * m: base + (k + 1) * m] for k in range(cnt)]
    return ts, us


def finite_or_nan(x) -> float:
    x = float(x)
    return x if math.isfinite(x) else float("nan")
