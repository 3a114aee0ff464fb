"""Snapshot streaming: the ``u`` / ``t`` snapshots of an evolve (every ``store_freq``
accepted steps, rkstiff/solveras.py:643-646 appends them to the solver's lists) written by
the running kernel into a ring in pinned, mapped host memory and taken by the host while
the launch is still running, so a long run needs neither a device snapshot buffer nor a
relaunch whenever one fills.  ``NpzSnapshotWriter`` writes the stream to an ``.npz`` file
(arrays ``t`` and ``u``) with bounded host memory.
"""

from __future__ import annotations

import ctypes
import os
import tempfile
import time
import zipfile
from typing import Callable, Optional

import numpy as np
import torch

from . import _native as nat


class SnapshotStreamOverrun(RuntimeError):
    """The kernel found the ring full for longer than its timeout (the host did not take
    the snapshots in time); the snapshot of that step was not written."""


class SnapshotRing:
    """``slots`` slots of pinned, mapped host memory, each holding one snapshot of up to
    ``m_max`` modes in the working precision (``rk_ring_create`` / ``rk_ring_take``)."""

    def __init__(self, slots: int, m_max: int, precision: int, timeout_ms: int = 10_000):
        self.lib = nat.load()
        self.cdtype = np.complex128 if precision == nat.RK_FP64 else np.complex64
        self.elem = np.dtype(self.cdtype).itemsize
        self.slot_bytes = (nat.RK_RING_HEADER + int(m_max) * self.elem + 15) // 16 * 16
        self.timeout_ms = int(timeout_ms)
        self.ring = nat.RkRing()
        nat.check(self.lib.rk_ring_create(int(slots), self.slot_bytes, ctypes.byref(self.ring)), "rk_ring_create")
        self.buf = np.empty(self.slot_bytes, dtype=np.uint8)
        self.next = 0

    def reset(self) -> None:
        nat.check(self.lib.rk_ring_reset(ctypes.byref(self.ring)), "rk_ring_reset")
        self.next = 0

    def fill_batch(self, b: nat.RkBatch) -> None:
        b.ring_data = self.ring.data
        b.ring_slot_bytes = self.slot_bytes
        b.ring_slots = self.ring.slots
        b.ring_timeout_ms = self.timeout_ms
        b.ring_head = self.ring.head
        b.ring_tail = self.ring.tail

    def claimed(self) -> int:
        return int(ctypes.c_uint64.from_address(self.ring.head).value)

    def take(self, ms) -> Optional[tuple]:
        """The next snapshot as (instance, t, step, states) if it is complete, else None;
        ``ms`` gives each instance's mode count."""
        rc = self.lib.rk_ring_take(ctypes.byref(self.ring), self.next, self.buf.ctypes.data, self.slot_bytes)
        if rc < 0:
            nat.check(rc, "rk_ring_take")
        if rc == 0:
            return None
        self.next += 1
        hdr = self.buf[:nat.RK_RING_HEADER].view(np.int64)
        inst, step = int(hdr[1]), int(hdr[3])
        t = float(self.buf[16:24].view(np.float64)[0])
        m = int(ms[inst])
        u = self.buf[nat.RK_RING_HEADER:nat.RK_RING_HEADER + m * self.elem].view(self.cdtype).copy()
        return inst, t, step, u

    def drain(self, done: Callable[[], bool], ms, sink: Callable, idle_s: float = 50e-6) -> int:
        """Take snapshots in order, handing each to ``sink(inst, t, step, u)``, until
        ``done()`` is true and every claimed slot was taken; returns the count."""
        count = 0
        while True:
            got = self.take(ms)
            if got is not None:
                sink(*got)
                count += 1
                continue
            if done():
                while (got := self.take(ms)) is not None:
                    sink(*got)
                    count += 1
                if self.claimed() > self.next:
                    raise SnapshotStreamOverrun(
                        f"snapshot stream overrun: {self.claimed() - self.next} claimed slot(s) never completed")
                return count
            time.sleep(idle_s)

    def close(self) -> None:
        if self.ring.data:
            self.lib.rk_ring_destroy(ctypes.byref(self.ring))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NpzSnapshotWriter:
    """Writes snapshots (t, u) to ``path`` as an ``.npz`` with arrays ``t`` (float64, n) and
    ``u`` (n x m, the states' dtype); the states go to a temporary file as they arrive and
    are copied into the archive by ``close()``, so host memory stays bounded."""

    def __init__(self, path: str):
        self.path = os.fspath(path)
        self.t = []
        self.m = None
        self.dtype = None
        fd, self.tmp = tempfile.mkstemp(prefix="rk_snap_", suffix=".bin",
                                        dir=os.path.dirname(os.path.abspath(self.path)) or None)
        self.f = os.fdopen(fd, "wb")

    def append(self, t: float, u) -> None:
        if isinstance(u, torch.Tensor):
            u = u.detach().cpu().numpy()
        u = np.ascontiguousarray(u)
        if self.m is None:
            self.m, self.dtype = u.shape[0], u.dtype
        elif u.shape[0] != self.m or u.dtype != self.dtype:
            raise ValueError("every snapshot must have the same length and dtype")
        self.f.write(u.tobytes())
        self.t.append(float(t))

    def close(self) -> str:
        self.f.close()
        n = len(self.t)
        m = self.m or 0
        dtype = self.dtype or np.dtype(np.complex128)
        try:
            with zipfile.ZipFile(self.path, "w", compression=zipfile.ZIP_STORED, allowZip64=True) as z:
                with z.open("t.npy", "w", force_zip64=True) as w:
                    np.lib.format.write_array(w, np.asarray(self.t, dtype=np.float64))
                with z.open("u.npy", "w", force_zip64=True) as w:
                    hdr = {"descr": np.lib.format.dtype_to_descr(dtype), "fortran_order": False, "shape": (n, m)}
                    np.lib.format.write_array_header_2_0(w, hdr)
                    with open(self.tmp, "rb") as src:
                        while True:
                            chunk = src.read(1 << 22)
                            if not chunk:
                                break
                            w.write(chunk)
        finally:
            os.unlink(self.tmp)
        return self.path

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
