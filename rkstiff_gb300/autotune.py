"""Autotuner for the launch shape of each grid-size class of an ensemble.

For every class (instances sharing one grid size, launched as one kernel) it times the
candidate thread counts and scratch placements on a sample of that class's own instances
over a short span of simulated time, and keeps the fastest.  Results are cached per
(device, method, precision, operator kind, nonlinearity, n) for the process, and can be
saved to / loaded from a JSON file.
"""

from __future__ import annotations

import json
import os
import time
from typing import Dict, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native as nat
from .engine import DiagEnsemble

# (threads per instance group, groups per block)
SHAPES = ((32, 4), (32, 8), (64, 2), (64, 4), (128, 1), (128, 2), (256, 1))
PLACES = (nat.RK_PLACE_SMEM_ALL, nat.RK_PLACE_SMEM_STATE, nat.RK_PLACE_GLOBAL)

_CACHE: Dict[Tuple, Tuple[int, int, int]] = {}


def _key(eng: DiagEnsemble, n: int) -> Tuple:
    return (torch.cuda.get_device_name(eng.device), eng.method_name, eng.prec, eng.coef_complex, eng.nl_kind, int(n))


def save(path: str) -> None:
    data = [{"key": list(k), "threads": v[0], "place": v[1], "groups": v[2]} for k, v in _CACHE.items()]
    with open(path, "w") as f:
        json.dump(data, f, indent=1)


def load(path: str) -> int:
    if not os.path.exists(path):
        return 0
    with open(path) as f:
        data = json.load(f)
    for item in data:
        _CACHE[tuple(item["key"])] = (int(item["threads"]), int(item["place"]), int(item.get("groups", 1)))
    return len(data)


def _time_candidate(sub: DiagEnsemble, u0: torch.Tensor, span: float, h: float, threads: int, place: int,
                    groups: int, reps: int) -> Optional[float]:
    sub.class_threads = np.full(len(sub.class_n), threads, dtype=np.int32)
    sub.class_place = np.full(len(sub.class_n), place, dtype=np.int32)
    sub.class_groups = np.full(len(sub.class_n), groups, dtype=np.int32)
    u = torch.empty_like(u0)
    best = None
    for _ in range(reps + 1):
        u.copy_(u0)
        torch.cuda.synchronize(sub.device)
        t0 = time.perf_counter()
        try:
            st = sub.evolve(u, 0.0, span, h)
        except nat.NativeError:
            return None  # the placement does not fit this size
        torch.cuda.synchronize(sub.device)
        dt = time.perf_counter() - t0
        work = float(np.sum(sub.ms * st["steps"]))
        rate = work / dt
        best = rate if best is None else max(best, rate)
    return best


def tune(eng: DiagEnsemble, u0s: Sequence, lin_ops: Sequence, kxs: Optional[Sequence], span: float,
         h_init: Optional[float] = None, sample: Optional[int] = None, reps: int = 1,
         shapes: Sequence[Tuple[int, int]] = SHAPES, places: Sequence[int] = PLACES,
         force: bool = False) -> Dict[int, dict]:
    """Choose (threads, groups per block, placement) per class of ``eng`` and install them.

    ``u0s``/``lin_ops``/``kxs`` are the ensemble's per-instance inputs (host arrays),
    ``span`` the simulated time each trial integrates.  Returns {n: {threads, place,
    rates}}."""
    nsm = torch.cuda.get_device_properties(eng.device).multi_processor_count
    sample = sample or 4 * nsm
    h = h_init if h_init is not None else span / 100.0
    chosen_t, chosen_p, chosen_g, report = [], [], [], {}
    for n in eng.class_n:
        key = _key(eng, n)
        if key in _CACHE and not force:
            t, p, gr = _CACHE[key]
            chosen_t.append(t)
            chosen_p.append(p)
            chosen_g.append(gr)
            report[int(n)] = {"threads": t, "place": p, "groups": gr, "cached": True}
            continue
        idx = [i for i in range(eng.n_inst) if eng.ns[i] == n][:sample]
        sub = DiagEnsemble(eng.method_name, [lin_ops[i] for i in idx], eng.nl_kind, eng.nl_coef,
                           None if kxs is None else [kxs[i] for i in idx], [int(n)] * len(idx),
                           precision="fp64" if eng.prec == nat.RK_FP64 else "fp32", device=eng.device,
                           complex_operator=bool(eng.coef_complex))
        sub.ctl, sub.etd = eng.ctl, eng.etd
        u0 = sub.pack_u([u0s[i] for i in idx])
        rates = {}
        for t, gr in shapes:
            for p in places:
                r = _time_candidate(sub, u0, span, h, t, p, gr, reps)
                if r is not None:
                    rates[(t, gr, p)] = r
        if not rates:
            raise RuntimeError(f"no launch shape fits grid size {n}")
        (t, gr, p), _ = max(rates.items(), key=lambda kv: kv[1])
        _CACHE[key] = (t, p, gr)
        chosen_t.append(t)
        chosen_p.append(p)
        chosen_g.append(gr)
        report[int(n)] = {"threads": t, "place": p, "groups": gr,
                          "rates": {f"{a}x{c}/{b}": v for (a, c, b), v in rates.items()}}
    eng.class_threads = np.asarray(chosen_t, dtype=np.int32)
    eng.class_place = np.asarray(chosen_p, dtype=np.int32)
    eng.class_groups = np.asarray(chosen_g, dtype=np.int32)
    return report
