"""Autotuner for the launch shape of each grid-size class of an ensemble.

Each class (instances sharing one grid size) runs as its own kernel, concurrently with the
other classes.  The tuner takes the classes one at a time, each on its own: the class's
instances (up to ``per_class`` of them) as a one-class ensemble, every candidate (threads
per instance group, groups per block, scratch placement) timed over a short span of
simulated time (best of ``reps`` + 1 runs), and keeps the candidate with the highest
mode-steps/s.  Timing a class alone measures that class's kernel: in a mixed run the
slowest class sets the wall time, so a trial of one class inside the mix cannot tell its
candidates apart unless that class is the slowest.  Results are cached per (device,
method, precision, operator kind, nonlinearity, grid-size mix) for the process and can be
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
SHAPES = ((32, 4), (32, 8), (32, 16), (64, 2), (64, 4), (64, 8), (128, 1), (128, 2), (128, 4), (256, 1),
          (256, 2))
PLACES = (nat.RK_PLACE_SMEM_ALL, nat.RK_PLACE_SMEM_STATE, nat.RK_PLACE_GLOBAL)

_CACHE: Dict[Tuple, Tuple[Tuple[int, int, int], ...]] = {}


def _key(eng: DiagEnsemble) -> Tuple:
    return (torch.cuda.get_device_name(eng.device), eng.method_name, eng.prec, eng.coef_complex, eng.nl_kind,
            tuple(int(n) for n in eng.class_n))


def save(path: str) -> None:
    data = [{"key": list(k), "shapes": [list(v) for v in vals]} for k, vals in _CACHE.items()]
    with open(path, "w") as f:
        json.dump(data, f, indent=1)


def load(path: str) -> int:
    if not os.path.exists(path):
        return 0
    with open(path) as f:
        data = json.load(f)
    for item in data:
        key = tuple(tuple(x) if isinstance(x, list) else x for x in item["key"])
        _CACHE[key] = tuple(tuple(v) for v in item["shapes"])
    return len(data)


def _install(eng: DiagEnsemble, shapes) -> None:
    eng.class_threads = np.asarray([s[0] for s in shapes], dtype=np.int32)
    eng.class_groups = np.asarray([s[1] for s in shapes], dtype=np.int32)
    eng.class_place = np.asarray([s[2] for s in shapes], dtype=np.int32)


def _rate(sub: DiagEnsemble, u0: torch.Tensor, span: float, h: float, reps: int) -> Optional[float]:
    u = torch.empty_like(u0)
    best = None
    for _ in range(reps + 1):
        u.copy_(u0)
        torch.cuda.synchronize(sub.device)
        t0 = time.perf_counter()
        try:
            st = sub.evolve(u, 0.0, span, h)
        except nat.NativeError:
            return None  # a shape that does not fit this size
        torch.cuda.synchronize(sub.device)
        rate = float(np.sum(sub.ms * st["steps"])) / (time.perf_counter() - t0)
        best = rate if best is None else max(best, rate)
    return best


def tune(eng: DiagEnsemble, u0s: Sequence, lin_ops: Sequence, kxs: Optional[Sequence], span: float,
         h_init: Optional[float] = None, per_class: Optional[int] = None, reps: int = 2,
         shapes: Sequence[Tuple[int, int]] = SHAPES, places: Sequence[int] = PLACES,
         force: bool = False) -> Dict[int, dict]:
    """Choose (threads, groups per block, placement) per class of ``eng`` and install them.

    ``u0s``/``lin_ops``/``kxs`` are the ensemble's per-instance inputs (host arrays) and
    ``span`` the simulated time of each trial.  Returns {n: {threads, groups, place, rates}}."""
    key = _key(eng)
    if key in _CACHE and not force:
        chosen = list(_CACHE[key])
        _install(eng, chosen)
        return {int(n): {"threads": c[0], "groups": c[1], "place": c[2], "cached": True}
                for n, c in zip(eng.class_n, chosen)}
    nsm = torch.cuda.get_device_properties(eng.device).multi_processor_count
    per_class = per_class or 8 * nsm
    h = h_init if h_init is not None else span / 100.0
    chosen = []
    report = {}
    for n in eng.class_n:
        idx = [i for i in range(eng.n_inst) if eng.ns[i] == n][:per_class]
        sub = DiagEnsemble(eng.method_name, [lin_ops[i] for i in idx], eng.nl_kind, eng.nl_coef,
                           None if kxs is None else [kxs[i] for i in idx], [int(eng.ns[i]) for i in idx],
                           precision="fp64" if eng.prec == nat.RK_FP64 else "fp32", device=eng.device,
                           complex_operator=bool(eng.coef_complex))
        sub.ctl, sub.etd = eng.ctl, eng.etd
        sub.mlp, sub.mlp_target = eng.mlp, eng.mlp_target
        u0 = sub.pack_u([u0s[i] for i in idx])
        rates = {}
        for t, gr in shapes:
            for p in places:
                _install(sub, [(t, gr, p)])
                r = _rate(sub, u0, span, h, reps)
                if r is not None:
                    rates[(t, gr, p)] = r
        if not rates:
            raise RuntimeError(f"no launch shape fits grid size {n}")
        best = max(rates.items(), key=lambda kv: kv[1])[0]
        chosen.append(best)
        report[int(n)] = {"threads": best[0], "groups": best[1], "place": best[2],
                          "rates": {f"{a}x{b}/{p}": v for (a, b, p), v in rates.items()}}
    _CACHE[key] = tuple(chosen)
    _install(eng, chosen)
    return report
