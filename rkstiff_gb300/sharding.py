"""Instance sharding for runs on several GPUs (one process per GPU).

Instances are independent, so a multi-GPU run partitions them by index with no exchange
during stepping; the only cross-rank operations are a barrier and the max-over-ranks of
the elapsed time.  Weak scaling gives every rank its own instance set (rank-derived
seed); strong scaling splits one fixed set.
"""

from __future__ import annotations

from typing import Tuple

import numpy as np


def strong_partition(n_inst: int, world: int, rank: int) -> Tuple[int, int]:
    """Contiguous [lo, hi) block of a fixed instance set for ``rank`` (sizes differ by <= 1)."""
    if not (0 <= rank < world):
        raise ValueError("rank out of range")
    base, extra = divmod(n_inst, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def weak_seed(seed: int, rank: int) -> int:
    """Seed of rank ``rank``'s own instance set under weak scaling."""
    return int(np.random.SeedSequence([seed, rank]).generate_state(1)[0])


def max_over_ranks(value: float, device=None) -> float:
    """Max of a float over the default process group (identity without one)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
