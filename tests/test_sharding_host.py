"""Instance sharding for several GPUs, on CPU (no device): the partitions and seeds, and the
cross-rank reductions the bench's multi-GPU timing uses, run as two `gloo` ranks."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from rkstiff_gb300 import sharding


@pytest.mark.parametrize("n_inst", [0, 1, 7, 4096, 4097])
@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_strong_partition_covers_every_instance_once(n_inst, world):
    blocks = [sharding.strong_partition(n_inst, world, r) for r in range(world)]
    assert blocks[0][0] == 0 and blocks[-1][1] == n_inst
    for (lo, hi), (lo2, _) in zip(blocks, blocks[1:]):
        assert hi == lo2
    sizes = [hi - lo for lo, hi in blocks]
    assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        sharding.strong_partition(n_inst, world, world)


def test_weak_seeds_differ_by_rank_and_repeat():
    seeds = [sharding.weak_seed(5, r) for r in range(8)]
    assert len(set(seeds)) == 8
    assert seeds == [sharding.weak_seed(5, r) for r in range(8)]


def test_reductions_without_a_process_group():
    assert sharding.max_over_ranks(2.5) == 2.5
    assert sharding.sum_over_ranks(2.5) == 2.5


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank's elapsed time and work, as the bench's timed region reports them
        elapsed = 1.0 + rank
        work = 100.0 * (rank + 1)
        dist.barrier()
        out[rank, 0] = sharding.max_over_ranks(elapsed)
        out[rank, 1] = sharding.sum_over_ranks(work)
        lo, hi = sharding.strong_partition(4097, world, rank)
        out[rank, 2] = hi - lo
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_time_and_work():
    world = 2
    out = torch.zeros((world, 3), dtype=torch.float64).share_memory_()
    mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
    res = out.numpy()
    np.testing.assert_array_equal(res[:, 0], [2.0, 2.0])  # the slowest rank's time on every rank
    np.testing.assert_array_equal(res[:, 1], [300.0, 300.0])  # the whole job's work
    assert res[:, 2].sum() == 4097
