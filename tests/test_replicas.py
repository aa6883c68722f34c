"""Replica sharding across processes (one per GPU on a multi-GPU node),
exercised on the CPU with two gloo ranks: the batch split covers every
transform exactly once, and the timing reduction returns the slowest rank."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from tcfft_gb300.replicas import local_batch, max_over_ranks


def test_local_batch_partitions():
    for world in (1, 2, 3, 8):
        for batch in (0, 1, 7, 64, 1000):
            seen = []
            for r in range(world):
                first, count = local_batch(batch, r, world)
                seen.extend(range(first, first + count))
            assert seen == list(range(batch))
            counts = [local_batch(batch, r, world)[1] for r in range(world)]
            assert max(counts) - min(counts) <= (1 if batch else 0)
    with pytest.raises(ValueError):
        local_batch(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        first, count = local_batch(10, rank, world)
        # each rank "times" its own replica; the job time is the slowest rank's
        slowest = max_over_ranks(0.5 + rank, dist)
        cover = torch.zeros(10)
        cover[first:first + count] = 1
        dist.all_reduce(cover)
        out[rank] = (slowest, cover.tolist())
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        slowest, cover = res[rank]
        assert slowest == 1.5
        assert cover == [1.0] * 10


def test_max_over_ranks_single_process():
    assert max_over_ranks(2.5) == 2.5
