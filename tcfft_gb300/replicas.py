"""Replica sharding for several GPUs, one process per GPU.

Transforms in a batch are independent, so the path shards by transform with
no collective in the data path: each rank runs its own plan on its own
transforms.  Two layouts are supported:

* weak scaling (the benchmark): every rank transforms a batch of the same
  size, so the job's work grows with the number of ranks;
* strong scaling: a fixed global batch is split into contiguous, nearly equal
  runs of transforms, one per rank (``local_batch``).

The only communication is timing: ``max_over_ranks`` reduces a per-rank
duration to the slowest rank's (the job is as slow as its slowest replica).
The reference library has no multi-GPU code; this is the process-level
replication its batch layout allows.
"""


def local_batch(global_batch, rank, world):
    """(first transform, count) of rank `rank` when `global_batch` transforms
    are split over `world` ranks: contiguous runs, sizes differing by at most
    one, earlier ranks taking the larger runs."""
    if world < 1 or not 0 <= rank < world or global_batch < 0:
        raise ValueError("bad rank/world/batch: %r/%r/%r" % (rank, world, global_batch))
    base, extra = divmod(global_batch, world)
    count = base + (1 if rank < extra else 0)
    first = rank * base + min(rank, extra)
    return first, count


def max_over_ranks(value, dist=None, device="cpu"):
    """Maximum of a per-rank float over all ranks (the value itself when not
    distributed).  `dist` is torch.distributed (initialised) or None."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
