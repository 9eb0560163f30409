"""Replicas across ranks: one process per GPU and no data exchange.

One cutting scene does not shard cheaply (a slab decomposition would need two
halo exchanges per substep and the migration of pair history), so a scene
runs whole on each rank.  A batched sweep is a list of independent instances
(scripts/force_convergence.py:92-129 runs them one after another): each rank
takes a contiguous share of the list.  The only collectives are for timing
and for the totals a report needs: a barrier around the timed region, the
slowest rank's time, and the sum of the work done.
"""

import os


def init(backend="nccl"):
    """(dist or None, rank, world, local rank) from the torchrun environment."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world <= 1:
        return None, rank, world, local
    import torch
    import torch.distributed as dist

    if backend == "nccl":
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        dist.init_process_group(backend)
    return dist, rank, world, local


def shard(count, rank, world):
    """The contiguous range of `count` units this rank takes (sizes differ by at most one)."""
    if count < 0 or world < 1 or not 0 <= rank < world:
        raise ValueError("shard needs count >= 0 and 0 <= rank < world")
    base, extra = divmod(count, world)
    begin = rank * base + min(rank, extra)
    return range(begin, begin + base + (1 if rank < extra else 0))


def _reduce(dist, value, op, device):
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(dist, value, device="cpu"):
    """The largest value over all ranks (the slowest rank's time)."""
    return _reduce(dist, value, None if dist is None else dist.ReduceOp.MAX, device)


def sum_over_ranks(dist, value, device="cpu"):
    """The total of a per-rank value (work units done)."""
    return _reduce(dist, value, None if dist is None else dist.ReduceOp.SUM, device)


def barrier(dist, device=None):
    """Every rank reaches this point (and, with a CUDA device, its queued work is done) before any goes on."""
    if device is not None:
        import torch

        torch.cuda.synchronize(device)
    if dist is not None:
        dist.barrier()
