"""Rank bookkeeping for runs on several GPUs of one node (one process per GPU).

The operator path shards by lines (every line is independent), so N ranks either run
independent replicas of the same workload (the benchmark's weak scaling) or split the
lines of one field with no collective on the data path.  The only collective is the
timing reduction: every rank's time for the same number of steps, maximised.
"""
import os


def rank_and_world():
    """(rank, world_size) from the torchrun environment (0, 1 without it)."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def shard(n, rank, world):
    """Contiguous share [lo, hi) of n units for `rank` of `world` (sizes differ by <= 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank outside the world")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def max_over_ranks(value, device=None):
    """The maximum of a per-rank float over all ranks (the value itself without a process group)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()
