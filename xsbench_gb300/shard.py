"""Host logic of multi-GPU runs: one process per GPU, each on its own range
of event indices (lookup i's sample is a pure function of i, so ranges need
no exchange).  The only collectives are the sum of the verification partials
(exact in any order: integers) and the max of the ranks' timed spans."""
from __future__ import annotations


def shard_range(rank: int, world: int, n: int, scaling: str = "weak") -> tuple[int, int]:
    """(first, count) of rank's event indices: weak scaling gives every rank
    n lookups of its own ([rank*n, (rank+1)*n)); strong scaling splits [0, n)."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    if scaling == "weak":
        return rank * n, n
    if scaling == "strong":
        a = n * rank // world
        b = n * (rank + 1) // world
        return a, b - a
    raise ValueError(f"unknown scaling {scaling!r}")


def reduce_verification(partial: int, dist=None) -> int:
    """Sum of the ranks' un-modded verification sums (on every rank)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return int(partial)
    import torch
    t = torch.tensor([int(partial)], dtype=torch.int64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())


def reduce_time_max(seconds: float, dist=None) -> float:
    """The slowest rank's timed span (every rank returns it)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(seconds)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
