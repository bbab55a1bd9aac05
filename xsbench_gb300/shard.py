"""Host logic of multi-GPU runs: one process per GPU, each on its own range
of event indices (lookup i's sample is a pure function of i, so ranges need
no exchange).  The collectives are the sum of the verification partials
(exact in any order: integers), the max of the ranks' timed spans and, for
the adjoint, the sum of the ranks' gradient arrays in rank order (floating
point: a fixed order keeps the result bit-reproducible)."""
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


def reduce_gradients(arrays, dist=None):
    """Sum each rank's gradient arrays (dL/dconcs, dL/dxs: tensors of the same
    shape on every rank) into every rank, adding the ranks' contributions in
    rank order 0, 1, ..., so the bits do not depend on the collective's own
    reduction order.  Returns new tensors; a single process gets copies."""
    import torch
    arrays = list(arrays)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [a.clone() for a in arrays]
    world = dist.get_world_size()
    out = []
    for a in arrays:
        parts = [torch.empty_like(a) for _ in range(world)]
        dist.all_gather(parts, a.contiguous())
        acc = parts[0].clone()
        for p in parts[1:]:
            acc += p
        out.append(acc)
    return out
