"""Event-parallel replicas across ranks (one GPU per rank, torch.distributed).

The solver shards by event: events are independent simulations on the same mesh, so each
rank runs its share of the events in its own handle and no collective touches the wave
fields. The only exchange is the sum of per-event results at the end -- the Frechet
kernels or misfit gradients of an inversion (the reference's multi-event kernels are
summed by post-processing in the same way) -- and the max-over-ranks of the step time.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np


def shard_events(n_events: int, rank: int, world: int) -> List[int]:
    """Contiguous block of event indices for `rank` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n_events, world)
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))


def sum_over_ranks(arrays: Sequence[np.ndarray], group=None) -> List[np.ndarray]:
    """Elementwise sum of FP64 arrays over all ranks (all ranks receive the sum)."""
    import torch
    import torch.distributed as dist
    out = []
    backend = dist.get_backend(group) if dist.is_initialized() else None
    dev = "cuda" if backend == "nccl" else "cpu"
    for a in arrays:
        t = torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(dev)
        if dist.is_initialized() and dist.get_world_size(group) > 1:
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        out.append(t.cpu().numpy())
    return out


def max_over_ranks(x: float, group=None) -> float:
    """Largest value of a scalar over all ranks (the step time of a replicated run)."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size(group) == 1:
        return float(x)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
