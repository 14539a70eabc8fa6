"""Replicas across GPUs: the batch units (configurations, edges, IK problems, trajectories) are
independent, so N processes (one per GPU) each take a contiguous slice of the global batch, run
the same kernels on it, and only their outcomes are gathered on the host.  There is no data-path
collective; torch.distributed carries the barrier, the max-over-ranks time and the gather.
"""
from __future__ import annotations

from typing import Tuple


def shard(n: int, rank: int, world: int) -> Tuple[int, int]:
    """[start, stop) of rank's contiguous slice of n units (the first n % world ranks take one more)."""
    if world < 1 or not (0 <= rank < world) or n < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(x: float, dist=None, device=None) -> float:
    """The maximum of a per-rank scalar (e.g. elapsed ms) over all ranks; x itself on one process."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_outcomes(local, dist=None):
    """Concatenate the ranks' outcome arrays (numpy, rank order) on every rank."""
    import numpy as np

    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return np.asarray(local)
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, np.asarray(local))
    return np.concatenate(parts)
