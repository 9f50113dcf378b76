"""Replicas across GPUs of one node: the expansion shards over frontier
states with no exchange on the data path (pairs of different nodes are
independent), so each rank expands its own batch and only the step's
timing and unit counts are reduced.

Used by bench.py under torchrun (NCCL); the CPU tests run the same
functions on `gloo` ranks.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous block of [0, n) owned by `rank` (sizes differ by <= 1)."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard(nodes: np.ndarray, rank: int, world: int) -> np.ndarray:
    lo, hi = shard_bounds(len(nodes), rank, world)
    return nodes[lo:hi]


def reduce_step(seconds: float, units: float, device=None) -> tuple[float, float]:
    """(max over ranks of `seconds`, sum over ranks of `units`); the
    identity without an initialised process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds), float(units)
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
