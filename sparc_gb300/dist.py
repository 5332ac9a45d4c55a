"""Multi-GPU plumbing: sources shard across ranks (no data-path collective).

Each source's forward + adjoint solve is independent (full.py:22-26,
linesearch.py:30-31), so rank r of W runs a disjoint set of sources.  The only
exchanges are the timing reduction (max over ranks) and the final sum of the
per-source kernels (grad.py:158-165), done once after the time loop.
"""
from __future__ import annotations

import numpy as np


def shard_sources(n_total: int, rank: int, world: int) -> list[int]:
    """Round-robin assignment of source indices to ranks."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    return list(range(rank, n_total, world))


def max_over_ranks(x: float, group=None) -> float:
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def sum_kernels(arr: np.ndarray, group=None) -> np.ndarray:
    """Sum per-rank kernel fields (FP64) across ranks: the grad.py:158-165 sum."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return arr
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64)).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()
