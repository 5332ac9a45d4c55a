"""Multi-GPU plumbing: sources shard across ranks (no data-path collective).

Each source's forward + adjoint solve is independent (full.py:22-26,
linesearch.py:30-31), so rank r of W runs a disjoint set of sources: the
global source list is split round-robin (shard_sources).  The only exchanges
are the timing reduction (max over ranks) and the final sum of the kernels
(grad.py:158-165), one FP64 all-reduce of the ranks' kernel sums in device
memory after the time loop (reduce_kernels; pipeline.run_sharded).
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


def rank_world(group=None) -> tuple[int, int]:
    """(rank, world size) of the process group, (0, 1) without one."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def reduce_kernels(t, group=None):
    """Sum a rank's kernel sums (a float64 tensor: K_c, K_rho, hessian) over
    all ranks in place, one all-reduce (grad.py:158-165 sums the per-source
    kernel files).  A CUDA tensor is reduced in device memory over NCCL; a
    CPU tensor over gloo.  Returns t."""
    import torch
    import torch.distributed as dist
    if t.dtype != torch.float64:
        raise TypeError("kernel sums are reduced in FP64")
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t


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
