"""Shot sharding across ranks (one process per GPU).

Shots are independent: rank r of N migrates shots r, r+N, r+2N, ... and the
stacked images and illuminations are summed with one all-reduce, the
exchange step that corresponds to the serial reduction of per-thread image
buffers in compute_function_gradient.f90:314-330.  The FWI misfit is summed
the same way.  Works with any torch.distributed backend (NCCL on GPUs, gloo
on CPUs).
"""
from __future__ import annotations

import numpy as np


def shard(n: int, rank: int, world: int) -> list[int]:
    """Indices of the shots this rank owns (round robin)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    return list(range(rank, n, world))


def allreduce_sum(arrays: list[np.ndarray], device=None) -> list[np.ndarray]:
    """Sums float32/float64 numpy arrays over all ranks (in place semantics)."""
    import torch
    import torch.distributed as dist
    out = []
    for a in arrays:
        t = torch.from_numpy(np.ascontiguousarray(a))
        if device is not None:
            t = t.to(device)
        dist.all_reduce(t)
        out.append(t.cpu().numpy())
    return out


def allreduce_max(x: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
