"""Independent replicas across ranks (one process per GPU).

Nested-sampling runs are independent, so the multi-GPU path shards runs, not data: rank k
runs its own runs with keys PRNGKey(k * runs_per_rank + r), and there is no collective on the
data path.  The only collective is the timing reduction of a benchmark: the slowest rank's
time and the total number of units processed.
"""
from __future__ import annotations

from typing import Tuple

import numpy as np


def replica_keys(rank: int, runs_per_rank: int) -> np.ndarray:
    """[runs_per_rank, 2] jax-layout keys, disjoint across ranks."""
    from .random import PRNGKey
    base = int(rank) * int(runs_per_rank)
    return np.array([PRNGKey(base + r) for r in range(int(runs_per_rank))], np.uint32).reshape(-1, 2)


def reduce_timing(ms: float, units: int, device=None) -> Tuple[float, int]:
    """(max of ms over ranks, sum of units over ranks); the local values without a process
    group.  device: where the reduction tensors live (a CUDA device under NCCL, CPU under gloo)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(ms), int(units)
    t_ms = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    t_units = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t_ms, op=dist.ReduceOp.MAX)
    dist.all_reduce(t_units, op=dist.ReduceOp.SUM)
    return float(t_ms.item()), int(round(t_units.item()))
