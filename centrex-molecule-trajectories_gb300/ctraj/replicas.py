"""Replica sharding: one process per GPU, no data-path collective.

Molecules are independent, so N GPUs run N independent replicas on disjoint
Philox counter ranges (the reference's joblib workers, trajectory_simulator.py
:81-83, likewise run independent chunks) and the per-label counts, the
molecule-step totals and the elapsed times are reduced once at the end
(the reference merges its workers' Counters, :94-97).
"""
from __future__ import annotations

import numpy as np


def shard(n_total: int, rank: int, world: int) -> tuple[int, int]:
    """(offset, n) of rank's contiguous share of n_total molecules."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    base, rem = divmod(int(n_total), world)
    n = base + (1 if rank < rem else 0)
    offset = rank * base + min(rank, rem)
    return offset, n


def reduce_run(counts, molecule_steps: int, seconds: float, group=None, device=None):
    """Sum counts and molecule-steps, max the elapsed time over the ranks of a
    torch.distributed group (gloo on CPU tensors, nccl with device=cuda)."""
    import torch
    import torch.distributed as dist

    c = torch.as_tensor(np.asarray(counts, dtype=np.int64), device=device)
    s = torch.tensor([int(molecule_steps)], dtype=torch.int64, device=device)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(c, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(s, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return c.cpu().numpy(), int(s.item()), float(t.item())
