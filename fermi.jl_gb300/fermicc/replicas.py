"""Replica bookkeeping for runs on N GPUs of one node.

The coupled-cluster path runs one independent replica per GPU (the same
workload on every rank: weak scaling); there is no data-path collective.  The
only cross-rank step is the measurement: the time of a step is the maximum
over ranks, taken after a barrier.
"""
from __future__ import annotations


def max_over_ranks(value: float, world: int, device=None) -> float:
    """Max of `value` over all ranks of the default process group (identity
    for a single rank).  Works with the gloo (CPU) and nccl backends."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.barrier()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
