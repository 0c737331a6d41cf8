"""Timing aggregation for independent replicas (one process per GPU).

The SimPLIC step does not shard in this build: under torchrun every rank
advances its own copy of the workload.  The job's time is the slowest
rank's, and its throughput counts the cells of every rank.
"""

from __future__ import annotations


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """All-reduce MAX of a per-rank float (identity without a process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, cells: int, steps: int, max_ms: float) -> float:
    """Whole-job cell-steps/s of `world` replicas that each advanced
    `cells` cells for `steps` steps, the slowest taking `max_ms`."""
    if max_ms <= 0:
        raise ValueError("elapsed time must be positive")
    return world * cells * steps / (max_ms * 1e-3)
