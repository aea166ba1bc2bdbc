"""Replica timing across ranks (one process per GPU, no data exchange).

The GI stage has no exchange step between GPUs: every rank renders its own
views, so N GPUs run N independent replicas. The only cross-rank operations are
the barrier before the timed region and the max-over-ranks of the elapsed time;
the whole-job throughput counts the units every rank processed.
"""
from __future__ import annotations


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of `value` over all ranks of the default process group (the
    value itself when no group is initialised). `device` is the tensor device of
    the backend (a CUDA device for NCCL, None = CPU for gloo)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier() -> None:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def job_throughput(units_per_rank: float, world: int, elapsed_ms: float) -> float:
    """Units per second of the whole job: every rank processed units_per_rank in
    (at most) elapsed_ms, the slowest rank's time."""
    if elapsed_ms <= 0.0:
        raise ValueError("elapsed time must be positive")
    return world * units_per_rank / (elapsed_ms / 1e3)
