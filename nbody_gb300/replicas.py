"""Whole-job throughput of independent replicas (one process per GPU, no data-path
collective): each rank steps its own system; the job's time is the slowest rank's.

The direct sum would shard by target ranges with an all-gather of pos_mass per step, and
batched systems by system with no exchange; one GPU per box in this build means the bench
runs N independent replicas, and this is the only cross-rank operation it performs.
"""
from __future__ import annotations


def whole_job_value(local_ms: float, bodies_per_rank: int, steps: int, device=None):
    """(value, max_ms, world): body-steps/s of the whole job from this rank's timed total.
    Collective only when torch.distributed is initialised (gloo: CPU tensor; nccl: `device`)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    max_ms = float(local_ms)
    if world > 1:
        t = torch.tensor([max_ms], dtype=torch.float64,
                         device=device if dist.get_backend() == "nccl" else "cpu")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        max_ms = float(t.item())
    return bodies_per_rank * steps * world / (max_ms * 1e-3), max_ms, world
