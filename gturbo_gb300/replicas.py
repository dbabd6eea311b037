"""Independent replicas on several GPUs (one process per GPU).

A single Gturbo field has no natural sharding: a slab decomposition would need all-to-all
transposes inside every FFT. Several GPUs therefore advance independent replicas: each rank
owns its own field (initial condition seeded by its rank), with no collective on the data
path. Only the timing is combined: the whole-job throughput is the units processed by all ranks
over the slowest rank's time.
"""
from __future__ import annotations


def replica_ic_seed(rank: int) -> int:
    """Seed of the random-phase initial field of replica ``rank``."""
    return 1 + int(rank)


def whole_job_rate(local_units: float, local_seconds: float) -> tuple[float, float, float]:
    """(units of all ranks, max seconds over ranks, units / max seconds).

    Uses the default process group when one is initialised (NCCL on GPUs, gloo on CPU);
    otherwise the local figures.
    """
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(local_units), float(local_seconds), float(local_units) / float(local_seconds)
    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    units = torch.tensor([float(local_units)], dtype=torch.float64, device=dev)
    secs = torch.tensor([float(local_seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(units, op=dist.ReduceOp.SUM)
    dist.all_reduce(secs, op=dist.ReduceOp.MAX)
    u, s = float(units.item()), float(secs.item())
    return u, s, u / s
