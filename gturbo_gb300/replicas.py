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


def member_cost(n: int, rko: int) -> float:
    """Relative cost of one step of a member of size n: the FFT work n^2 log2 n per stage."""
    import math

    return (4 if rko == 4 else 2) * float(n) * float(n) * math.log2(n)


def shard_members(costs: list[float], world: int) -> list[list[int]]:
    """Partition member indices over ``world`` ranks, balancing the summed cost: members are
    independent (own field, own Philox key), so an ensemble shards by member with no collective
    on the data path. Longest-processing-time greedy: largest cost first, each member to the
    rank with the least load so far (ties to the lowest rank), so the result is deterministic
    and every rank computes the same partition. Each rank's list keeps ascending order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    shards: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        shards[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in shards]
