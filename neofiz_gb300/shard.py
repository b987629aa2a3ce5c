"""Sharding a batch over ranks: one process per GPU, each stepping its own instances.

Batched work (sweeps, adjoint batches, burst sweeps) is a set of independent instances, so
it splits by instance with no collective in the data path: each rank builds a BatchSolver of
its share and runs it on its GPU; per-instance results come back to rank 0 by a host-side
gather. Shares are balanced by an estimate of each instance's cost -- elements times the
steps its first stable step predicts to t_end -- greedily, most expensive first (the same
order the batched kernel's own queue uses), so the partition is deterministic.
"""
from __future__ import annotations

from typing import List, Sequence


def instance_cost(instance, cfl: float) -> float:
    """Elements x the step count the first CFL step predicts to t_end."""
    mesh = instance.mesh
    wave = instance.material.barWaveSpeed()
    dt0 = cfl * mesh.minimumEdgeLength() / wave
    steps = instance.t_end / dt0 if dt0 > 0.0 else 1.0
    return float(mesh.elementCount) * max(1.0, steps)


def partition(costs: Sequence[float], world: int) -> List[List[int]]:
    """Instance indices per rank: most expensive first, each to the least-loaded rank (the
    lowest rank on ties); each rank's list in ascending instance order."""
    if world < 1:
        raise ValueError("world size must be positive")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def shard(instances, world: int, rank: int, cfl: float) -> List[int]:
    """This rank's instance indices."""
    return partition([instance_cost(x, cfl) for x in instances], world)[rank]


def gather(local: dict, world: int) -> dict:
    """Rank 0 receives every rank's {instance index: result}; other ranks get {}. Host-side,
    through torch.distributed (gloo on CPU, NCCL between GPUs); with world 1, `local`."""
    if world == 1:
        return dict(local)
    import torch.distributed as dist
    parts = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(local, parts, dst=0)
    if dist.get_rank() != 0:
        return {}
    out = {}
    for p in parts:
        out.update(p)
    return out
