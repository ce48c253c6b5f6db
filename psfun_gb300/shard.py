"""Instance sharding for multi-GPU runs (one process per GPU).

The f(A)x path does not shard within one problem on this hardware (one GPU
per process, no halo exchange); independent problems -- the instances of a
batch -- are partitioned across ranks with no data-path collective.  The
partition is a greedy longest-processing-time assignment by stored entries
(the SpMV cost), deterministic on every rank.  Results are gathered only for
reporting.
"""
from __future__ import annotations

import numpy as np


def shard_instances(costs, world: int):
    """Returns, for each rank, the sorted list of instance indices it owns.
    costs: per-instance work (e.g. nnz * nrhs).  Deterministic: ties break by
    index, so every rank computes the same partition without communication."""
    costs = np.asarray(costs, dtype=np.float64)
    order = sorted(range(len(costs)), key=lambda k: (-costs[k], k))
    load = np.zeros(world)
    owner = np.empty(len(costs), dtype=np.int64)
    for k in order:
        r = int(np.argmin(load))  # argmin returns the lowest rank on ties
        owner[k] = r
        load[r] += costs[k]
    return [sorted(np.flatnonzero(owner == r).tolist()) for r in range(world)]


def my_instances(costs, rank: int, world: int):
    return shard_instances(costs, world)[rank]


def gather_results(local: dict, world: int):
    """All-gathers {instance index: numpy array} dictionaries (reporting only)."""
    import torch.distributed as dist
    if world == 1:
        return dict(local)
    parts = [None] * world
    dist.all_gather_object(parts, local)
    out = {}
    for p in parts:
        out.update(p)
    return out
