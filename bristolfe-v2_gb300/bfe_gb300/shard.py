"""Sharding of independent load steps (sources) and models across ranks.

Sources of an array capture and sub-domain models are independent: each rank
marches its own share with no exchange, and A-scans are gathered on rank 0
once at the end (subdoms/fn_run_main_model.m:101-115 runs the same units one
after the other on one process).
"""
import numpy as np


def partition(n_units, world, rank):
    """Contiguous balanced share [start, stop) of n_units for `rank`."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad world/rank")
    base, extra = divmod(int(n_units), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def weighted_partition(costs, world):
    """Greedy longest-first assignment of units with the given costs (e.g.
    bytes per step of uneven sub-domain models) to `world` ranks; returns a
    list of unit-index lists, one per rank."""
    order = np.argsort(-np.asarray(costs, float), kind="stable")
    load = np.zeros(world)
    out = [[] for _ in range(world)]
    for u in order:
        r = int(np.argmin(load))
        out[r].append(int(u))
        load[r] += costs[u]
    return [sorted(x) for x in out]


def gather_ascans(local, start, n_units, dist, group=None):
    """Gather per-rank A-scan blocks (units along the last axis) on every
    rank with torch.distributed; returns the full (..., n_units) array."""
    import torch
    world = dist.get_world_size(group)
    t = torch.as_tensor(np.ascontiguousarray(local))
    meta = [None] * world
    dist.all_gather_object(meta, (int(start), tuple(t.shape)), group=group)
    full = np.zeros(tuple(t.shape[:-1]) + (int(n_units),), dtype=np.asarray(local).dtype)
    parts = [None] * world
    dist.all_gather_object(parts, np.asarray(local), group=group)
    for (s, shp), p in zip(meta, parts):
        full[..., s:s + shp[-1]] = p
    return full
