"""Sharding of independent models and sources (load steps) across ranks.

Sub-domain / scatterer models and the sources of an array capture are
independent units: the reference marches them one after the other
(per-transmitter steps, subdoms/fn_run_main_model.m:100-115; sub-domain
models, subdoms/fn_run_subdomain_model.m:26-116). Here each rank marches its
own share with no exchange on the data path, and the A-scans are gathered on
rank 0 once at the end.

Models are the first unit: they are assigned to ranks by estimated cost
(bytes one time step moves), longest first, and every rank marches all
sources of its models. Only when there are more ranks than models are the
sources split instead: every rank then marches every model for a contiguous
share of the sources.
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


def rank_share(costs, n_src, world, rank):
    """The models and the source range [lo, hi) that `rank` marches.

    costs: per-model cost (any unit). With world <= number of models, the
    models are split by cost and each rank takes all sources; otherwise every
    rank takes every model and a contiguous share of the sources."""
    n_models = len(costs)
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad world/rank")
    if world <= n_models:
        return weighted_partition(costs, world)[rank], (0, int(n_src))
    return list(range(n_models)), partition(n_src, world, rank)


def gather_model_ascans(local, lo, n_src, dist, dst=0):
    """Collect per-model A-scans on rank `dst`.

    local: {model id: array (sources hi - lo, ...)} from this rank, for its
    source range starting at lo. Returns {model id: array (n_src, ...)} on
    `dst` (None on the other ranks); torch.distributed object collectives,
    outside any timed region."""
    rank = dist.get_rank()
    parts = [None] * dist.get_world_size() if rank == dst else None
    dist.gather_object({k: (int(lo), np.asarray(v)) for k, v in local.items()}, parts, dst=dst)
    if rank != dst:
        return None
    out = {}
    for part in parts:
        for k, (s0, a) in part.items():
            if k not in out:
                out[k] = np.zeros((int(n_src),) + a.shape[1:], a.dtype)
            out[k][s0:s0 + a.shape[0]] = a
    return out


def sharded_march(costs, n_src, march, dist=None):
    """Run `march` on this rank's share and gather the A-scans on rank 0.

    march(models, lo, hi) marches sources [lo, hi) of the listed models and
    returns {model id: A-scans (hi - lo, ...)}. Returns the full
    {model id: (n_src, ...)} on rank 0 (None elsewhere); without `dist` the
    caller is the only rank."""
    rank, world = (dist.get_rank(), dist.get_world_size()) if dist is not None else (0, 1)
    models, (lo, hi) = rank_share(costs, n_src, world, rank)
    local = march(models, lo, hi)
    if dist is None:
        return {k: np.asarray(v) for k, v in local.items()}
    return gather_model_ascans(local, lo, n_src, dist)
