"""Multi-rank path on CPU (gloo, world_size 2): source sharding and A-scan
gathering, as bench.py and multi-process users run them."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from bfe_gb300 import shard


def test_partition_covers_all_units():
    for n in (0, 1, 7, 64):
        for w in (1, 2, 3, 8):
            spans = [shard.partition(n, w, r) for r in range(w)]
            idx = np.concatenate([np.arange(a, b) for a, b in spans]) if n else np.zeros(0)
            assert np.array_equal(idx, np.arange(n))


def test_weighted_partition_balances():
    costs = np.random.default_rng(1).uniform(50e3, 400e3, 32)
    parts = shard.weighted_partition(costs, 4)
    assert sorted(sum(parts, [])) == list(range(32))
    loads = [costs[p].sum() for p in parts]
    assert max(loads) <= 1.15 * costs.sum() / 4 + costs.max()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_units, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a, b = shard.partition(n_units, world, rank)
        # stand-in A-scans: (receivers, samples, sources) filled with the unit id
        local = np.zeros((3, 5, b - a))
        local += np.arange(a, b)[None, None, :]
        full = shard.gather_ascans(local, a, n_units, dist)
        q.put((rank, full))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("n_units", [64, 7])
def test_two_rank_gather_gloo(n_units):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n_units, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, full in res:
        assert full.shape == (3, 5, n_units)
        assert np.array_equal(full[0, 0], np.arange(n_units))
