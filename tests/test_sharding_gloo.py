"""Multi-rank path on CPU (gloo, world_size 2): the sharding driver that
bench.py runs under torchrun - models split across ranks by cost (sources
split when ranks outnumber models), each rank marching its share, A-scans
gathered on rank 0 - end to end, with the march injected as a callable (the
oracle's C port of the v6 loop, one model at a time). The gathered A-scans
must equal the single-rank result exactly."""
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


def test_rank_share_models_first_then_sources():
    costs = [5.0, 1.0, 3.0]
    shares = [shard.rank_share(costs, 8, 2, r) for r in range(2)]
    assert sorted(sum([m for m, _ in shares], [])) == [0, 1, 2]
    assert all(src == (0, 8) for _, src in shares)
    shares = [shard.rank_share(costs, 8, 4, r) for r in range(4)]          # more ranks than models
    assert all(m == [0, 1, 2] for m, _ in shares)
    assert [s for _, s in shares] == [(0, 2), (2, 4), (4, 6), (6, 8)]


def _models():
    """Three small independent models: two steel plates of different sizes
    (absorbers on one) and a coupled water/steel model with an interface."""
    import modelgen
    out = []
    for m in (modelgen.solid_plate(W=1.6e-3, H=0.8e-3, h=0.1e-3),
              modelgen.solid_plate(W=2.0e-3, H=1.0e-3, h=0.1e-3, abs_thick=0.3e-3),
              modelgen.coupled_model(W=1.6e-3, Hw=0.8e-3, Hs=0.8e-3, h=0.1e-3, abs_thick=0.3e-3)):
        dof = 4 if (m["gl"].shape[1] >= 4 and np.any(m["gl"][:, 3] > 0)) else 2
        top = m["mon_nds"]
        srcs = [modelgen.gi_of(m["gl"], [top[(3 * r) % top.size]], dof) for r in range(4)]
        out.append(dict(K=m["K"], C=m["C"], M=m["M"], dt=m["dt"], srcs=srcs,
                        mons=modelgen.gi_of(m["gl"], top, dof)))
    return out


def _oracle_march(models, n_t):
    """march(model ids, lo, hi) for shard.sharded_march: the C port of the v6
    loop, per model and per source; A-scans (sources, n_t, monitors)."""
    from oracle import cpu_port, signals

    def march(ids, lo, hi):
        out = {}
        for k in ids:
            m = models[k]
            dt = min(x["dt"] for x in models)
            t = np.arange(n_t) * dt
            sig = signals.gaussian_pulse(t, 5e6, 5)
            op = cpu_port.CpuOperator(m["K"], m["C"], m["M"], dt)
            out[k] = np.stack([op.march(t, m["srcs"][r] - 1, sig[None, :], m["mons"] - 1).T
                               for r in range(lo, hi)])
        return out
    return march


def _costs(models):
    return [m["K"].nnz * 8 + 12 * m["K"].shape[0] for m in models]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_models, n_t, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    os.environ["OMP_NUM_THREADS"] = "2"
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        models = _models()[:n_models]
        full = shard.sharded_march(_costs(models), 4, _oracle_march(models, n_t), dist)
        q.put((rank, full))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("n_models", [3, 1])
def test_two_rank_sharded_march_equals_one_rank(n_models):
    """3 models over 2 ranks (split by model) and 1 model over 2 ranks (split
    by source): rank 0 gathers exactly the single-rank A-scans."""
    n_t = 120
    models = _models()[:n_models]
    single = shard.sharded_march(_costs(models), 4, _oracle_march(models, n_t))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n_models, n_t, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert res[1] is None
    full = res[0]
    assert sorted(full) == list(range(n_models))
    for k in range(n_models):
        assert full[k].shape == single[k].shape == (4, n_t, models[k]["mons"].size)
        assert np.abs(single[k]).max() > 0
        assert np.array_equal(full[k], single[k])
