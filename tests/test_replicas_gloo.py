"""Multi-rank host logic of the replica split (gloo, world_size 2, CPU)."""
import os
import socket

import numpy as np
import pytest

from eobgpu_gb300 import replicas


def test_shard_range_covers():
    for n in (0, 1, 7, 1024, 1025):
        for w in (1, 2, 3, 8):
            parts = [replicas.shard_range(n, w, r) for r in range(w)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(w - 1))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard_range(4, 2, 2)


def test_shard_by_cost_balances_longest():
    rng = np.random.default_rng(3)
    cost = rng.pareto(1.5, 1000) + 1
    parts = replicas.shard_by_cost(cost, 4)
    allidx = np.sort(np.concatenate(parts))
    assert np.array_equal(allidx, np.arange(1000))
    loads = [cost[p].sum() for p in parts]
    assert max(loads) - min(loads) <= cost.max()
    for p in parts:
        assert np.all(np.diff(cost[p]) <= 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, q):
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        cost = np.arange(n, dtype=np.float64) % 13 + 1
        mine = replicas.shard_by_cost(cost, world)[rank]
        # stand-in per-binary lnL: a function of the global index only
        lnl = -(mine.astype(np.float64) * 0.5 + 1.0)
        full = replicas.gather_lnl(torch.tensor(lnl), torch.tensor(mine), n)
        t = replicas.max_over_ranks(float(rank + 1))
        q.put((rank, full.numpy().tolist(), t))
    finally:
        dist.destroy_process_group()


def test_gather_lnl_gloo_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    n = 37
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = -(np.arange(n) * 0.5 + 1.0)
    for rank, full, t in res:
        assert np.array_equal(np.asarray(full), want)
        assert t == 2.0
