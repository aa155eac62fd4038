"""Replica sharding over ranks (world size 2, gloo, CPU): every replica is owned by exactly one
rank, loads are balanced, and the gathered series reassemble in replica order."""
import importlib
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ens = importlib.import_module("2dtissue_gb300.ensemble")
    n, eta, v0 = ens.ragged_replicas(seed=3, n_replicas=257)
    shards = ens.shard_replicas(n, world)
    mine = shards[rank]
    # a stand-in per-replica series: replica index + step / 10, only for this rank's replicas
    series = np.array([[i + t / 10.0 for i in mine] for t in range(5)])
    gathered = [None] * world
    dist.all_gather_object(gathered, (mine, series))
    if rank == 0:
        merged = ens.merge_series([g[0] for g in gathered], [g[1] for g in gathered], len(n))
        q.put((shards, merged, n))
    dist.barrier()
    dist.destroy_process_group()


def test_shards_are_a_balanced_partition():
    ens = importlib.import_module("2dtissue_gb300.ensemble")
    n, eta, v0 = ens.ragged_replicas(seed=0)
    assert len(n) == 4096 and n.min() >= 64 and n.max() <= 8192
    assert 0 <= eta.min() and eta.max() <= 2 * np.pi and 0.5 <= v0.min() and v0.max() <= 1.5
    for world in (1, 2, 3, 8):
        shards = ens.shard_replicas(n, world)
        allidx = np.sort(np.concatenate([np.array(s, dtype=int) for s in shards]))
        np.testing.assert_array_equal(allidx, np.arange(len(n)))
        loads = [n[s].sum() for s in shards]
        assert max(loads) - min(loads) <= n.max()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_gather_series():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    shards, merged, n = q.get(timeout=100)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(shards[0] + shards[1]) == list(range(len(n)))
    expect = np.array([[i + t / 10.0 for i in range(len(n))] for t in range(5)])
    np.testing.assert_allclose(merged, expect)
