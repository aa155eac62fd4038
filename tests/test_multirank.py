"""Replica sharding over ranks (world size 2, gloo, CPU): every replica is owned by exactly one
rank, loads are balanced, each rank simulates its own replicas (FP64 oracle steps on the CPU) and
the gathered series reassemble in replica order, equal to a one-process run."""
import importlib
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


REPLICAS = 6
STEPS = 4


def _replica_series(ens, mesh_arrays, replicas):
    """Per-step order parameter of each replica in `replicas` (FP64 oracle steps on the CPU from a
    seeded placement): [steps][len(replicas)]. A replica's run depends only on its own index."""
    import oracle
    from conftest import place_particles
    om = oracle.Mesh(mesh_arrays["v3"], mesh_arrays["f3"], mesh_arrays["uv"], mesh_arrays["fuv"])
    cen = mesh_arrays["v3"].mean(0)
    n, eta, v0 = ens.ragged_replicas(seed=3, n_replicas=REPLICAS)
    n = np.minimum(n, 400)
    out = np.zeros((STEPS, len(replicas)))
    for c, r in enumerate(replicas):
        prm = dict(R=0.05, k=10.0, k_adh=0.75, r_max=0.12, v0=float(v0[r]), mu=1.0, tau=1.0, align=0.5,
                   eta=float(eta[r]), dt=0.02)
        st = place_particles(om, mesh_arrays, int(n[r]), 100 + r)
        for t in range(STEPS):
            o = oracle.model_step(om, prm, st, t, 7 + r, centroid=cen, threads=1)
            st = dict(uv=o["uv"], theta=o["theta"], face=o["face"], r3d=o["r3d"], ids=st["ids"])
            out[t, c] = np.linalg.norm(o["phi_sums"][:3]) / len(st["ids"])
    return out, n


def _worker(rank, world, port, mesh_arrays, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ens = importlib.import_module("2dtissue_gb300.ensemble")
    n, _, _ = ens.ragged_replicas(seed=3, n_replicas=REPLICAS)
    shards = ens.shard_replicas(np.minimum(n, 400), world)
    mine = shards[rank]
    # this rank simulates only its own replicas; the series are gathered at the end (no per-step
    # exchange between ranks)
    series, _ = _replica_series(ens, mesh_arrays, mine)
    gathered = [None] * world
    dist.all_gather_object(gathered, (mine, series))
    if rank == 0:
        merged = ens.merge_series([g[0] for g in gathered], [g[1] for g in gathered], REPLICAS)
        q.put((shards, merged))
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


@pytest.mark.timeout(180)
def test_two_gloo_ranks_run_their_shards(tg):
    """Two gloo ranks each run the replicas of their shard (oracle steps on the CPU) and gather the
    order-parameter series; the merged series equal a one-process run of every replica."""
    import torch.multiprocessing as mp
    ens = importlib.import_module("2dtissue_gb300.ensemble")
    arrays = tg.Mesh.ellipsoid(3, (2.0, 1.0, 1.0)).arrays()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, arrays, q)) for r in range(2)]
    for p in procs:
        p.start()
    shards, merged = q.get(timeout=150)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(shards[0] + shards[1]) == list(range(REPLICAS)) and shards[0] and shards[1]
    alone, _ = _replica_series(ens, arrays, list(range(REPLICAS)))
    np.testing.assert_array_equal(merged, alone)
    assert (merged > 0).all() and (merged <= 1).all()
