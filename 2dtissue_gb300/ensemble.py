"""Host-side ensemble helpers: the ragged replica workloads and their partition over GPUs.

Replicas are independent systems, so several GPUs split an ensemble by replica with no per-step
exchange; only the per-replica order-parameter series are gathered at the end.
"""
import numpy as np


def ragged_replicas(seed=0, n_replicas=4096):
    """The batched ragged ensemble: particle counts log-uniform in [64, 8192], eta uniform in
    [0, 2 pi], v0 uniform in [0.5, 1.5] (seeded)."""
    rng = np.random.default_rng(seed)
    n = np.rint(64.0 * 128.0 ** rng.random(n_replicas)).astype(np.int64)
    eta = rng.random(n_replicas) * 2.0 * np.pi
    v0 = 0.5 + rng.random(n_replicas)
    return n, eta, v0


def shard_replicas(n_per_replica, world_size):
    """Assigns replicas to ranks, balancing the particle count per rank (largest replica first to
    the least-loaded rank; ties go to the lower rank). Returns one sorted index list per rank."""
    n = np.asarray(n_per_replica, dtype=np.int64)
    order = np.lexsort((np.arange(len(n)), -n))  # by size descending, then index
    load = np.zeros(world_size, dtype=np.int64)
    shards = [[] for _ in range(world_size)]
    for i in order:
        r = int(np.argmin(load))
        shards[r].append(int(i))
        load[r] += n[i]
    return [sorted(s) for s in shards]


def merge_series(shards, series_per_rank, n_replicas):
    """Reassembles per-rank order-parameter series ([steps][replicas of that rank]) into
    [steps][all replicas]."""
    steps = series_per_rank[0].shape[0]
    out = np.zeros((steps, n_replicas))
    for idx, s in zip(shards, series_per_rank):
        out[:, idx] = s
    return out
