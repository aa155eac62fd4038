"""Tuning choices (tds_create_ex) and the autotuner (tds_autotune): the step block changes no
bit; a coarser cell level and 2 or 4 lanes per particle keep per-step parity with the oracle; the
autotuner returns one of its candidates with a positive rate."""
import numpy as np
import pytest

from conftest import oracle_mesh
from test_gpu_parity import compare_step

pytestmark = pytest.mark.gpu


def test_step_block_changes_no_bit(tg, mesh_l4):
    outs = []
    for b in (128, 256):
        sim = tg.Simulation(mesh_l4, tg.Params(), 3000, seed=4, tuning=dict(cells_per_particle=4.0, step_block=b,
                                                                            graph_steps=16))
        assert sim.tuning()["step_block"] == b
        sim.start()
        sim.step(37)
        outs.append(sim.get_state())
    for k in outs[0]:
        np.testing.assert_array_equal(outs[0][k], outs[1][k])


@pytest.mark.parametrize("cpp", [0.25, 64.0])
def test_cell_level_rule_keeps_parity(tg, orc, mesh_l4, cpp):
    """Ragged replicas with a coarse (0.25 cells per particle) and a fine (64) cell-level rule."""
    om, arr = oracle_mesh(orc, mesh_l4)
    cen = arr["v3"].mean(0)
    ns = [64, 300, 1000]
    sim = tg.Simulation(mesh_l4, [tg.Params()] * 3, ns, seed=6, precision=64,
                        tuning=dict(cells_per_particle=cpp, step_block=256, graph_steps=16))
    sim.start()
    sim.step(3)
    g0 = sim.get_state()
    sim.step(1)
    g1 = sim.get_state()
    lb = int(np.ceil(np.log2(max(ns))))
    off = np.concatenate([[0], np.cumsum(ns)])
    for r, n in enumerate(ns):
        sl = slice(off[r], off[r + 1])
        a = {k: v[sl] for k, v in g0.items()}
        b = {k: v[sl] for k, v in g1.items()}
        ids = ((r << lb) | np.arange(n)).astype(np.int32)
        compare_step(orc, om, tg.Params().oracle_dict(), a, b, 3, 6, 64, ids=ids, local_bits=lb, centroid=cen)


def test_autotune_returns_a_candidate(tg, mesh_l4):
    ns = [200, 800, 3000]
    t, rate = tg.autotune(mesh_l4, [tg.Params()] * 3, ns, trial_steps=32)
    assert t["cells_per_particle"] in (1.0, 4.0, 16.0) and t["step_block"] in (128, 256)
    assert t["graph_steps"] in (0, 16) and t["lanes_per_particle"] in (1, 2, 4) and rate > 0
    sim = tg.Simulation(mesh_l4, [tg.Params()] * 3, ns, tuning=t)
    sim.start()
    sim.step(16)
    assert sim.status() == 0


@pytest.mark.parametrize("lanes", [2, 4])
@pytest.mark.parametrize("precision", [32, 64])
def test_lanes_per_particle_keep_parity(tg, orc, mesh_l4, lanes, precision):
    """2 and 4 lanes per particle (16 or 8 particles per warp): per-step parity with the oracle on a
    dense system, and two runs give the same bits (the lanes' partial sums are added in a fixed
    order)."""
    om, arr = oracle_mesh(orc, mesh_l4)
    cen = arr["v3"].mean(0)
    p = tg.Params()
    tun = dict(cells_per_particle=4.0, step_block=128, graph_steps=0, lanes_per_particle=lanes)
    runs = []
    for _ in range(2):
        sim = tg.Simulation(mesh_l4, p, 2000, seed=5, precision=precision, tuning=tun)
        assert sim.tuning()["lanes_per_particle"] == lanes
        sim.start()
        sim.step(3)
        g0 = sim.get_state()
        sim.step(1)
        g1 = sim.get_state()
        out = compare_step(orc, om, p.oracle_dict(), g0, g1, 3, 5, precision, centroid=cen)
        assert out["nbr"].mean() > 1.0
        sim.step(20)
        runs.append(sim.get_state())
    for k in runs[0]:
        np.testing.assert_array_equal(runs[0][k], runs[1][k])


def test_lanes_need_128_thread_blocks(tg, mesh_l4):
    with pytest.raises(tg.TdsError):
        tg.Simulation(mesh_l4, tg.Params(), 100, tuning=dict(cells_per_particle=4.0, step_block=256, graph_steps=0,
                                                            lanes_per_particle=2))
    with pytest.raises(tg.TdsError):
        tg.Simulation(mesh_l4, tg.Params(), 100, tuning=dict(cells_per_particle=4.0, step_block=128, graph_steps=0,
                                                            lanes_per_particle=3))


def test_autotune_ranks_the_candidates(tg):
    """On a dense 200,000-particle system the candidates differ by up to 2x (4 lanes per particle run
    the particle update four times over): the tuner must not pick a slow one, and its pick must run
    at least about as fast as the default tuning timed here the same way."""
    torch = pytest.importorskip("torch")
    mesh = tg.Mesh.ellipsoid(4, (6.0, 3.0, 3.0))
    n = 200000
    R = float(np.sqrt(0.5 * mesh.area / (np.pi * n)))
    p = tg.Params(radius=R, r_max=2.4 * R, eta=0.3, dt=0.01)
    t, rate = tg.autotune(mesh, p, n, trial_steps=64)
    assert t["lanes_per_particle"] == 1

    def timed(tuning):
        sim = tg.Simulation(mesh, p, n, seed=0, tuning=tuning)
        sim.start()
        sim.step(16)
        stream = torch.cuda.ExternalStream(sim.stream())
        best = None
        for _ in range(2):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            sim.step_async(64)
            b.record(stream)
            torch.cuda.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        sim.close()
        return n * 64 / (best * 1e-3)

    default = timed(dict(cells_per_particle=4.0, step_block=128, graph_steps=0, lanes_per_particle=1))
    slow = timed(dict(cells_per_particle=4.0, step_block=128, graph_steps=0, lanes_per_particle=4))
    assert slow < 0.8 * default  # the candidates do differ
    assert timed(t) > 0.9 * default
