"""Edge cases of the CUDA step against the FP64 oracle (per step from identical state): a system of
one particle, two coincident particles (d = 0 contributes no force but counts as a neighbour),
particles on the chart's border and at its corner (the step crosses the seam), ragged ensembles
with replicas of one and two particles, and sizes the C-ABI rejects."""
import numpy as np
import pytest

from conftest import get_mesh, oracle_mesh
from test_gpu_parity import compare_step

pytestmark = pytest.mark.gpu


def _state(tg, sim, uv, theta, face=None):
    sim.set_state(np.asarray(uv, np.float64), np.asarray(theta, np.float64), face)
    return sim.get_state()


@pytest.mark.parametrize("precision", [64, 32])
def test_single_particle(tg, orc, mesh_l4, precision):
    om, arr = oracle_mesh(orc, mesh_l4)
    p = tg.Params()
    sim = tg.Simulation(mesh_l4, p, 1, seed=3, precision=precision)
    g0 = _state(tg, sim, [[0.4, 0.6]], [0.3])
    for t in range(5):
        sim.step(1)
        g1 = sim.get_state()
        assert g1["nbr"][0] == 0
        compare_step(orc, om, p.oracle_dict(), g0, g1, t, 3, precision, centroid=arr["v3"].mean(0))
        g0 = g1


@pytest.mark.parametrize("precision", [64, 32])
def test_coincident_pair(tg, orc, mesh_l4, precision):
    om, arr = oracle_mesh(orc, mesh_l4)
    p = tg.Params()
    sim = tg.Simulation(mesh_l4, p, 2, seed=8, precision=precision)
    g0 = _state(tg, sim, [[0.3, 0.45], [0.3, 0.45]], [0.0, 2.0])
    np.testing.assert_array_equal(g0["r3d"][0], g0["r3d"][1])
    sim.step(1)
    g1 = sim.get_state()
    assert list(g1["nbr"]) == [1, 1]
    assert np.isfinite(g1["uv"]).all() and np.isfinite(g1["theta"]).all()
    compare_step(orc, om, p.oracle_dict(), g0, g1, 0, 8, precision, centroid=arr["v3"].mean(0))


@pytest.mark.parametrize("precision", [64, 32])
def test_particles_on_the_chart_border(tg, orc, mesh_l4, precision):
    """Points on the four sides of the unit square and at a corner, heading out of the chart."""
    om, arr = oracle_mesh(orc, mesh_l4)
    uv = np.array([[0.0, 0.37], [1.0, 0.61], [0.29, 0.0], [0.73, 1.0], [0.0, 0.0], [1.0, 1.0]])
    theta = np.array([np.pi, 0.0, -np.pi / 2, np.pi / 2, -3 * np.pi / 4, np.pi / 4])
    p = tg.Params(eta=0.0)
    sim = tg.Simulation(mesh_l4, p, len(uv), seed=2, precision=precision)
    g0 = _state(tg, sim, uv, theta)
    for t in range(3):
        sim.step(1)
        g1 = sim.get_state()
        assert ((g1["uv"] >= 0) & (g1["uv"] <= 1)).all()
        compare_step(orc, om, p.oracle_dict(), g0, g1, t, 2, precision, centroid=arr["v3"].mean(0))
        g0 = g1


def test_ensemble_with_one_and_two_particle_replicas(tg, orc, mesh_l4):
    om, arr = oracle_mesh(orc, mesh_l4)
    ns = [1, 2, 300, 1, 2]
    ps = [tg.Params(eta=e) for e in (0.2, 0.4, 0.6, 0.8, 1.0)]
    sim = tg.Simulation(mesh_l4, ps, ns, seed=6, precision=64)
    sim.start()
    sim.step(1)
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
        compare_step(orc, om, ps[r].oracle_dict(), a, b, 1, 6, 64, ids=ids, local_bits=lb,
                     centroid=arr["v3"].mean(0))


def test_sizes_the_c_abi_rejects(tg, mesh_l4):
    with pytest.raises(tg.TdsError) as e:
        tg.Simulation(mesh_l4, tg.Params(), 0)
    assert e.value.code == 1
    with pytest.raises(tg.TdsError) as e:
        tg.Simulation(mesh_l4, [tg.Params()] * 2, [5, 0])
    assert e.value.code == 1
    with pytest.raises(tg.TdsError):
        tg.Simulation(mesh_l4, tg.Params(radius=0.05, r_max=0.05), 10)  # r_max must exceed 2R


def test_size_limits(tg, mesh_l4):
    """Beyond the stated maxima the C-ABI answers TDS_ERR_LIMIT before allocating: more than 2^30
    particles in total, or replica and local indices that do not fit the 31-bit particle id."""
    with pytest.raises(tg.TdsError) as e:
        tg.Simulation(mesh_l4, [tg.Params()] * 2, [1 << 30, 1])
    assert e.value.code == 6
    ns = [1] * (1 << 17)
    ns[0] = 1 << 15  # 17 replica bits + 15 local bits > 31
    with pytest.raises(tg.TdsError) as e:
        tg.Simulation(mesh_l4, [tg.Params()] * len(ns), ns)
    assert e.value.code == 6
