"""Reference-semantics step on the device (tds_ref_*): the reference's own per-step algorithm
(2DTissue.cpp:136-268, Locomotion.cpp:57-162, ForceHelper.cpp:34-104, OrientationHelper.cpp:29-116,
EuclideanTiling.cpp:31-208, CellHelper.cpp:43-230) in FP64 on the GPU, against the oracle's
ref-form step (orc_ref_step), whose parts are pinned by the reference's own known answers.

Per step from identical state: chart positions, velocities and 3D positions within 1e-12, neighbour
counts and the order parameter exactly, integer polarity exactly except where the circular mean
lies within 1e-9 of an integer, where it may differ by one degree: CUDA's and the C library's
cos/sin/atan2 may differ in the last place and the reference truncates the mean to int. An
isolated particle's mean is its own angle up to rounding, so in a sparse system such flips are
common (each is checked against the near-integer condition); the nearest vertex is exact except on
ties between corners.
"""
import numpy as np
import pytest

from conftest import get_mesh

TOL = 1e-12


def _dist_matrix(D, nearest, n):
    a = nearest[:, None]
    b = nearest[None, :]
    d = np.minimum(D[a, b], D[b, a])
    np.fill_diagonal(d, 0.0)
    return d


def _raw_means(orc, D, nearest, n_deg, sigma):
    dl = _dist_matrix(D, nearest, len(n_deg))
    out = np.zeros(len(n_deg))
    for i in range(len(n_deg)):
        out[i] = orc.ref_mean_angle_deg(n_deg[dl[i] < 2 * sigma].astype(np.float64))
    return out


def test_vertex_distances_are_edge_graph_shortest_paths(tg):
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    mesh = get_mesh(tg, 2, (2.0, 1.0, 1.0))
    a = mesh.arrays()
    D = tg.ref_vertex_distances(mesh)
    rows, cols, w = [], [], []
    for f in a["fuv"]:
        for k in range(3):
            i, j = f[k], f[(k + 1) % 3]
            w.append(np.linalg.norm(a["v3"][a["uv2v"][i]] - a["v3"][a["uv2v"][j]]))
            rows.append(i)
            cols.append(j)
    G = sp.coo_matrix((w, (rows, cols)), shape=(mesh.Vuv, mesh.Vuv)).tocsr()
    ref = csgraph.dijkstra(G, directed=False)
    np.testing.assert_allclose(D, ref, rtol=1e-12, atol=1e-14)
    assert np.all(np.diag(D) == 0)
    np.testing.assert_allclose(D, D.T, rtol=1e-12, atol=1e-14)


def test_oracle_ref_step_properties(orc, tg):
    """The oracle's ref-form step on a small system: positions stay in the chart, polarity stays
    an integer, neighbour counts match the distance rule, order parameter in [0, 1]."""
    mesh = get_mesh(tg, 3, (2.0, 1.0, 1.0))
    a = mesh.arrays()
    D = tg.ref_vertex_distances(mesh)
    rng = np.random.default_rng(3)
    N = 60
    f = rng.integers(0, mesh.F, N)
    uv = a["uv"][a["fuv"][f]].mean(1)
    n = rng.integers(0, 360, N).astype(np.int32)
    nearest = a["fuv"][f, 0].astype(np.int32)
    prm = dict(v0=0.1, k=1.0, sigma=0.41667, r_adh=1.0, k_adh=0.75, step_size=0.001)
    out = orc.ref_step(a, D, prm, uv, n, nearest)
    assert np.all((out["uv"] >= 0) & (out["uv"] <= 1))
    dl = _dist_matrix(D, nearest, N)
    np.testing.assert_array_equal(out["nbr"], ((dl != 0) & (dl <= 2.4 * prm["sigma"])).sum(1))
    assert 0 <= out["order"] <= 1
    # speed v0 + |F| along the old polarity
    sp = np.linalg.norm(out["r_dot"], axis=1)
    assert np.all(sp >= prm["v0"] - 1e-12)


CASES = {
    # the 100-particle (2,1,1) ellipsoid system's values (R = 0.05, k = 10, v0 = 1, dt = 0.02,
    # r_adh = r_max = 0.12)
    "sparse_100": (100, dict(v0=1.0, k=10.0, sigma=0.05, r_adh=0.12, k_adh=0.75, step_size=0.02), 50),
    # the reference's constructor defaults (2DTissue.h:37-54)
    "defaults_100": (100, dict(v0=0.1, k=1.0, sigma=0.41667, r_adh=1.0, k_adh=0.75, step_size=0.001), 30),
    # a dense system (each particle has tens of neighbours within 2 sigma)
    "defaults_1000": (1000, dict(v0=0.1, k=1.0, sigma=0.41667, r_adh=1.0, k_adh=0.75, step_size=0.001), 5),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_ref_step_matches_oracle_per_step(tg, orc, case):
    N, prm, steps = CASES[case]
    mesh = get_mesh(tg, 4, (2.0, 1.0, 1.0))
    a = mesh.arrays()
    D = tg.ref_vertex_distances(mesh)
    sim = tg.RefSimulation(mesh, tg.RefParams(**prm), N, seed=7, vertex_dist=D)
    sim.start()
    for t in range(steps):
        s0 = sim.get_state()
        sim.step(1)
        g = sim.get_state()
        o = orc.ref_step(a, D, prm, s0["uv"], s0["n_deg"], s0["nearest"])
        np.testing.assert_allclose(g["r_dot"], o["r_dot"], rtol=TOL, atol=TOL)
        np.testing.assert_array_equal(g["nbr"], o["nbr"])
        bad_n = g["n_deg"] != o["n_deg"]
        if bad_n.any():
            raw = _raw_means(orc, D, s0["nearest"], s0["n_deg"], prm["sigma"])
            assert np.all(np.abs(raw[bad_n] - np.round(raw[bad_n])) < 1e-9), (case, t, np.where(bad_n))
            assert np.all(np.abs(g["n_deg"][bad_n] - o["n_deg"][bad_n]) == 1)
        np.testing.assert_allclose(g["uv"], o["uv"], rtol=TOL, atol=TOL)
        np.testing.assert_allclose(g["r3d"], o["r3d"], rtol=TOL, atol=TOL)
        bad_v = g["nearest"] != o["nearest"]
        if bad_v.any():
            X = o["r3d"][bad_v]
            dg = np.linalg.norm(X - a["v3"][a["uv2v"][g["nearest"][bad_v]]], axis=1)
            do = np.linalg.norm(X - a["v3"][a["uv2v"][o["nearest"][bad_v]]], axis=1)
            np.testing.assert_allclose(dg, do, rtol=1e-12, atol=1e-14)
        assert sim.order_parameter()[-1] == o["order"]


@pytest.mark.gpu
def test_ref_start_is_the_seeded_centroid_placement(tg, orc):
    """start(): face = floor(u0 F), chart centroid, angle floor(u1 360) from Philox4x32-10 with
    counter (i, 0, 0xFFFFFFFE, 0) and key = seed; then the face search."""
    mesh = get_mesh(tg, 4, (2.0, 1.0, 1.0))
    a = mesh.arrays()
    seed = (5 << 32) | 11
    sim = tg.RefSimulation(mesh, tg.RefParams(), 64, seed=seed)
    sim.start()
    g = sim.get_state()
    key = [seed & 0xFFFFFFFF, seed >> 32]
    for i in range(64):
        o = orc.philox4x32_10([i, 0, 0xFFFFFFFE, 0], key)
        f = (int(o[0]) * mesh.F) >> 32
        ang = (int(o[1]) * 360) >> 32
        c = a["uv"][a["fuv"][f]]
        assert g["n_deg"][i] == ang
        np.testing.assert_array_equal(g["uv"][i], ((0.0 + c[0]) + c[1] + c[2]) / 3.0)
    assert sim.order_parameter().size == 0


@pytest.mark.gpu
def test_ref_step_rejects_bad_input(tg):
    mesh = get_mesh(tg, 4, (2.0, 1.0, 1.0))
    with pytest.raises(tg.TdsError) as e:
        tg.RefSimulation(mesh, tg.RefParams(sigma=0.0), 10)
    assert e.value.code == 1
    sim = tg.RefSimulation(mesh, tg.RefParams(), 10)
    with pytest.raises(tg.TdsError) as e:
        sim.set_state(np.full((10, 2), 0.5), np.zeros(10, np.int32), np.full(10, mesh.Vuv, np.int32))
    assert e.value.code == 1
    with pytest.raises(tg.TdsError) as e:
        tg.RefSimulation(mesh, tg.RefParams(), 65537)  # the O(N^2) step's stated maximum
    assert e.value.code == 6
