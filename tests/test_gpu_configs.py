"""Per-step parity of the CUDA path with the FP64 oracle on the inputs of the three larger workloads,
through the C-ABI, from identical state with identical Philox noise (tolerances as in
test_gpu_parity.py: neighbour counts and faces exact outside the 1e-6 bands, positions and polarity
1e-5 relative in FP32, 1e-12 in FP64):

  * the batched ragged ensemble: 4,096 replicas on the (4,2,2) ellipsoid (level-4 icosphere),
    particle counts log-uniform in [64, 8192] (area packing up to 0.75), eta uniform in [0, 2 pi],
    v0 uniform in [0.5, 1.5], R 0.05, dt 0.02 -- the whole ensemble steps on the GPU and 16 replicas
    (the densest, the noisiest and 14 seeded ones) are checked one by one against the oracle;
  * the differentiable step: 10,000 particles on the (6,3,3) ellipsoid (area packing 0.41) with
    (v0 1, k 10, tau 1, align 0.5); one step in FP32 and FP64, and the adjoint of 6 steps against the
    chained forward-mode (dual-number) oracle step;
  * the batched adjoint's ensemble: the bumpy sphere r = 1 + 0.2 Re Y_4^2 scaled x5 (level-6
    icosphere), 3 replicas with particle counts and (v0, k, tau, eta) drawn from that workload's
    ranges (k up to 20); one step per replica in FP32 and FP64, and the adjoint of 4 steps of the
    ensemble against the dual-number oracle, replica by replica.

The per-step rules restated by the oracle follow Locomotion.cpp:57-89 and CellHelper.cpp:104-160
of the reference (model form)."""
import importlib

import numpy as np
import pytest

from scipy.spatial import cKDTree

from conftest import face_map_residual, get_mesh, oracle_mesh
from test_gpu_parity import compare_step

pytestmark = pytest.mark.gpu

GRAD_TO_ORACLE = dict(k_rep="k", k_adh="k_adh", v0="v0", mu="mu", tau="tau", align="align", eta="eta")


def _slice(state, a, b):
    return {k: v[a:b] for k, v in state.items()}


def _tangent_r3(om, face, duv, J=None):
    if J is not None:  # every face's chart map, [F][6]
        Jf = J[np.asarray(face)]
        return Jf[:, :3] * duv[:, :1] + Jf[:, 3:] * duv[:, 1:]
    dr = np.zeros((len(face), 3))
    for i, f in enumerate(face):
        J, _, _ = om.face_data(int(f))
        dr[i] = J[:3] * duv[i, 0] + J[3:] * duv[i, 1]
    return dr


def _chain(orc, om, cen, prm, state, ids, lb, seed, t0, T, tgt, phit, dprm=None, duv=None, dth=None, J=None):
    """Loss of T oracle steps of one replica (its ids carry the replica index for the noise) and,
    with tangents, its directional derivative along (dprm, duv, dth)."""
    n = len(state["theta"])
    st = dict(uv=state["uv"].copy(), theta=state["theta"].copy(), face=state["face"].copy(),
              r3d=state["r3d"].copy(), ids=ids)
    dual = dprm is not None
    if dual:
        ds = dict(uv=duv.copy(), theta=dth.copy(), r3d=_tangent_r3(om, st["face"], duv, J))
    loss, dloss = 0.0, 0.0
    for t in range(T):
        if dual:
            out = orc.model_step_dual(om, prm, dprm, st, ds, t0 + t, seed, local_bits=lb, centroid=cen)
        else:
            out = orc.model_step(om, prm, st, t0 + t, seed, local_bits=lb, centroid=cen)
        S = out["phi_sums"][:3]
        phi = np.linalg.norm(S) / n
        loss += (phi - phit[t]) ** 2
        if dual:
            dphi = S @ out["dphi_sums"][:3] / (np.linalg.norm(S) * n)
            dloss += 2 * (phi - phit[t]) * dphi
            ds = dict(uv=out["duv"], theta=out["dtheta"], r3d=out["dr3d"])
        st = dict(uv=out["uv"], theta=out["theta"], face=out["face"], r3d=out["r3d"], ids=ids)
    d = st["r3d"] - tgt
    loss += (d * d).sum() / n
    if dual:
        dloss += 2 * (d * ds["r3d"]).sum() / n
    return loss, dloss


def _local_bits(ns):
    return 31 if len(ns) == 1 else max(1, int(np.ceil(np.log2(max(ns)))))


def _check_adjoint(tg, orc, om, cen, sim, ns, seed, T, rtol, rng):
    """Adjoint of T steps of `sim` (the loss of every replica summed) against the dual-number
    oracle chained replica by replica: the directional derivative along a random direction of
    (parameters, initial uv, initial theta), and each parameter of each replica on its own."""
    s0 = sim.get_state()
    t0 = sim.step_count
    R = len(ns)
    N = sum(ns)
    off = np.concatenate([[0], np.cumsum(ns)])
    lb = _local_bits(ns)
    tgt = s0["r3d"] + 0.01 * rng.normal(size=(N, 3))
    phit = np.full((T, R), 0.3)
    res = sim.adjoint(T, r3d_target=tgt, w_pos=1.0, phi_target=phit, w_phi=1.0)
    direction = rng.normal(size=(R, len(tg.GRAD_PARAMS)))
    duv = 1e-2 * rng.normal(size=(N, 2))
    dth = rng.normal(size=N)
    loss, dloss = 0.0, 0.0
    for r in range(R):
        a, b = off[r], off[r + 1]
        prm = sim.params[r].oracle_dict()
        dprm = {k: 0.0 for k in prm}
        for j, name in enumerate(tg.GRAD_PARAMS):
            dprm[GRAD_TO_ORACLE[name]] = direction[r, j]
        ids = (((r << lb) if R > 1 else 0) | np.arange(ns[r])).astype(np.int32)
        l, dl = _chain(orc, om, cen, prm, _slice(s0, a, b), ids, lb, seed, t0, T, tgt[a:b], phit[:, r], dprm,
                       duv[a:b], dth[a:b])
        loss += l
        dloss += dl
        for j, name in enumerate(tg.GRAD_PARAMS):
            dp = {k: 0.0 for k in prm}
            dp[GRAD_TO_ORACLE[name]] = 1.0
            _, dlj = _chain(orc, om, cen, prm, _slice(s0, a, b), ids, lb, seed, t0, T, tgt[a:b], phit[:, r], dp,
                            np.zeros((ns[r], 2)), np.zeros(ns[r]))
            np.testing.assert_allclose(res["d_params"][r, j], dlj, rtol=rtol,
                                       atol=max(1e-9 * max(1.0, abs(dlj)), rtol * 1e-3 * np.abs(res["d_params"][r]).max()),
                                       err_msg="replica %d, %s" % (r, name))
    gpu = (res["d_params"] * direction).sum() + (res["d_uv0"] * duv).sum() + res["d_theta0"] @ dth
    np.testing.assert_allclose(res["loss"], loss, rtol=1e-9)
    np.testing.assert_allclose(gpu, dloss, rtol=rtol)


def _whole_ensemble_invariants(arr, ns, r_max, g0, g1):
    """The whole ensemble's state after a step: every neighbour count against a k-d tree over the
    step's starting positions (replicas set 100 apart along x, so that no pair crosses replicas;
    the meshes span less than 15), particles with a pair within 1e-5 of r_max excepted; every 3D
    position is its face's chart map of its chart position, inside that face."""
    rep = np.repeat(np.arange(len(ns)), ns)
    r0 = g0["r3d"]
    assert np.abs(r0).max() < 40.0
    shifted = r0 + np.outer(100.0 * rep, [1.0, 0.0, 0.0])
    tree = cKDTree(shifted)
    cnt = tree.query_ball_point(shifted, r_max, return_length=True, workers=-1) - 1
    off = np.nonzero(cnt != g1["nbr"])[0]
    if len(off):
        pairs = tree.query_pairs(r_max + 1e-4, output_type="ndarray")
        d = np.linalg.norm(r0[pairs[:, 0]] - r0[pairs[:, 1]], axis=1)
        band = np.zeros(len(r0), bool)
        band[pairs[np.abs(d - r_max) < 1e-5].ravel()] = True
        assert np.all(band[off]), off[~band[off]][:10]
    assert len(off) <= 1e-5 * len(r0)
    assert g1["nbr"].mean() > 0.5
    wmin, res = face_map_residual(arr, g1["uv"], g1["face"], g1["r3d"])
    assert wmin.min() > -1e-3
    assert res.max() < 1e-4  # coordinates up to ~6: FP32 rounding of the map is ~1e-6


# ---------------------------------------------------------------------------------------------
# batched ragged ensemble: 4,096 replicas on the (4,2,2) ellipsoid
# ---------------------------------------------------------------------------------------------
def test_ragged_ensemble_4096_replicas_parity(tg, orc):
    ens = importlib.import_module("2dtissue_gb300.ensemble")
    mesh = get_mesh(tg, 4, (4.0, 2.0, 2.0))
    om, arr = oracle_mesh(orc, mesh)
    cen = arr["v3"].mean(0)
    n, eta, v0 = ens.ragged_replicas(seed=0, n_replicas=4096)
    ns = [int(x) for x in n]
    ps = [tg.Params(radius=0.05, r_max=0.12, v0=float(v), eta=float(e), dt=0.02) for e, v in zip(eta, v0)]
    sim = tg.Simulation(mesh, ps, ns, seed=0, precision=32)
    sim.start()
    sim.step(3)
    g0 = sim.get_state()
    sim.step(1)
    g1 = sim.get_state()
    phi, psi = sim.order_parameter()
    assert sim.status() == 0
    lb = _local_bits(ns)
    off = np.concatenate([[0], np.cumsum(ns)])
    packing = n * np.pi * 0.05 ** 2 / mesh.area
    assert packing.max() > 0.7
    pick = {int(np.argmax(n)), int(np.argmax(eta))}
    pick |= set(int(i) for i in np.random.default_rng(11).choice(len(ns), 14, replace=False))
    assert len(pick) >= 15
    for r in sorted(pick):
        a, b = off[r], off[r + 1]
        ids = ((r << lb) | np.arange(ns[r])).astype(np.int32)
        out = compare_step(orc, om, ps[r].oracle_dict(), _slice(g0, a, b), _slice(g1, a, b), 3, 0, 32, ids=ids,
                           local_bits=lb, centroid=cen)
        np.testing.assert_allclose(phi[3, r], np.linalg.norm(out["phi_sums"][:3]) / ns[r], rtol=1e-4, atol=1e-6)
        np.testing.assert_allclose(psi[3, r], np.linalg.norm(out["phi_sums"][3:]) / ns[r], rtol=1e-4, atol=1e-6)
    _whole_ensemble_invariants(arr, ns, 0.12, g0, g1)
    # every replica against the oracle: values within the FP32 tolerance but for a few in 10^5
    # (the ill-conditioned directions where the velocity nearly cancels), phi and psi within a
    # quarter of one particle's largest share and at 1e-4 in all but 1% of the replicas
    tally, loose = {}, 0
    for r in range(len(ns)):
        a, b = off[r], off[r + 1]
        ids = ((r << lb) | np.arange(ns[r])).astype(np.int32)
        out = compare_step(orc, om, ps[r].oracle_dict(), _slice(g0, a, b), _slice(g1, a, b), 3, 0, 32, ids=ids,
                           local_bits=lb, centroid=cen, tally=tally)
        for gpu, ref in ((phi[3, r], np.linalg.norm(out["phi_sums"][:3]) / ns[r]),
                         (psi[3, r], np.linalg.norm(out["phi_sums"][3:]) / ns[r])):
            assert abs(gpu - ref) < 0.5 / ns[r], (r, gpu, ref)
            loose += abs(gpu - ref) > 1e-4 * ref
    assert loose <= 0.01 * len(ns), loose
    outside = sum(v for k, v in tally.items() if k not in ("n", "worst"))
    assert tally["n"] > 0.99 * sum(ns)
    assert outside <= 1e-4 * tally["n"] and tally["worst"] < 100.0, tally
    assert tally["uv"] == 0 and tally["vel_uv"] == 0, tally
    sim.close()


def test_ragged_ensemble_4096_replicas_fp64(tg, orc):
    """The FP64 build on the batched ragged ensemble (4,096 replicas, 6.75M particles): every
    replica's step against the oracle's at 1e-12, and its order parameters."""
    ens = importlib.import_module("2dtissue_gb300.ensemble")
    mesh = get_mesh(tg, 4, (4.0, 2.0, 2.0))
    om, arr = oracle_mesh(orc, mesh)
    cen = arr["v3"].mean(0)
    n, eta, v0 = ens.ragged_replicas(seed=0, n_replicas=4096)
    ns = [int(x) for x in n]
    ps = [tg.Params(radius=0.05, r_max=0.12, v0=float(v), eta=float(e), dt=0.02) for e, v in zip(eta, v0)]
    sim = tg.Simulation(mesh, ps, ns, seed=0, precision=64)
    sim.start()
    sim.step(2)
    g0 = sim.get_state()
    sim.step(1)
    g1 = sim.get_state()
    phi, psi = sim.order_parameter()
    assert sim.status() == 0
    lb = _local_bits(ns)
    off = np.concatenate([[0], np.cumsum(ns)])
    for r in range(len(ns)):
        a, b = off[r], off[r + 1]
        ids = ((r << lb) | np.arange(ns[r])).astype(np.int32)
        out = compare_step(orc, om, ps[r].oracle_dict(), _slice(g0, a, b), _slice(g1, a, b), 2, 0, 64, ids=ids,
                           local_bits=lb, centroid=cen)
        np.testing.assert_allclose(phi[2, r], np.linalg.norm(out["phi_sums"][:3]) / ns[r], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(psi[2, r], np.linalg.norm(out["phi_sums"][3:]) / ns[r], rtol=1e-9, atol=1e-12)
    sim.close()


# ---------------------------------------------------------------------------------------------
# differentiable step: 10,000 particles on the (6,3,3) ellipsoid
# ---------------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def diff_mesh(tg, orc):
    mesh = get_mesh(tg, 4, (6.0, 3.0, 3.0))
    om, arr = oracle_mesh(orc, mesh)
    return mesh, om, arr["v3"].mean(0)


DIFF_PARAMS = dict(v0=1.0, k_rep=10.0, tau=1.0, align=0.5)


@pytest.mark.parametrize("precision", [32, 64])
def test_differentiable_system_10000_particles_parity(tg, orc, diff_mesh, precision):
    mesh, om, cen = diff_mesh
    p = tg.Params(**DIFF_PARAMS)
    sim = tg.Simulation(mesh, p, 10000, seed=0, precision=precision)
    sim.start()
    sim.step(5)
    g0 = sim.get_state()
    sim.step(1)
    g1 = sim.get_state()
    out = compare_step(orc, om, p.oracle_dict(), g0, g1, 5, 0, precision, centroid=cen)
    assert out["nbr"].mean() > 1.0
    phi, _ = sim.order_parameter()
    np.testing.assert_allclose(phi[5, 0], np.linalg.norm(out["phi_sums"][:3]) / 10000,
                               rtol=1e-5 if precision == 32 else 1e-10, atol=1e-7)
    sim.close()


def test_differentiable_system_adjoint_matches_dual_oracle(tg, orc, diff_mesh):
    """FP64 build, 6 steps at the differentiable workload's parameters (10,000 particles)."""
    mesh, om, cen = diff_mesh
    sim = tg.Simulation(mesh, tg.Params(**DIFF_PARAMS), 10000, seed=0, precision=64)
    sim.start()
    sim.step(2)
    _check_adjoint(tg, orc, om, cen, sim, [10000], 0, 6, 1e-6, np.random.default_rng(4))
    sim.close()


# ---------------------------------------------------------------------------------------------
# batched adjoint's ensemble: bumpy sphere, level-6 icosphere
# ---------------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def bumpy(tg, orc):
    mesh = tg.Mesh.bumpy_sphere(6, 0.2, 5.0)
    assert mesh.F == 81920
    om, arr = oracle_mesh(orc, mesh)
    rng = np.random.default_rng(21)
    ns = [int(x) for x in rng.integers(1000, 20001, size=3)]
    ps = [tg.Params(v0=float(rng.uniform(0.5, 1.5)), k_rep=float(rng.uniform(5, 20)), tau=float(rng.uniform(0.5, 2)),
                    eta=float(rng.uniform(0.1, 1.0))) for _ in range(3)]
    ps[0].k_rep = 20.0  # the stiffest contact of the workload's range
    return mesh, om, arr["v3"].mean(0), ns, ps


@pytest.mark.parametrize("precision", [32, 64])
def test_bumpy_sphere_ensemble_parity(tg, orc, bumpy, precision):
    mesh, om, cen, ns, ps = bumpy
    sim = tg.Simulation(mesh, ps, ns, seed=1, precision=precision)
    sim.start()
    sim.step(3)
    g0 = sim.get_state()
    sim.step(1)
    g1 = sim.get_state()
    phi, _ = sim.order_parameter()
    lb = _local_bits(ns)
    off = np.concatenate([[0], np.cumsum(ns)])
    for r in range(len(ns)):
        a, b = off[r], off[r + 1]
        ids = ((r << lb) | np.arange(ns[r])).astype(np.int32)
        out = compare_step(orc, om, ps[r].oracle_dict(), _slice(g0, a, b), _slice(g1, a, b), 3, 1, precision,
                           ids=ids, local_bits=lb, centroid=cen)
        np.testing.assert_allclose(phi[3, r], np.linalg.norm(out["phi_sums"][:3]) / ns[r],
                                   rtol=1e-4 if precision == 32 else 1e-10, atol=1e-7)
    sim.close()


def test_bumpy_sphere_512_replica_ensemble(tg, orc, bumpy):
    """The batched-adjoint workload's own ensemble at its full size: 512 replicas on the bumpy
    sphere, 1,000-20,000 particles each (5.2M), per-replica v0, k, tau, eta drawn from the workload's
    ranges, FP32, one step from identical state: the whole ensemble's invariants, and every
    replica against the oracle's step of that replica (neighbour counts and faces as everywhere).
    With contact stiffness up to k = 20 a few particles in 10^5 exceed the per-value tolerance by
    a small factor (measured: 57 of 5.2M, in theta or r3d, at most 14x; none in uv or the
    velocity): at most 1 in 10^4 may, by at most 100x. Each replica's order parameters phi and psi
    match the oracle's at 1e-4 relative in all but 1% of the replicas (measured: median 2e-7,
    worst but one 2e-6), and in every replica to less than a quarter of one particle's largest
    possible share, 0.5 / n: a particle whose velocity v0 p + mu F_t nearly cancels turns its
    unit terms normalize((r - c) x v) and v / |v| by a large angle for a small change of v
    (measured worst: 0.17 / n for phi, 0.29 / n for psi)."""
    mesh, om, cen, _, _ = bumpy
    arr = mesh.arrays()
    rng = np.random.default_rng(5)
    ns = [int(x) for x in rng.integers(1000, 20001, size=512)]
    ps = [tg.Params(v0=float(rng.uniform(0.5, 1.5)), k_rep=float(rng.uniform(5, 20)), tau=float(rng.uniform(0.5, 2)),
                    eta=float(rng.uniform(0.1, 1.0))) for _ in range(512)]
    sim = tg.Simulation(mesh, ps, ns, seed=1, precision=32)
    sim.start()
    sim.step(3)
    g0 = sim.get_state()
    sim.step(1)
    g1 = sim.get_state()
    phi, psi = sim.order_parameter()
    assert sim.status() == 0
    _whole_ensemble_invariants(arr, ns, 0.12, g0, g1)
    lb = _local_bits(ns)
    off = np.concatenate([[0], np.cumsum(ns)])
    tally, loose = {}, 0
    for r in range(len(ns)):
        a, b = off[r], off[r + 1]
        ids = ((r << lb) | np.arange(ns[r])).astype(np.int32)
        out = compare_step(orc, om, ps[r].oracle_dict(), _slice(g0, a, b), _slice(g1, a, b), 3, 1, 32, ids=ids,
                           local_bits=lb, centroid=cen, tally=tally)
        for gpu, ref in ((phi[3, r], np.linalg.norm(out["phi_sums"][:3]) / ns[r]),
                         (psi[3, r], np.linalg.norm(out["phi_sums"][3:]) / ns[r])):
            assert abs(gpu - ref) < 0.5 / ns[r], (r, gpu, ref)
            loose += abs(gpu - ref) > 1e-4 * ref
    assert loose <= 0.01 * len(ns), loose
    outside = sum(v for k, v in tally.items() if k not in ("n", "worst"))
    assert tally["n"] > 0.99 * sum(ns)
    assert outside <= 1e-4 * tally["n"] and tally["worst"] < 100.0, tally
    assert tally["uv"] == 0 and tally["vel_uv"] == 0, tally
    sim.close()


def test_bumpy_sphere_512_replica_ensemble_fp64(tg, orc, bumpy):
    """The FP64 build on the batched-adjoint workload's whole 512-replica ensemble (5.2M
    particles, k up to 20): every replica's step and order parameters against the oracle's at
    1e-12."""
    mesh, om, cen, _, _ = bumpy
    rng = np.random.default_rng(5)
    ns = [int(x) for x in rng.integers(1000, 20001, size=512)]
    ps = [tg.Params(v0=float(rng.uniform(0.5, 1.5)), k_rep=float(rng.uniform(5, 20)), tau=float(rng.uniform(0.5, 2)),
                    eta=float(rng.uniform(0.1, 1.0))) for _ in range(512)]
    sim = tg.Simulation(mesh, ps, ns, seed=1, precision=64)
    sim.start()
    sim.step(2)
    g0 = sim.get_state()
    sim.step(1)
    g1 = sim.get_state()
    phi, psi = sim.order_parameter()
    assert sim.status() == 0
    lb = _local_bits(ns)
    off = np.concatenate([[0], np.cumsum(ns)])
    for r in range(len(ns)):
        a, b = off[r], off[r + 1]
        ids = ((r << lb) | np.arange(ns[r])).astype(np.int32)
        out = compare_step(orc, om, ps[r].oracle_dict(), _slice(g0, a, b), _slice(g1, a, b), 2, 1, 64, ids=ids,
                           local_bits=lb, centroid=cen)
        np.testing.assert_allclose(phi[2, r], np.linalg.norm(out["phi_sums"][:3]) / ns[r], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(psi[2, r], np.linalg.norm(out["phi_sums"][3:]) / ns[r], rtol=1e-9, atol=1e-12)
    sim.close()

def test_bumpy_sphere_512_replica_adjoint_fp64(tg, orc, bumpy):
    """The FP64 adjoint of 3 steps of the batched-adjoint workload's whole 512-replica ensemble
    (5.2M particles, k up to 20) against the dual-number oracle chained replica by replica: the
    directional derivative of the summed loss along a random direction of every replica's
    parameters and of the initial chart positions and angles (1e-6), and the loss (1e-9)."""
    mesh, om, cen, _, _ = bumpy
    rng = np.random.default_rng(5)
    ns = [int(x) for x in rng.integers(1000, 20001, size=512)]
    ps = [tg.Params(v0=float(rng.uniform(0.5, 1.5)), k_rep=float(rng.uniform(5, 20)), tau=float(rng.uniform(0.5, 2)),
                    eta=float(rng.uniform(0.1, 1.0))) for _ in range(512)]
    sim = tg.Simulation(mesh, ps, ns, seed=1, precision=64)
    sim.start()
    sim.step(2)
    s0 = sim.get_state()
    t0 = sim.step_count
    T, R, N = 3, len(ns), sum(ns)
    off = np.concatenate([[0], np.cumsum(ns)])
    lb = _local_bits(ns)
    rng = np.random.default_rng(9)
    tgt = s0["r3d"] + 0.01 * rng.normal(size=(N, 3))
    phit = np.full((T, R), 0.3)
    res = sim.adjoint(T, r3d_target=tgt, w_pos=1.0, phi_target=phit, w_phi=1.0)
    direction = rng.normal(size=(R, len(tg.GRAD_PARAMS)))
    duv = 1e-2 * rng.normal(size=(N, 2))
    dth = rng.normal(size=N)
    J = np.array([om.face_data(f)[0] for f in range(om.F)])
    loss, dloss = 0.0, 0.0
    for r in range(R):
        a, b = off[r], off[r + 1]
        prm = ps[r].oracle_dict()
        dprm = {k: 0.0 for k in prm}
        for j, name in enumerate(tg.GRAD_PARAMS):
            dprm[GRAD_TO_ORACLE[name]] = direction[r, j]
        ids = ((r << lb) | np.arange(ns[r])).astype(np.int32)
        l, dl = _chain(orc, om, cen, prm, _slice(s0, a, b), ids, lb, 1, t0, T, tgt[a:b], phit[:, r], dprm,
                       duv[a:b], dth[a:b], J=J)
        loss += l
        dloss += dl
    gpu = (res["d_params"] * direction).sum() + (res["d_uv0"] * duv).sum() + res["d_theta0"] @ dth
    np.testing.assert_allclose(res["loss"], loss, rtol=1e-9)
    np.testing.assert_allclose(gpu, dloss, rtol=1e-6)
    sim.close()

def test_bumpy_sphere_ensemble_adjoint_matches_dual_oracle(tg, orc, bumpy):
    """FP64 build, 4 steps of the 3-replica ensemble (k up to 20)."""
    mesh, om, cen, ns, ps = bumpy
    sim = tg.Simulation(mesh, ps, ns, seed=1, precision=64)
    sim.start()
    sim.step(2)
    _check_adjoint(tg, orc, om, cen, sim, ns, 1, 4, 1e-6, np.random.default_rng(8))
    sim.close()
