"""The hand-written adjoint (tds_adjoint_run) against the FP64 oracle: the directional derivative
of the loss along a random direction of (parameters, initial uv, initial theta) from the chained
forward-mode dual-number oracle step, and FP64 central differences (h = 1e-6) of the oracle's loss.

Loss = w_pos * mean_i |r_T,i - r*_i|^2 + w_phi * sum_t (phi_t - phi*_t)^2 over T steps."""
import importlib

import numpy as np
import pytest

from conftest import oracle_mesh

pytestmark = pytest.mark.gpu

N = 1500  # dense (area packing 0.55): an ill-conditioned, strongly interacting system
T = 6
SEED = 5
# tds_adjoint_result.d_params columns -> oracle parameter names
GRAD_TO_ORACLE = dict(k_rep="k", k_adh="k_adh", v0="v0", mu="mu", tau="tau", align="align", eta="eta")


def _tangent_r3(om, face, duv):
    dr = np.zeros((len(face), 3))
    for i, f in enumerate(face):
        J, _, _ = om.face_data(int(f))
        dr[i] = J[:3] * duv[i, 0] + J[3:] * duv[i, 1]
    return dr


def _oracle_chain(orc, om, cen, prm, state, t0, dprm=None, duv=None, dth=None, tgt=None, phit=None,
                  w_pos=1.0, w_phi=1.0, T=T, decisions=None):
    """Loss of T oracle steps from `state`; with tangents, also its directional derivative.
    decisions (a list) collects each step's faces, neighbour counts and wrap counts."""
    n = len(state["theta"])
    st = dict(uv=state["uv"].copy(), theta=state["theta"].copy(), face=state["face"].copy(),
              r3d=state["r3d"].copy(), ids=np.arange(n, dtype=np.int32))
    dual = dprm is not None
    if dual:
        ds = dict(uv=duv.copy(), theta=dth.copy(), r3d=_tangent_r3(om, st["face"], duv))
    loss, dloss = 0.0, 0.0
    for t in range(T):
        if dual:
            out = orc.model_step_dual(om, prm, dprm, st, ds, t0 + t, SEED, centroid=cen)
        else:
            out = orc.model_step(om, prm, st, t0 + t, SEED, centroid=cen)
        if decisions is not None:
            decisions.append(np.concatenate([out["face"], out["nbr"], out["wraps"]]))
        S = out["phi_sums"][:3]
        phi = np.linalg.norm(S) / n
        loss += w_phi * (phi - phit[t]) ** 2
        if dual:
            dphi = S @ out["dphi_sums"][:3] / (np.linalg.norm(S) * n)
            dloss += w_phi * 2 * (phi - phit[t]) * dphi
            ds = dict(uv=out["duv"], theta=out["dtheta"], r3d=out["dr3d"])
        st = dict(uv=out["uv"], theta=out["theta"], face=out["face"], r3d=out["r3d"], ids=st["ids"])
    d = st["r3d"] - tgt
    loss += w_pos * (d * d).sum() / n
    if dual:
        dloss += w_pos * 2 * (d * ds["r3d"]).sum() / n
    return loss, dloss


@pytest.fixture(scope="module")
def adj_setup(tg, orc, mesh_l4):
    om, arr = oracle_mesh(orc, mesh_l4)
    return om, arr["v3"].mean(0)


def _start(tg, mesh, precision, params=None, n=N):
    sim = tg.Simulation(mesh, params or tg.Params(), n, seed=SEED, precision=precision)
    sim.start()
    sim.step(2)
    return sim


@pytest.mark.parametrize("precision,n,rtol", [(64, N, 1e-6), (64, 200, 1e-8), (32, 200, 2e-3)])
def test_adjoint_matches_dual_number_oracle(tg, orc, mesh_l4, adj_setup, precision, n, rtol):
    """FP64: dense and sparse systems. FP32 on the sparse one (the 100-particle system's density), where an FP32
    trajectory stays close to the FP64 one; in the dense system single particles reach
    sensitivities of 1e3-1e4 and FP32 and FP64 trajectories part."""
    N = n
    om, cen = adj_setup
    sim = _start(tg, mesh_l4, precision, n=n)
    s0 = sim.get_state()
    t0 = sim.step_count
    rng = np.random.default_rng(1)
    tgt = s0["r3d"] + 0.01 * rng.normal(size=(N, 3))
    phit = np.full(T, 0.3)
    res = sim.adjoint(T, r3d_target=tgt, w_pos=1.0, phi_target=phit, w_phi=1.0)
    prm = sim.params[0].oracle_dict()
    dprm = {k: 0.0 for k in prm}
    direction = rng.normal(size=len(tg.GRAD_PARAMS))
    for j, name in enumerate(tg.GRAD_PARAMS):
        dprm[GRAD_TO_ORACLE[name]] = direction[j]
    duv = 1e-2 * rng.normal(size=(N, 2))
    dth = rng.normal(size=N)
    loss, dloss = _oracle_chain(orc, om, cen, prm, s0, t0, dprm, duv, dth, tgt, phit)
    gpu = res["d_params"][0] @ direction + (res["d_uv0"] * duv).sum() + res["d_theta0"] @ dth
    np.testing.assert_allclose(res["loss"], loss, rtol=1e-9 if precision == 64 else 5e-3)  # FP32: a free-running trajectory
    np.testing.assert_allclose(gpu, dloss, rtol=rtol)
    # each parameter on its own
    for j, name in enumerate(tg.GRAD_PARAMS):
        dp = {k: 0.0 for k in prm}
        dp[GRAD_TO_ORACLE[name]] = 1.0
        _, dl = _oracle_chain(orc, om, cen, prm, s0, t0, dp, np.zeros((N, 2)), np.zeros(N), tgt, phit)
        atol = 1e-9 * max(1.0, abs(dl)) if precision == 64 else rtol * np.abs(res["d_params"][0]).max()
        np.testing.assert_allclose(res["d_params"][0, j], dl, rtol=rtol, atol=atol, err_msg=name)


def test_adjoint_matches_central_differences(tg, orc, mesh_l4, adj_setup):
    """FP64 central differences of the oracle's loss, h = 1e-6, per parameter, where the +h and -h
    runs take the same discrete decisions (faces, neighbour sets, wraps): the model is piecewise
    smooth (the polarity follows the face's chart map, the adhesion force ends at r_max with a jump)
    and a difference quotient across a jump measures the jump, not the derivative."""
    om, cen = adj_setup
    n, steps = 400, 4
    sim = _start(tg, mesh_l4, 64, n=n)
    s0 = sim.get_state()
    t0 = sim.step_count
    tgt = s0["r3d"] + 0.01
    phit = np.full(steps, 0.2)
    res = sim.adjoint(steps, r3d_target=tgt, w_pos=1.0, phi_target=phit, w_phi=1.0)
    prm = sim.params[0].oracle_dict()
    checked = 0
    for j, name in enumerate(tg.GRAD_PARAMS):
        k = GRAD_TO_ORACLE[name]
        for h in (1e-6, 1e-7):
            hi, lo = dict(prm), dict(prm)
            hi[k] += h
            lo[k] -= h
            da, db = [], []
            la = _oracle_chain(orc, om, cen, hi, s0, t0, tgt=tgt, phit=phit, T=steps, decisions=da)[0]
            lb = _oracle_chain(orc, om, cen, lo, s0, t0, tgt=tgt, phit=phit, T=steps, decisions=db)[0]
            if all(np.array_equal(x, y) for x, y in zip(da, db)):
                fd = (la - lb) / (2 * h)
                np.testing.assert_allclose(res["d_params"][0, j], fd, rtol=1e-4 if h == 1e-6 else 1e-3, atol=1e-7,
                                           err_msg=name)
                checked += 1
                break
    assert checked >= 6


def test_checkpoint_stride_does_not_change_the_gradient(tg, mesh_l4):
    outs = []
    for K in (1, 4, 0):
        sim = _start(tg, mesh_l4, 32)
        s0 = sim.get_state()
        outs.append(sim.adjoint(T + 3, r3d_target=s0["r3d"], w_pos=1.0, phi_target=np.zeros(T + 3), w_phi=1.0,
                                checkpoint_stride=K))
        after = sim.get_state()
        ref = _start(tg, mesh_l4, 32)
        ref.step(T + 3)
        np.testing.assert_array_equal(after["uv"], ref.get_state()["uv"])  # handle ends as after tds_step
    assert outs[0]["checkpoint_stride"] == 1 and outs[1]["checkpoint_stride"] == 4
    for o in outs[1:]:
        for k in ("loss", "d_params", "d_uv0", "d_theta0"):
            np.testing.assert_array_equal(outs[0][k], o[k])


def test_ensemble_adjoint_is_per_replica(tg, mesh_l4):
    """Without noise, replica r of an ensemble has the gradients of the same system run alone."""
    ps = [tg.Params(eta=0.0, v0=0.8), tg.Params(eta=0.0, v0=1.3, k_rep=12.0)]
    ns = [700, 900]
    singles, states = [], []
    for r in range(2):
        a = tg.Simulation(mesh_l4, ps[r], ns[r], seed=10 + r, precision=64)
        a.start()
        states.append(a.get_state())
        singles.append(a.adjoint(4, r3d_target=states[r]["r3d"], w_pos=1.0, phi_target=np.full(4, 0.1), w_phi=1.0))
    e = tg.Simulation(mesh_l4, ps, ns, seed=3, precision=64)
    cat = {k: np.concatenate([states[0][k], states[1][k]]) for k in ("uv", "theta", "face", "r3d")}
    e.set_state(**cat)
    res = e.adjoint(4, r3d_target=cat["r3d"], w_pos=1.0, phi_target=np.full((4, 2), 0.1), w_phi=1.0)
    np.testing.assert_allclose(res["loss"], singles[0]["loss"] + singles[1]["loss"], rtol=1e-12)
    off = [0, ns[0], ns[0] + ns[1]]
    for r in range(2):
        # all but eta: its term weighs the noise draws, which depend on the replica index
        np.testing.assert_allclose(res["d_params"][r, :6], singles[r]["d_params"][0, :6], rtol=1e-10, atol=1e-14)
        np.testing.assert_allclose(res["d_uv0"][off[r]:off[r + 1]], singles[r]["d_uv0"], rtol=1e-10, atol=1e-14)


def test_autograd_function(tg, mesh_l4):
    torch = pytest.importorskip("torch")
    ag = importlib.import_module("2dtissue_gb300.autograd")
    sim = _start(tg, mesh_l4, 64)
    s0 = sim.get_state()
    base = sim.params[0]
    params = torch.tensor([[getattr(base, k) for k in tg.GRAD_PARAMS]], dtype=torch.float64, requires_grad=True)
    uv0 = torch.tensor(s0["uv"], requires_grad=True)
    th0 = torch.tensor(s0["theta"], requires_grad=True)
    loss = ag.TissueLoss.apply(params, uv0, th0, sim, s0["face"], 3, s0["r3d"], 1.0, np.zeros(3), 1.0)
    (2.0 * loss).backward()
    # the same run through the C-ABI directly, on a handle with the same step counter (noise)
    ref = _start(tg, mesh_l4, 64)
    ref.set_state(s0["uv"], s0["theta"], face=s0["face"])
    out = ref.adjoint(3, r3d_target=s0["r3d"], w_pos=1.0, phi_target=np.zeros(3), w_phi=1.0)
    np.testing.assert_allclose(loss.item(), out["loss"], rtol=1e-12)
    np.testing.assert_allclose(params.grad.numpy()[0], 2.0 * out["d_params"][0], rtol=1e-12)
    np.testing.assert_allclose(uv0.grad.numpy(), 2.0 * out["d_uv0"], rtol=1e-12, atol=1e-300)


def test_repeated_adjoint_calls_reuse_the_work_memory(tg, mesh_l4):
    """The handle keeps the adjoint's work memory between calls: a repeated call, a longer call
    (the block grows) and a call after tds_adjoint_release give the same gradients as the first.
    No noise (eta = 0): each call starts from the same state but at a later step counter."""
    sim = _start(tg, mesh_l4, 32, params=tg.Params(eta=0.0))
    s0 = sim.get_state()

    def run(steps):
        sim.set_state(s0["uv"], s0["theta"], s0["face"])
        return sim.adjoint(steps, r3d_target=s0["r3d"], w_pos=1.0, phi_target=np.zeros(steps), w_phi=1.0,
                           checkpoint_stride=2)

    first = run(T)
    again = run(T)
    longer = run(T + 4)
    after_longer = run(T)
    sim.adjoint_release()
    released = run(T)
    assert longer["d_params"].shape == first["d_params"].shape
    for o in (again, after_longer, released):
        for k in ("loss", "d_uv0", "d_theta0"):
            np.testing.assert_array_equal(first[k], o[k])
        # all but eta: dL/d eta weighs the noise draws, which follow the step counter
        np.testing.assert_array_equal(first["d_params"][:, :6], o["d_params"][:, :6])


@pytest.mark.parametrize("precision", [64, 32])
def test_windowed_adjoint_is_the_adjoint_of_its_window(tg, mesh_l4, precision):
    """window = W < n_steps: the run takes n_steps - W steps forward only, then the adjoint of the
    last W steps (a truncated gradient). It equals, bit for bit, a plain adjoint of W steps started
    after the same forward steps; the loss adds the earlier steps' order-parameter terms."""
    T, W = 10, 4
    a = _start(tg, mesh_l4, precision, n=400)
    b = _start(tg, mesh_l4, precision, n=400)
    s0 = a.get_state()
    tgt = s0["r3d"] + 0.01
    phit = np.linspace(0.1, 0.3, T)
    ra = a.adjoint(T, r3d_target=tgt, w_pos=1.0, phi_target=phit, w_phi=1.0, window=W)
    b.step(T - W)
    pre = b.order_parameter()[0][-(T - W):, 0]
    rb = b.adjoint(W, r3d_target=tgt, w_pos=1.0, phi_target=phit[T - W:], w_phi=1.0)
    for k in ("d_params", "d_uv0", "d_theta0"):
        np.testing.assert_array_equal(ra[k], rb[k], err_msg=k)
    np.testing.assert_allclose(ra["loss"], rb["loss"] + ((pre - phit[:T - W]) ** 2).sum(), rtol=1e-12)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        np.testing.assert_array_equal(sa[k], sb[k])
    # a window covering the whole run is the exact gradient
    c = _start(tg, mesh_l4, precision, n=400)
    d = _start(tg, mesh_l4, precision, n=400)
    rc = c.adjoint(T, r3d_target=tgt, w_pos=1.0, phi_target=phit, w_phi=1.0, window=T)
    rd = d.adjoint(T, r3d_target=tgt, w_pos=1.0, phi_target=phit, w_phi=1.0)
    np.testing.assert_array_equal(rc["d_params"], rd["d_params"])


def test_gather_lanes_agree(tg, orc, mesh_l4, adj_setup):
    """The reverse neighbour gather with one and with four lanes per particle (the choice by system
    size, or the caller's): the same gradients to rounding (FP64), each equal to the dual-number
    oracle's directional derivative, each deterministic; other widths are refused."""
    om, cen = adj_setup
    res = {}
    for lanes in (1, 4):
        sim = _start(tg, mesh_l4, 64)
        s0 = sim.get_state()
        tgt = s0["r3d"] + 0.01
        phit = np.full(T, 0.3)
        res[lanes] = [sim.adjoint(T, r3d_target=tgt, w_pos=1.0, phi_target=phit, w_phi=1.0, gather_lanes=lanes)]
        sim2 = _start(tg, mesh_l4, 64)
        res[lanes].append(sim2.adjoint(T, r3d_target=tgt, w_pos=1.0, phi_target=phit, w_phi=1.0,
                                       gather_lanes=lanes))
    for lanes in (1, 4):
        for k in ("d_params", "d_uv0", "d_theta0"):
            np.testing.assert_array_equal(res[lanes][0][k], res[lanes][1][k], err_msg=k)
    for k in ("d_params", "d_uv0", "d_theta0"):
        np.testing.assert_allclose(res[1][0][k], res[4][0][k], rtol=1e-9, atol=1e-12 * np.abs(res[1][0][k]).max(),
                                   err_msg=k)
    # the default (by size: four lanes at this size) is the four-lane gather
    sim = _start(tg, mesh_l4, 64)
    s0 = sim.get_state()
    r0 = sim.adjoint(T, r3d_target=s0["r3d"] + 0.01, w_pos=1.0, phi_target=np.full(T, 0.3), w_phi=1.0)
    np.testing.assert_array_equal(r0["d_uv0"], res[4][0]["d_uv0"])
    # against the oracle's directional derivative along a random parameter direction
    rng = np.random.default_rng(3)
    prm = sim.params[0].oracle_dict()
    direction = rng.normal(size=len(tg.GRAD_PARAMS))
    dprm = {k: 0.0 for k in prm}
    for j, name in enumerate(tg.GRAD_PARAMS):
        dprm[GRAD_TO_ORACLE[name]] = direction[j]
    _, dl = _oracle_chain(orc, om, cen, prm, s0, 2, dprm, np.zeros((N, 2)), np.zeros(N), s0["r3d"] + 0.01,
                          np.full(T, 0.3))
    for lanes in (1, 4):
        np.testing.assert_allclose(res[lanes][0]["d_params"][0] @ direction, dl, rtol=1e-6)
    with pytest.raises(tg.TdsError):
        sim.adjoint(T, r3d_target=s0["r3d"], w_pos=1.0, gather_lanes=2)


@pytest.mark.parametrize("lanes", [2, 4])
def test_adjoint_with_lanes_per_particle(tg, orc, mesh_l4, adj_setup, lanes):
    """A handle whose step kernel runs 2 or 4 lanes per particle: its stored steps keep the pair
    sums those lanes computed, and the reverse sweep uses them; the gradient matches the
    dual-number oracle (FP64, the dense system) and the run is deterministic."""
    om, cen = adj_setup
    tun = dict(cells_per_particle=4.0, step_block=128, graph_steps=0, lanes_per_particle=lanes)
    outs = []
    for _ in range(2):
        sim = tg.Simulation(mesh_l4, tg.Params(), N, seed=SEED, precision=64, tuning=tun)
        sim.start()
        sim.step(2)
        s0 = sim.get_state()
        t0 = sim.step_count
        tgt = s0["r3d"] + 0.01
        phit = np.full(T, 0.3)
        outs.append(sim.adjoint(T, r3d_target=tgt, w_pos=1.0, phi_target=phit, w_phi=1.0, checkpoint_stride=4))
    for k in ("loss", "d_params", "d_uv0", "d_theta0"):
        np.testing.assert_array_equal(outs[0][k], outs[1][k], err_msg=k)
    rng = np.random.default_rng(7)
    prm = sim.params[0].oracle_dict()
    direction = rng.normal(size=len(tg.GRAD_PARAMS))
    dprm = {k: 0.0 for k in prm}
    for j, name in enumerate(tg.GRAD_PARAMS):
        dprm[GRAD_TO_ORACLE[name]] = direction[j]
    duv = 1e-2 * rng.normal(size=(N, 2))
    dth = rng.normal(size=N)
    loss, dloss = _oracle_chain(orc, om, cen, prm, s0, t0, dprm, duv, dth, tgt, phit)
    res = outs[0]
    gpu = res["d_params"][0] @ direction + (res["d_uv0"] * duv).sum() + res["d_theta0"] @ dth
    np.testing.assert_allclose(res["loss"], loss, rtol=1e-9)
    np.testing.assert_allclose(gpu, dloss, rtol=1e-6)


def test_kernel_timing_changes_no_result(tg, mesh_l4):
    """With per-kernel timing on, steps and the adjoint's segments launch kernel by kernel between
    CUDA events instead of as graphs: the same state and gradients bit for bit, and every launch of
    the four step kernels counted."""
    outs = []
    for timing in (False, True):
        sim = _start(tg, mesh_l4, 32)
        s0 = sim.get_state()
        sim.kernel_timing(timing)
        sim.step(5)
        sim.step(1)
        r = sim.adjoint(T + 3, r3d_target=s0["r3d"], w_pos=1.0, phi_target=np.zeros(T + 3), w_phi=1.0,
                        checkpoint_stride=4)
        outs.append((sim.get_state(), r))
        if timing:
            kt = sim.kernel_times()
            n = kt["step"][1]
            # 6 plain steps, the forward's T + 3 and the recompute of the two earlier segments
            assert n == 6 + (T + 3) + 8
            assert kt["scan"][1] == kt["scatter"][1] == kt["order"][1] == n
            assert all(ms > 0 for ms, c in kt.values() if c)
        sim.close()
    for k in ("uv", "theta", "face", "r3d"):
        np.testing.assert_array_equal(outs[0][0][k], outs[1][0][k])
    for k in ("loss", "d_params", "d_uv0", "d_theta0"):
        np.testing.assert_array_equal(outs[0][1][k], outs[1][1][k])
