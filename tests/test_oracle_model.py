"""Model-form oracle: invariants of one step and its forward-mode derivative (dual numbers)
against central finite differences."""
import numpy as np
import pytest

from conftest import oracle_mesh, place_particles


@pytest.fixture(scope="module")
def setup(orc, mesh_l4, tg):
    om, arr = oracle_mesh(orc, mesh_l4)
    return om, arr, tg.Params().oracle_dict()


def test_step_keeps_particles_on_surface(orc, setup):
    om, arr, p = setup
    st = place_particles(om, arr, 300, 1)
    for step in range(20):
        out = orc.model_step(om, p, st, step, seed=3)
        assert out["status"] == 0
        assert out["uv"].min() >= 0 and out["uv"].max() <= 1
        for i in range(0, 300, 7):
            np.testing.assert_allclose(om.map(out["face"][i], *out["uv"][i]), out["r3d"][i], atol=1e-12)
            f, mode = om.locate(*out["uv"][i], out["face"][i])
            assert f == out["face"][i]
        assert np.all(np.abs(out["theta"]) <= np.pi)
        st = dict(uv=out["uv"], theta=out["theta"], face=out["face"], r3d=out["r3d"], ids=st["ids"])


def test_neighbour_count_matches_brute_force(orc, setup):
    om, arr, p = setup
    st = place_particles(om, arr, 400, 2)
    out = orc.model_step(om, p, st, 0, seed=0)
    r = st["r3d"]
    d = np.linalg.norm(r[:, None, :] - r[None, :, :], axis=2)
    np.fill_diagonal(d, np.inf)
    np.testing.assert_array_equal(out["nbr"], (d < p["r_max"]).sum(1))


def test_subset_equals_full(orc, setup):
    om, arr, p = setup
    st = place_particles(om, arr, 500, 3)
    full = orc.model_step(om, p, st, 5, seed=9)
    sub = np.array([3, 77, 150, 499], np.int32)
    part = orc.model_step(om, p, st, 5, seed=9, subset=sub)
    for k in ("uv", "theta", "face", "r3d", "nbr"):
        np.testing.assert_array_equal(part[k], full[k][sub])


def test_injected_noise_equals_philox(orc, setup):
    """The Philox draw is u = (word0 >> 8) / 2^24, xi = eta (u - 1/2); injecting exactly that
    increment gives the same step."""
    om, arr, p = setup
    st = place_particles(om, arr, 50, 4)
    step, seed = 7, 11
    xi = np.zeros(50)
    for i in range(50):
        w = orc.philox4x32_10([step, 0, i, 0], [seed, 0])[0]
        xi[i] = p["eta"] * ((w >> 8) / 16777216.0 - 0.5)
    a = orc.model_step(om, p, st, step, seed=seed)
    b = orc.model_step(om, p, st, step, seed=seed, noise=xi)
    np.testing.assert_allclose(a["theta"], b["theta"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(a["uv"], b["uv"], rtol=0, atol=0)


def test_dual_numbers_match_central_differences(orc, setup):
    """Forward-mode tangent of one step vs FP64 central differences (h = 1e-6) on particles
    whose neighbour set, face and wraps do not change within +-h."""
    om, arr, p = setup
    st = place_particles(om, arr, 200, 5)
    rng = np.random.default_rng(0)
    duv = rng.normal(size=(200, 2)) * 1e-2
    dth = rng.normal(size=200)
    dr3 = np.zeros((200, 3))
    # tangent of r3d consistent with duv through the face map
    for i in range(200):
        J, _, _ = om.face_data(st["face"][i])
        dr3[i] = J[:3] * duv[i, 0] + J[3:] * duv[i, 1]
    dprm = dict((k, 0.0) for k in p)
    dprm["v0"] = 0.3
    dprm["k"] = 1.0
    dprm["tau"] = -0.2
    dprm["align"] = 0.4
    out = orc.model_step_dual(om, p, dprm, st, dict(uv=duv, theta=dth, r3d=dr3), 0, seed=1)
    h = 1e-6

    def run(sign):
        q = {k: p[k] + sign * h * dprm[k] for k in p}
        s2 = dict(uv=st["uv"] + sign * h * duv, theta=st["theta"] + sign * h * dth,
                  face=st["face"], r3d=st["r3d"] + sign * h * dr3, ids=st["ids"])
        return orc.model_step(om, q, s2, 0, seed=1)

    a, b = run(+1), run(-1)
    ok = (a["face"] == b["face"]) & (a["face"] == out["face"]) & (a["nbr"] == b["nbr"]) & (a["wraps"] == b["wraps"])
    assert ok.sum() > 150
    fd_uv = (a["uv"] - b["uv"]) / (2 * h)
    fd_r3 = (a["r3d"] - b["r3d"]) / (2 * h)
    dth_fd = np.angle(np.exp(1j * (a["theta"] - b["theta"]))) / (2 * h)
    np.testing.assert_allclose(out["duv"][ok], fd_uv[ok], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(out["dr3d"][ok], fd_r3[ok], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(out["dtheta"][ok], dth_fd[ok], rtol=1e-5, atol=1e-6)
