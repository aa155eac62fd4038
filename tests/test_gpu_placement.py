"""Device placement (tds_start -> k_place) against a numpy restatement of the placement rule:
face drawn with probability proportional to its 3D area (lower bound of u1 in the cumulative
area table), uniform barycentric point, polarity at angle 2 pi u4 from normalize(B - A) in the
face's tangent frame; draws from Philox4x32-10(ctr = (local index, replica, 0xFFFFFFFF, 0),
key = seed)."""
import numpy as np
import pytest

from conftest import oracle_mesh

pytestmark = pytest.mark.gpu


def _restated(orc, om, arr, n, seed, rep):
    v3, f3, uv, fuv = arr["v3"], arr["f3"], arr["uv"], arr["fuv"]
    A, B, C = v3[f3[:, 0]], v3[f3[:, 1]], v3[f3[:, 2]]
    E0, E1 = B - A, C - A
    nv = np.stack([E0[:, 1] * E1[:, 2] - E0[:, 2] * E1[:, 1], E0[:, 2] * E1[:, 0] - E0[:, 0] * E1[:, 2],
                   E0[:, 0] * E1[:, 1] - E0[:, 1] * E1[:, 0]], 1)
    nn = np.sqrt(nv[:, 0] * nv[:, 0] + nv[:, 1] * nv[:, 1] + nv[:, 2] * nv[:, 2])
    cdf = np.cumsum(0.5 * nn)
    cdf = cdf / cdf[-1]
    cdf[-1] = 1.0
    out = dict(uv=np.zeros((n, 2)), theta=np.zeros(n), face=np.zeros(n, np.int64), r3d=np.zeros((n, 3)))
    for i in range(n):
        w = orc.philox4x32_10([i, rep, 0xFFFFFFFF, 0], [seed & 0xFFFFFFFF, seed >> 32])
        u1 = ((w[0] >> 11) + 0.5) / 2097152.0
        u2, u3, u4 = (w[1] >> 8) / 16777216.0, (w[2] >> 8) / 16777216.0, (w[3] >> 8) / 16777216.0
        f = min(int(np.searchsorted(cdf, u1, side="left")), len(cdf) - 1)
        a, b, c = uv[fuv[f, 0]], uv[fuv[f, 1]], uv[fuv[f, 2]]
        s2 = np.sqrt(u2)
        p_uv = (1 - s2) * a + s2 * (1 - u3) * b + s2 * u3 * c
        J, Jp, nrm = om.face_data(f)
        e1 = E0[f] / np.linalg.norm(E0[f])
        e2 = np.cross(nrm, e1)
        phi = 2 * np.pi * u4
        p = np.cos(phi) * e1 + np.sin(phi) * e2
        out["uv"][i] = p_uv
        out["face"][i] = f
        out["r3d"][i] = om.map(f, *p_uv)
        out["theta"][i] = np.arctan2(Jp[3:] @ p, Jp[:3] @ p)
    return out


@pytest.mark.parametrize("ns", [[3000], [700, 1300]])
def test_device_placement_matches_restatement(tg, orc, mesh_l4, ns):
    om, arr = oracle_mesh(orc, mesh_l4)
    seed = 12
    params = tg.Params() if len(ns) == 1 else [tg.Params()] * len(ns)
    sim = tg.Simulation(mesh_l4, params, ns[0] if len(ns) == 1 else ns, seed=seed, precision=64)
    sim.start()
    s = sim.get_state()
    off = 0
    for rep, n in enumerate(ns):
        ref = _restated(orc, om, arr, n, seed, rep)
        sl = slice(off, off + n)
        same = s["face"][sl] == ref["face"]
        assert same.mean() > 0.999  # a draw within rounding of a table boundary may pick the neighbour
        np.testing.assert_allclose(s["uv"][sl][same], ref["uv"][same], rtol=0, atol=1e-12)
        np.testing.assert_allclose(s["r3d"][sl][same], ref["r3d"][same], rtol=0, atol=1e-12)
        dth = np.angle(np.exp(1j * (s["theta"][sl][same] - ref["theta"][same])))
        assert np.abs(dth).max() < 1e-10
        off += n
