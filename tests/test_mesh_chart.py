"""Mesh generation and the unit-square UV chart (the reference's MeshCartographyLib is absent;
the chart is pinned by the gluing rule of EuclideanTiling::processPoints and by invariants)."""
import os

import numpy as np
import pytest

from conftest import get_mesh


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4])
def test_icosphere_counts(tg, level):
    m = get_mesh(tg, level, (2.0, 1.0, 1.0))
    assert m.V == 10 * 4 ** level + 2
    assert m.F == 20 * 4 ** level


def _chart_checks(m):
    a = m.arrays()
    uv, fuv, uv2v, v3, f3 = a["uv"], a["fuv"], a["uv2v"], a["v3"], a["f3"]
    # faces correspond corner by corner
    assert np.array_equal(uv2v[fuv], f3)
    # every chart triangle counter-clockwise, chart covers the unit square exactly once
    p0, p1, p2 = uv[fuv[:, 0]], uv[fuv[:, 1]], uv[fuv[:, 2]]
    a2 = (p1[:, 0] - p0[:, 0]) * (p2[:, 1] - p0[:, 1]) - (p1[:, 1] - p0[:, 1]) * (p2[:, 0] - p0[:, 0])
    assert np.all(a2 > 0)
    assert abs(0.5 * a2.sum() - 1.0) < 1e-9
    assert uv.min() >= 0 and uv.max() <= 1
    # glued twins: (s,0)<->(0,s), (1,s)<->(s,1) are the same 3D vertex
    onb = np.where((uv[:, 1] == 0) | (uv[:, 0] == 1))[0]
    lut = {(round(x, 12), round(y, 12)): uv2v[i] for i, (x, y) in enumerate(uv)}
    for i in onb:
        x, y = uv[i]
        assert lut[(round(y, 12), round(x, 12))] == uv2v[i]
    # the four corners are chart vertices
    for c in [(0, 0), (1, 0), (0, 1), (1, 1)]:
        assert (float(c[0]), float(c[1])) in lut
    # outward orientation of the 3D faces
    A, B, C = v3[f3[:, 0]], v3[f3[:, 1]], v3[f3[:, 2]]
    n = np.cross(B - A, C - A)
    assert np.all(np.einsum("ij,ij->i", n, (A + B + C) / 3 - v3.mean(0)) > 0)


@pytest.mark.parametrize("level,axes", [(2, (1, 1, 1)), (3, (2, 1, 1)), (4, (2, 1, 1)), (4, (4, 2, 2))])
def test_chart_valid(tg, level, axes):
    _chart_checks(get_mesh(tg, level, axes))


def test_bumpy_sphere_chart(tg):
    m = tg.Mesh.bumpy_sphere(3, 0.2, 5.0)
    _chart_checks(m)
    r = np.linalg.norm(m.arrays()["v3"], axis=1)
    assert r.min() < 5.0 < r.max()


def test_area_matches_ellipsoid(tg, mesh_l4):
    # area of the (2,1,1) prolate spheroid: 2 pi b^2 (1 + a/(b e) asin e), e = sqrt(1 - b^2/a^2)
    a, b = 2.0, 1.0
    e = np.sqrt(1 - b * b / (a * a))
    exact = 2 * np.pi * b * b * (1 + a / (b * e) * np.arcsin(e))
    assert abs(mesh_l4.area - exact) / exact < 5e-3


def test_off_roundtrip(tg, tmp_path):
    m = get_mesh(tg, 2, (2.0, 1.0, 1.0))
    p = os.path.join(tmp_path, "e.off")
    m.save_off(p)
    m2 = tg.Mesh.load_off(p)
    a, b = m.arrays(), m2.arrays()
    np.testing.assert_array_equal(a["f3"], b["f3"])
    np.testing.assert_allclose(a["v3"], b["v3"], rtol=0, atol=0)
    np.testing.assert_array_equal(a["uv"], b["uv"])


def test_from_arrays_and_errors(tg):
    m = get_mesh(tg, 1, (1.0, 1.0, 1.0))
    a = m.arrays()
    m2 = tg.Mesh.from_arrays(a["v3"], a["f3"])
    assert m2.F == m.F
    with pytest.raises(tg.TdsError):
        tg.Mesh.from_arrays(a["v3"], a["f3"][:-1])  # not closed
    with pytest.raises(tg.TdsError):
        tg.Mesh.load_off("/nonexistent/mesh.off")


def test_chart_is_deterministic(tg):
    a = tg.Mesh.ellipsoid(3, (2, 1, 1)).arrays()
    b = tg.Mesh.ellipsoid(3, (2, 1, 1)).arrays()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
