import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on CPU")


@pytest.fixture(scope="session")
def tg():
    """The product package (name starts with a digit)."""
    return importlib.import_module("2dtissue_gb300")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


_MESHES = {}


def get_mesh(tg, level, axes):
    key = (level, tuple(axes))
    if key not in _MESHES:
        _MESHES[key] = tg.Mesh.ellipsoid(level, axes)
    return _MESHES[key]


@pytest.fixture(scope="session")
def mesh_l4(tg):
    """Level-4 icosphere scaled to the (2,1,1) ellipsoid (the 100-particle system's mesh)."""
    return get_mesh(tg, 4, (2.0, 1.0, 1.0))


def oracle_mesh(orc, mesh):
    a = mesh.arrays()
    return orc.Mesh(a["v3"], a["f3"], a["uv"], a["fuv"]), a


def place_particles(orc_mesh, arrays, n, seed):
    """Seeded area-weighted placement for CPU-only tests (numpy draws; the product's placement
    is tested on the GPU)."""
    rng = np.random.default_rng(seed)
    v3, f3, uv, fuv = arrays["v3"], arrays["f3"], arrays["uv"], arrays["fuv"]
    A, B, C = v3[f3[:, 0]], v3[f3[:, 1]], v3[f3[:, 2]]
    ar = 0.5 * np.linalg.norm(np.cross(B - A, C - A), axis=1)
    cdf = np.cumsum(ar) / ar.sum()
    f = np.minimum(np.searchsorted(cdf, rng.random(n)), len(cdf) - 1)
    s, t = np.sqrt(rng.random(n)), rng.random(n)
    w = np.stack([1 - s, s * (1 - t), s * t], 1)
    p = w[:, 0, None] * uv[fuv[f, 0]] + w[:, 1, None] * uv[fuv[f, 1]] + w[:, 2, None] * uv[fuv[f, 2]]
    r3 = np.array([orc_mesh.map(f[i], *p[i]) for i in range(n)])
    th = rng.random(n) * 2 * np.pi - np.pi
    return dict(uv=p, theta=th, face=f.astype(np.int32), r3d=r3, ids=np.arange(n, dtype=np.int32))


def face_map_residual(arrays, uv, face, r3d):
    """Per particle: the smallest barycentric coordinate of its chart position in its face's chart
    triangle, and the distance from its 3D position to the face's chart map of that position."""
    fuv, f3 = arrays["fuv"][face], arrays["f3"][face]
    a, b, c = (arrays["uv"][fuv[:, k]] for k in range(3))
    e1, e2, d = b - a, c - a, uv - a
    det = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
    w1 = (d[:, 0] * e2[:, 1] - d[:, 1] * e2[:, 0]) / det
    w2 = (e1[:, 0] * d[:, 1] - e1[:, 1] * d[:, 0]) / det
    w0 = 1 - w1 - w2
    v = arrays["v3"]
    r = w0[:, None] * v[f3[:, 0]] + w1[:, None] * v[f3[:, 1]] + w2[:, None] * v[f3[:, 2]]
    return np.minimum(np.minimum(w0, w1), w2), np.linalg.norm(r - r3d, axis=1)
