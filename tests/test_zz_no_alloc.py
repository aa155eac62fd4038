"""State read-back without device allocation (tds_get_state_noalloc).

For callers that cannot allocate device memory where they read the state back (a framework that
owns all device memory, a fixed memory budget, a loop that must not synchronise on cudaMalloc):
the entry point stages the state in the library's fixed 16 MiB device array. This file is named so
that pytest collects it last; it must also pass alone in a fresh process.
"""
import numpy as np
import pytest

from conftest import get_mesh

pytestmark = pytest.mark.gpu


def _assert_same(a, b):
    # both calls run the same gather kernel on the same device state: identical results
    for k in ("uv", "theta", "face", "r3d", "vel_uv", "nbr"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("precision", [32, 64])
def test_noalloc_read_back_matches_get_state_on_two_calls(tg, precision):
    mesh = get_mesh(tg, 4, (2.0, 1.0, 1.0))
    sim = tg.Simulation(mesh, tg.Params(), 3000, seed=21, precision=precision)
    sim.start()
    sim.step(3)
    first = sim.get_state_noalloc()
    _assert_same(first, sim.get_state())
    sim.step(2)  # the state changes; the shared array keeps the previous call's contents
    second = sim.get_state_noalloc()
    _assert_same(second, sim.get_state())
    assert not np.array_equal(first["uv"], second["uv"])


def test_noalloc_rejects_sizes_above_the_fixed_staging(tg):
    mesh = get_mesh(tg, 4, (2.0, 1.0, 1.0))
    sim = tg.Simulation(mesh, tg.Params(radius=0.004, r_max=0.0096), 233017, seed=2)
    with pytest.raises(tg.TdsError) as e:
        sim.get_state_noalloc()
    assert e.value.code == 6 and "233016" in str(e.value)
