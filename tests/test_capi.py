"""The C-ABI library loads, exports every entry point declared in include/tds.h, and the
simulation path fails loudly (no CPU fallback) when there is no CUDA device."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "tds.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tds_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "tds_create" in names and "tds_step" in names and "tds_get_state" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(tg):
    L = tg.lib()
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing


def test_library_is_in_tree(tg):
    path = tg.library_path()
    assert path.startswith(ROOT) and os.path.exists(path)


def test_params_validation_and_no_cpu_fallback(tg, mesh_l4):
    import torch
    if torch.cuda.is_available():
        pytest.skip("this check is for hosts without a GPU")
    with pytest.raises(tg.TdsError) as e:
        tg.Simulation(mesh_l4, tg.Params(), 100)
    assert e.value.code in (1, 2)


def test_null_handles_rejected(tg):
    L = tg.lib()
    assert L.tds_start(None) == 1
    assert L.tds_step(None, 1, None) == 1
    assert L.tds_get_state(None, None) == 1
    assert L.tds_last_error(None) == b"null handle"


def _handle_without_device(tg, n):
    """A Simulation object with a particle count and no device handle: for the checks that the
    Python layer makes before it calls the library."""
    sim = object.__new__(tg.Simulation)
    sim.N, sim.R, sim.h = n, 1, None
    return sim


@pytest.mark.parametrize("who", ["get_state", "get_state_noalloc"])
def test_read_back_arrays_are_checked_before_the_call(tg, who):
    """A float32 array where the entry point writes doubles, a short array or a strided one would
    be written past its end by the library: they are refused with ValueError before any call."""
    n = 10
    sim = _handle_without_device(tg, n)
    fn = getattr(sim, who)
    good = dict(uv=np.zeros((n, 2)), theta=np.zeros(n), face=np.zeros(n, np.int32), r3d=np.zeros((n, 3)))
    for bad in (dict(good, uv=np.zeros((n - 1, 2))), dict(good, theta=np.zeros(2 * n)[::2]),
                dict(good, face=np.zeros(n, np.int64)), dict(good, r3d=np.zeros((n, 3), np.float32))):
        with pytest.raises(ValueError):
            fn(bad)
    if who == "get_state_noalloc":
        f32 = {k: (v.astype(np.float32) if v.dtype == np.float64 else v) for k, v in good.items()}
        with pytest.raises(ValueError):
            fn(f32)
