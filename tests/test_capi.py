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
