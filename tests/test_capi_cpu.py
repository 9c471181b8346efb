"""C-ABI checks that need no GPU: the library loads, exports every symbol the header
declares, validates configurations before touching a device, and lists modes in the
oracle's order."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "wb_capi.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(wb1?d?_\w+)\s*\(", txt, re.M)))


def test_exports_every_declared_symbol(wb):
    L = wb.lib()
    syms = header_symbols()
    assert len(syms) > 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_config_validation_without_device(wb):
    L = wb.lib()
    bad = [dict(nx=0), dict(order=5), dict(basis=7), dict(gamma=1.0), dict(precision=3),
           dict(eq_kind=2, kpoly=1.0, gy=10.0), dict(tile_x=7, tile_y=3),
           # cells per thread: only with a tile, and only the compiled shapes
           dict(cells_per_thread=2),
           dict(precision=1, order=2, basis=1, tile_x=32, tile_y=16),
           dict(precision=1, order=2, basis=0, tile_x=32, tile_y=16, cells_per_thread=2),
           dict(precision=1, order=1, basis=1, tile_x=32, tile_y=32, cells_per_thread=4),
           dict(precision=0, order=1, basis=1, tile_x=32, tile_y=16, cells_per_thread=2)]
    for kw in bad:
        c = wb.default_config(**kw)
        ctx = ctypes.c_void_p()
        rc = L.wb_create(ctypes.byref(c), ctypes.byref(ctx))
        assert rc == wb.WB_ERR_CONFIG, kw
        assert len(L.wb_last_error(ctx)) > 0
        L.wb_destroy(ctx)


def test_status_strings(wb):
    L = wb.lib()
    for s in range(0, -8, -1):
        assert L.wb_status_string(s)


@pytest.mark.parametrize("order,basis", [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1)])
def test_mode_lists_match_oracle(wb, orc, order, basis):
    a, b = wb.mode_list(order, basis)
    oa, ob = orc.modes(order, basis)
    np.testing.assert_array_equal(a, oa)
    np.testing.assert_array_equal(b, ob)


def test_no_device_reports_cuda_error(wb):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(wb.WbError) as ei:
        wb.Solver(nx=8, ny=8)
    assert ei.value.status == wb.WB_ERR_CUDA
