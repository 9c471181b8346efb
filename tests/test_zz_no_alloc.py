"""The allocation-free norm entry point, called through the C ABI and checked against the
context's own norms (wb_norms).

Callers whose device memory is all owned by their own pool or by another runtime, or
whose time loop must not take the device-wide synchronisation of cudaMalloc/cudaFree,
cannot allocate where they need error norms; wb_norms_device_noalloc serves them from a
fixed scratch array inside the library.  This file is collected last, so a run that stops
at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from helpers import base_cfg, random_delta, solver

pytestmark = pytest.mark.gpu


def _entry(wb):
    f = wb.lib().wb_norms_device_noalloc
    f.argtypes = ([ctypes.c_int32] * 4 + [ctypes.c_double] * 2 + [ctypes.c_void_p] * 2 +
                  [ctypes.c_size_t, ctypes.c_void_p] + [ctypes.c_void_p] * 3)
    f.restype = ctypes.c_int32
    return f


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_noalloc_norms_match_context_norms(wb):
    f = _entry(wb)
    c = base_cfg(nx=40, ny=24, order=2, basis=1, limiter=0, bc_x=0)
    with solver(wb, c, 0) as a, solver(wb, c, 0) as b:
        a.upload(random_delta(c, seed=31))
        b.upload(random_delta(c, seed=32))
        r1, rinf, r2 = a.compute_error(b)       # the context path (its own scratch)
        s1, sinf, s2 = a.compute_error(None)
        pa, plane = a.device_state()
        pb, _ = b.device_state()
        for _ in range(2):  # consecutive calls reuse the same fixed scratch
            l1, linf, l2 = np.zeros(4), np.zeros(4), np.zeros(4)
            rc = f(c["nx"], c["ny"], c["order"], c["basis"], c["lx"], c["ly"], pa, pb, plane,
                   None, _ptr(l1), _ptr(linf), _ptr(l2))
            assert rc == wb.WB_OK
            np.testing.assert_allclose(l1, r1, rtol=1e-13)
            np.testing.assert_allclose(linf, rinf, rtol=1e-13)
            np.testing.assert_allclose(l2, r2, rtol=1e-13)
            # b = NULL gives the norms of a alone
            rc = f(c["nx"], c["ny"], c["order"], c["basis"], c["lx"], c["ly"], pa, None, plane,
                   None, _ptr(l1), _ptr(linf), _ptr(l2))
            assert rc == wb.WB_OK
            np.testing.assert_allclose(l1, s1, rtol=1e-13)
            np.testing.assert_allclose(linf, sinf, rtol=1e-13)
            np.testing.assert_allclose(l2, s2, rtol=1e-13)


def test_noalloc_rejects_grids_beyond_its_scratch(wb):
    f = _entry(wb)
    c = base_cfg(nx=8, ny=8, order=1, basis=1)
    with solver(wb, c, 0) as a:
        pa, plane = a.device_state()
        l1, linf, l2 = np.zeros(4), np.zeros(4), np.zeros(4)
        # 4096 x 2048 cells exceed WB_NORMS_NOALLOC_MAX_CELLS: rejected before any launch
        rc = f(4096, 2048, 1, 1, 1.0, 1.0, pa, None, 4096 * 2048, None, _ptr(l1), _ptr(linf),
               _ptr(l2))
        assert rc == wb.WB_ERR_ARG


def test_noalloc_at_its_largest_partial_array_on_a_stream(wb):
    """2048 x 2048 cells fill all 16,384 partial slots of the fixed scratch; the call runs on
    the context's own (non-default) stream, twice in a row, against wb_norms."""
    f = _entry(wb)
    c = base_cfg(nx=2048, ny=2048, order=1, basis=1, limiter=0, bc_x=0)
    with solver(wb, c, 0) as a, solver(wb, c, 0) as b:
        a.init_perturbation(wb.seeded_multimode(5, 16, 1e-2, 8))
        b.init_perturbation(wb.seeded_gaussian_bump(3, 1e-1, 0.05))
        r1, rinf, r2 = a.compute_error(b)
        pa, plane = a.device_state()
        pb, _ = b.device_state()
        for _ in range(2):
            l1, linf, l2 = np.zeros(4), np.zeros(4), np.zeros(4)
            rc = f(c["nx"], c["ny"], c["order"], c["basis"], c["lx"], c["ly"], pa, pb, plane,
                   a.stream(), _ptr(l1), _ptr(linf), _ptr(l2))
            assert rc == wb.WB_OK
            np.testing.assert_allclose(l1, r1, rtol=1e-13)
            np.testing.assert_allclose(linf, rinf, rtol=1e-13)
            np.testing.assert_allclose(l2, r2, rtol=1e-13)


def test_noalloc_rejects_narrow_grids_with_too_many_blocks(wb):
    """33 x 127000 cells are fewer than the cell limit but need 31,750 blocks of 32x8
    cells, more than the scratch's 16,384 partial slots: rejected before any launch."""
    f = _entry(wb)
    c = base_cfg(nx=8, ny=8, order=1, basis=1)
    assert 33 * 127000 <= 4194304
    with solver(wb, c, 0) as a:
        pa, _ = a.device_state()
        l1, linf, l2 = np.zeros(4), np.zeros(4), np.zeros(4)
        rc = f(33, 127000, 1, 1, 1.0, 1.0, pa, None, 33 * 127000, None, _ptr(l1), _ptr(linf),
               _ptr(l2))
        assert rc == wb.WB_ERR_ARG


def test_noalloc_refuses_a_capturing_stream(wb):
    """A call on a stream that is being captured into a graph returns WB_ERR_ARG (the call
    copies its results back and waits, which a capture does not allow) and leaves the
    capture intact: the graph still instantiates and replays."""
    torch = pytest.importorskip("torch")
    f = _entry(wb)
    c = base_cfg(nx=8, ny=8, order=1, basis=1)
    with solver(wb, c, 0) as a:
        pa, plane = a.device_state()
        l1, linf, l2 = np.zeros(4), np.zeros(4), np.zeros(4)
        x = torch.zeros(16, device="cuda:0")
        s = torch.cuda.Stream(device="cuda:0")
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            g.capture_begin()
            x.add_(1.0)
            rc = f(8, 8, 1, 1, 1.0, 1.0, pa, None, plane, ctypes.c_void_p(s.cuda_stream),
                   _ptr(l1), _ptr(linf), _ptr(l2))
            x.add_(1.0)
            g.capture_end()
        assert rc == wb.WB_ERR_ARG
        g.replay()
        torch.cuda.synchronize()
        assert float(x.sum().item()) == 32.0
