"""Checkpoint/restart and the reference's text snapshot format, on the GPU."""
import numpy as np
import pytest

from helpers import base_cfg, orc_cfg, random_delta, solver, violating_delta

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("limiter", [0, 1, 2])
def test_restart_is_bitwise(wb, tmp_path, precision, limiter):
    c = base_cfg(nx=20, ny=16, order=2, basis=1, limiter=limiter, bc_x=0)
    # rough data only with the limiter on (unlimited P2 steps of rough data go non-physical);
    # the positivity limiter gets a state that violates positivity, and fixed steps
    if limiter == 2:
        d = violating_delta(c, seed=4, ncells=6, depth=1.0)
        dt = 2e-4
    else:
        d = random_delta(c, amp=3e-2 if limiter else 5e-3, seed=4, smooth=not limiter)
        dt = -1.0
    with solver(wb, c, precision) as a:
        a.upload(d)
        a.step(10, dt)
        ref = a.download()
        tref, nref = a.time()
    with solver(wb, c, precision) as b:
        b.upload(d)
        b.step(5, dt)
        b.save_checkpoint(str(tmp_path / "ck.bin"))
    r = wb.Solver.from_checkpoint(str(tmp_path / "ck.bin"))
    r.step(5, dt)
    got = r.download()
    t, n = r.time()
    r.close()
    assert n == nref and t == tref
    np.testing.assert_array_equal(got, ref)


def test_output_file_format(wb, orc, tmp_path):
    c = base_cfg(nx=6, ny=5, order=1, basis=0, eq_kind=1)
    d = random_delta(c, amp=1e-2, seed=8)
    with solver(wb, c, 0) as s:
        s.upload(d)
        s.output_file(str(tmp_path / "snap.dat"), var=1)
        dl = s.download()
    lines = open(tmp_path / "snap.dat").read().splitlines()
    assert len(lines) == 30
    for ln in lines:
        assert len(ln) == 6 * 13 - 1  # six values of 12 columns, one blank between them
    oc = orc_cfg(c)
    nodes = orc.nodes_from_modes(oc, dl)
    x, _ = orc.gl(2)
    k = 0
    for i in range(6):          # x index outer, y index inner, as output_file loops
        for j in range(5):
            vals = [float(v) for v in lines[k].split()]
            xq = (i + 0.5) / 6 + 0.5 / 6 * x[0]
            yq = (j + 0.5) / 5 + 0.5 / 5 * x[0]
            re, pe = orc.eq_at(oc, xq, yq)
            u = nodes[:, 0, j, i] + np.array([re, 0, 0, pe / 0.4])
            w = [u[0] - re, u[1] / u[0], u[2] / u[0],
                 0.4 * (u[3] - 0.5 * (u[1] ** 2 + u[2] ** 2) / u[0]) - pe]
            np.testing.assert_allclose(vals, [xq, yq] + w, rtol=1e-5, atol=1e-16)
            k += 1


def test_autotune_preserves_state(wb, tmp_path, monkeypatch):
    monkeypatch.setenv("WB_TILE_CACHE", str(tmp_path / "tiles.txt"))
    c = base_cfg(nx=64, ny=48, order=2, basis=1, limiter=1)
    d = random_delta(c, amp=1e-2, seed=12)
    with solver(wb, c, 1) as s:
        s.upload(d)
        s.step(2)
        before = s.download()
        t0 = s.time()
        tx, ty, cpt = s.autotune(2)
        assert (tx, ty, cpt) in [(32, 8, 1), (16, 16, 1), (32, 16, 2)]
        np.testing.assert_array_equal(s.download(), before)
        assert s.time() == t0
    lines = open(tmp_path / "tiles.txt").read().split()
    assert [int(v) for v in lines[-3:]] == [tx, ty, cpt]
    with solver(wb, c, 1) as s2:   # a new context picks the cached shape up
        s2.upload(d)
        assert s2.autotune(1) in [(32, 8, 1), (16, 16, 1), (32, 16, 2)]


def test_step_io_pipeline_matches_sync_calls(wb):
    """wb_step_io_f32 (pipelined upload / steps / download) gives, call for call, what
    upload + step + download give."""
    import torch
    c = base_cfg(nx=40, ny=24, order=2, basis=1, eq_kind=1, limiter=1, bc_x=0)
    n = 3
    ins = [random_delta(c, amp=1e-2, seed=20 + k).astype(np.float32) for k in range(n)]
    with solver(wb, c, 1) as a, solver(wb, c, 1) as b:
        dof = a.dofs
        hin = [torch.from_numpy(x.reshape(-1).copy()).pin_memory() for x in ins]
        hout = [torch.empty(dof, dtype=torch.float32, pin_memory=True) for _ in range(n)]
        for k in range(n):
            a.step_io_f32_ptr(hin[k].data_ptr(), hout[k].data_ptr(), 2, 1e-3)
        a.sync()
        for k in range(n):
            b.upload_f32(ins[k])
            b.step(2, 1e-3)
            ref = b.download_f32()
            np.testing.assert_array_equal(hout[k].numpy().reshape(ref.shape), ref)
        ta, na = a.time()
        tb, nb = b.time()
        assert na == nb == 2 * n and ta == tb


@pytest.mark.parametrize("precision", [0, 1])
def test_bounded_wait_reports_timeout_and_context_survives(wb, precision):
    """Failure detection without a fault: the staging's mbarrier wait on a barrier that
    nothing completes gives up after its poll limit, the host reads WB_ERR_TIMEOUT, and
    the context keeps working."""
    c = base_cfg(nx=48, ny=40, order=2, basis=1, eq_kind=1)
    d = random_delta(c, amp=1e-2, seed=3)
    with solver(wb, c, precision) as s, solver(wb, c, precision) as ref:
        assert s.selftest_wait_timeout(4096) == wb.WB_ERR_TIMEOUT
        s.upload(d)
        ref.upload(d)
        s.step(3)
        ref.step(3)
        s.sync()
        np.testing.assert_array_equal(s.download(), ref.download())


@pytest.mark.parametrize("precision", [0, 1])
def test_set_equilibrium_matches_fresh_context(wb, precision):
    """wb_set_equilibrium swaps the equilibrium tables in place: steps after the switch are
    bit for bit those of a context created with the new equilibrium, and a zero
    perturbation of the new equilibrium stays at rest."""
    c0 = base_cfg(nx=40, ny=24, order=2, basis=1, eq_kind=1, gx=1.0, gy=1.0, limiter=1)
    c1 = dict(c0, eq_kind=2, gx=0.3, gy=-0.7, rho0=1.2, p0=0.9, kpoly=0.8)
    d = random_delta(c0, amp=1e-2, seed=31)
    with solver(wb, c0, precision) as a, solver(wb, c1, precision) as b:
        a.upload(d)
        a.step(2, 1e-3)
        a.set_equilibrium(2, 0.3, -0.7, rho0=1.2, p0=0.9, kpoly=0.8)
        assert (a.cfg.eq_kind, a.cfg.gx, a.cfg.rho0) == (2, 0.3, 1.2)
        mid = a.download()
        b.upload(mid)
        a.step(3, 1e-3)
        b.step(3, 1e-3)
        np.testing.assert_array_equal(a.download(), b.download())
        a.upload(np.zeros_like(d))
        a.step(4)
        assert np.abs(a.download()).max() < (1e-5 if precision else 1e-12)
        with pytest.raises(RuntimeError):
            a.set_equilibrium(7, 0.0, 0.0)
        assert a.cfg.eq_kind == 2   # a rejected call changes nothing


@pytest.mark.parametrize("var", [1, 3])
def test_output_file_round_trip_2d(wb, orc, tmp_path, var):
    """output_file -> wb_read_dat (as get_image reads it) -> the primitive perturbation at
    every cell's first Gauss point, to the format's six significant digits."""
    c = base_cfg(nx=9, ny=7, order=2, basis=1, eq_kind=2, gx=0.2, gy=0.9)
    d = random_delta(c, amp=1e-2, seed=18)
    with solver(wb, c, 0) as s:
        s.upload(d)
        s.step(2, 1e-3)
        s.output_file(str(tmp_path / "snap.dat"), var=var)
        dl = s.download()
    x, y, fields = wb.read_output_file(str(tmp_path / "snap.dat"), 9, 7, var=var)
    # byte for byte what the reference's output_file writes for these numbers (the
    # formatter below reproduces the reference's own initwo.dat, test_dat_cpu.py)
    from test_dat_cpu import f1pe12_5
    for ln in open(tmp_path / "snap.dat").read().splitlines():
        assert ln == " ".join(f1pe12_5(float(t)) for t in ln.split())
    assert x.shape == (9, 7) and len(fields) == 5 - var
    oc = orc_cfg(c)
    nodes = orc.nodes_from_modes(oc, dl)
    xg, _ = orc.gl(3)
    for i in range(9):
        for j in range(7):
            xq = (i + 0.5) / 9 + 0.5 / 9 * xg[0]
            yq = (j + 0.5) / 7 + 0.5 / 7 * xg[0]
            re, pe = orc.eq_at(oc, xq, yq)
            d = nodes[:, 0, j, i]
            r = re + d[0]
            w = [d[0], d[1] / r, d[2] / r, 0.4 * (d[3] - 0.5 * (d[1] ** 2 + d[2] ** 2) / r)]
            np.testing.assert_allclose([x[i, j], y[i, j]], [xq, yq], rtol=5e-6)
            np.testing.assert_allclose([f[i, j] for f in fields], w[var - 1:], rtol=5e-6,
                                       atol=1e-300)


@pytest.mark.parametrize("var", [1, 3])
def test_output_file_round_trip_1d(wb, orc, tmp_path, var):
    """The 1D output_file (benchmark_1d.f90:69-100): x and w - w_eq at the cell centres,
    read back through wb_read_dat, to six significant digits."""
    c = orc.make_fv1d(nx=64, bc=1, limiter=1, eq_kind=1, cfl=0.4)
    d0 = orc.fv1d_ic(c)
    with wb.Solver1D(nx=64, bc=1, limiter=1, eq_kind=1, cfl=0.4) as s:
        s.upload(d0)
        s.evolve(0.05)
        got = s.download()
        s.output_file(str(tmp_path / "snap1d.dat"), var=var)
    lines = open(tmp_path / "snap1d.dat").read().splitlines()
    assert len(lines) == 64 and all(len(ln) == (1 + 4 - var) * 13 - 1 for ln in lines)
    x, fields = wb.Solver1D.read_output_file(str(tmp_path / "snap1d.dat"), var=var)
    re, pe = orc.fv1d_eq_cells(c)
    rho = re + got[:, 0]
    v = got[:, 1] / rho
    w = [got[:, 0], v, 0.4 * (got[:, 2] - 0.5 * rho * v * v)]
    np.testing.assert_allclose(x, (np.arange(64) + 0.5) / 64, rtol=5e-6)
    for k, f in enumerate(fields):
        np.testing.assert_allclose(f, w[var - 1 + k], rtol=5e-6, atol=1e-300)
