"""GPU parity of the CUDA path (through the C ABI) against the CPU oracle.

Bars: FP64 plain matches the oracle to 1e-12 relative L1 per conserved variable of the
full state u_eq + delta (and, stricter, to a small multiple of round-off relative to
the perturbation itself); a zero perturbation gives an exactly zero update and stays
exactly zero; FP32-perturbation matches to L1 <= 1e-6.
"""
import itertools

import numpy as np
import pytest

from helpers import base_cfg, orc_cfg, random_delta, rel_l1_delta, rel_l1_full, solver

pytestmark = pytest.mark.gpu

BASES = [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1)]  # (order, basis)


@pytest.mark.parametrize("order,basis", BASES)
@pytest.mark.parametrize("eq_kind", [1, 2])
@pytest.mark.parametrize("precision", [0, 1])
def test_zero_perturbation_is_exactly_zero(wb, order, basis, eq_kind, precision):
    c = base_cfg(order=order, basis=basis, eq_kind=eq_kind, gx=0.3, gy=1.0, limiter=1)
    with solver(wb, c, precision) as s:
        z = np.zeros(s.shape)
        dudt = s.compute_update(z)
        assert np.all(dudt == 0.0)
        s.upload(z)
        s.step(20)          # CFL steps
        s.step(5, 1e-3)     # fixed steps
        assert np.all(s.download() == 0.0)


@pytest.mark.parametrize("order,basis", BASES)
@pytest.mark.parametrize("eq_kind,bc,llf", [(1, 1, 0), (2, 1, 0), (1, 0, 1), (0, 0, 0), (2, 0, 1)])
def test_rhs_parity_fp64(wb, orc, order, basis, eq_kind, bc, llf):
    c = base_cfg(order=order, basis=basis, eq_kind=eq_kind, bc_x=bc, bc_y=1 - bc, llf_speed=llf,
                 gx=0.7, gy=1.0)
    d = random_delta(c, amp=1e-2, seed=order * 10 + basis)
    if eq_kind == 0:
        d[0, 0] += 1.0  # a positive density/energy when the equilibrium is zero
        d[3, 0] += 2.5
    ref = orc.rhs(orc_cfg(c), d)
    with solver(wb, c, 0) as s:
        got = s.compute_update(d)
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(got - ref)) <= 1e-12 * scale
    for v in range(4):
        den = np.sum(np.abs(ref[v])) + 1e-300
        assert np.sum(np.abs(got[v] - ref[v])) / den < 1e-12


@pytest.mark.parametrize("order,basis", BASES)
def test_rhs_fortran_layout(wb, orc, order, basis):
    if basis != 0:
        pytest.skip("Fortran layout is the tensor basis only")
    c = base_cfg(order=order, basis=basis)
    d = random_delta(c, seed=3)
    a, b = orc.modes(order, basis)
    k = order + 1
    f = np.zeros((4, c["nx"], c["ny"], k, k), order="F")
    for m in range(len(a)):
        f[:, :, :, a[m], b[m]] = d[:, m].transpose(0, 2, 1)
    with solver(wb, c, 0) as s:
        soa = s.compute_update(d)
        fo = s.compute_update(f, layout=wb.LAYOUT_FORTRAN)
        s.upload(f, layout=wb.LAYOUT_FORTRAN)
        back = s.download(layout=wb.LAYOUT_FORTRAN)
    for m in range(len(a)):
        np.testing.assert_array_equal(fo[:, :, :, a[m], b[m]], soa[:, m].transpose(0, 2, 1))
    np.testing.assert_array_equal(back, f)


@pytest.mark.parametrize("order,basis", BASES)
@pytest.mark.parametrize("limiter", [0, 1])
@pytest.mark.parametrize("integrator", [0, 1])
def test_steps_parity_fp64(wb, orc, order, basis, limiter, integrator):
    c = base_cfg(order=order, basis=basis, limiter=limiter, eq_kind=1, bc_x=0, bc_y=1)
    d = random_delta(c, amp=2e-2, seed=11)
    dt = 2e-3
    n = 12
    run = orc.run_rk2 if integrator == 0 else orc.run_rk54
    ref, tref = run(orc_cfg(c), d, n, dt)
    with solver(wb, c, 0, integrator) as s:
        s.upload(d)
        s.step(n, dt)
        got = s.download()
        t, steps = s.time()
    assert steps == n and abs(t - tref) < 1e-15
    assert np.all(rel_l1_full(c, got, ref) < 1e-12)
    assert np.all(rel_l1_delta(c, got, ref)[[0, 1, 3]] < 1e-9)


@pytest.mark.parametrize("order,basis", [(1, 1), (2, 1), (1, 0)])
def test_cfl_steps_parity_fp64(wb, orc, order, basis):
    c = base_cfg(order=order, basis=basis, limiter=1, cfl=0.3)
    d = random_delta(c, amp=1e-2, seed=5)
    ref, tref = orc.run_rk2(orc_cfg(c), d, 15, -1.0)
    with solver(wb, c, 0) as s:
        s.upload(d)
        s.step(15)
        got = s.download()
        t, steps = s.time()
    assert steps == 15
    assert abs(t - tref) <= 1e-13 * tref
    assert np.all(rel_l1_full(c, got, ref) < 1e-12)


@pytest.mark.parametrize("order,basis", BASES)
@pytest.mark.parametrize("precision", [0, 1])
def test_max_speed_and_limiter(wb, orc, order, basis, precision):
    c = base_cfg(order=order, basis=basis, limiter=1, lim_tol=1e-8)
    d = random_delta(c, amp=5e-2, seed=7, smooth=False)
    oc = orc_cfg(c)
    sx, sy = orc.max_speed(oc, d)
    lim = orc.limit(oc, d)
    with solver(wb, c, precision) as s:
        s.upload(d)
        gx, gy = s.compute_max_speed()
        s.apply_limiter()
        s.limiter_off = True
        got = s.download()
    tol = 1e-14 if precision == 0 else 2e-6
    assert abs(gx - sx) <= tol * sx and abs(gy - sy) <= tol * sy
    if precision == 0:
        np.testing.assert_allclose(got, lim, rtol=0, atol=1e-15)
    else:
        np.testing.assert_allclose(got, lim, rtol=0, atol=1e-7)


@pytest.mark.parametrize("order,basis", BASES)
@pytest.mark.parametrize("kind", [1, 2])
def test_initial_perturbation_projection(wb, orc, order, basis, kind):
    c = base_cfg(order=order, basis=basis, eq_kind=2, gx=0.0, gy=1.0)
    if kind == 1:
        ic = wb.seeded_gaussian_bump(3, 1e-1, 0.05)
        oic = orc.make_ic(kind=1, amp=ic.amp, xc=ic.xc, yc=ic.yc, sigma=ic.sigma)
    else:
        ic = wb.seeded_multimode(5, 16, 1e-2, 8)
        oic = orc.make_ic(kind=2, amp=ic.amp, nmodes=16, kx=list(ic.kx), ky=list(ic.ky),
                          phase_u=list(ic.phase_u), phase_v=list(ic.phase_v), weight=list(ic.weight))
    ref = orc.project_ic(orc_cfg(c), oic)
    with solver(wb, c, 0) as s:
        s.init_perturbation(ic)
        got = s.download()
        t, n = s.time()
    assert t == 0.0 and n == 0
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-14 * np.max(np.abs(ref)))


@pytest.mark.parametrize("order,basis", [(1, 1), (2, 1), (2, 0)])
def test_fp32_perturbation_vs_fp64(wb, orc, order, basis):
    c = base_cfg(order=order, basis=basis, eq_kind=1, nx=24, ny=20, bc_x=0, bc_y=1, limiter=0)
    ic = wb.gaussian_bump(1e-1, 0.5, 0.4, 0.08)
    with solver(wb, c, 0) as s64, solver(wb, c, 1) as s32:
        s64.init_perturbation(ic)
        s32.init_perturbation(ic)
        s64.step(40, 1e-3)
        s32.step(40, 1e-3)
        l1, linf, _ = s32.compute_error(s64)
        d64 = s64.download()
    oic = orc.make_ic(kind=1, amp=1e-1, xc=0.5, yc=0.4, sigma=0.08)
    ref, _ = orc.run_rk2(orc_cfg(c), orc.project_ic(orc_cfg(c), oic), 40, 1e-3)
    assert np.all(rel_l1_full(c, d64, ref) < 1e-12)
    assert np.all(l1 <= 1e-6), l1


def test_equilibrium_preserved_1e4_steps(wb):
    c = base_cfg(nx=32, ny=32, order=1, basis=1, eq_kind=1, limiter=1)
    with solver(wb, c, 0) as s:
        s.upload(np.zeros(s.shape))
        s.step(10000)
        d = s.download()
        _, n = s.time()
    assert n == 10000
    assert np.max(np.abs(d)) <= 1e-13


def test_norms_and_sums(wb, orc):
    c = base_cfg(order=2, basis=1, bc_x=0, bc_y=0, eq_kind=1, gx=0.0, gy=0.0)
    d = random_delta(c, seed=9)
    e = random_delta(c, seed=10)
    with solver(wb, c, 0) as a, solver(wb, c, 0) as b:
        a.upload(d)
        b.upload(e)
        l1, linf, l2 = a.compute_error(b)
        s0 = a.conserved_sums()
        a.step(30, 1e-3)
        s1 = a.conserved_sums()
    r1, rinf, r2 = orc.norms(orc_cfg(c), d, e)
    np.testing.assert_allclose(l1, r1, rtol=1e-13)
    np.testing.assert_allclose(linf, rinf, rtol=1e-13)
    np.testing.assert_allclose(l2, r2, rtol=1e-13)
    # periodic domain, no gravity: mass, momentum and energy are conserved to round-off
    assert np.all(np.abs(s1 - s0) <= 1e-13 * (np.abs(s0) + 1.0))


def test_nonphysical_state_is_reported(wb):
    c = base_cfg(order=1, basis=1, eq_kind=1)
    with solver(wb, c, 0) as s:
        d = np.zeros(s.shape)
        d[0, 0, 3, 4] = -5.0  # negative density mean in one cell
        s.upload(d)
        s.step(1, 1e-4)
        with pytest.raises(wb.WbError) as ei:
            s.sync()
        assert ei.value.status == wb.WB_ERR_NONPHYSICAL


def test_evolve_reaches_tend(wb, orc):
    c = base_cfg(order=1, basis=1, limiter=1, cfl=0.3)
    d = random_delta(c, amp=1e-2, seed=2)
    with solver(wb, c, 0) as s:
        s.upload(d)
        n, t = s.evolve(0.05)
        got = s.download()
    assert abs(t - 0.05) < 1e-15
    assert n > 3
    # evolve = n - 1 CFL steps, then one step clipped at tend (dt = tend - t); the oracle
    # runs the same sequence
    oc = orc_cfg(c)
    ref, tref = orc.run_rk2(oc, d, n - 1, -1.0)
    assert tref < 0.05
    ref, _ = orc.run_rk2(oc, ref, 1, 0.05 - tref)
    assert np.all(rel_l1_full(c, got, ref) < 1e-12)


# every compiled (tile, cells per thread) of a precision and degree (the autotuner's
# candidates for the total-degree basis)
TILES = {(1, 0): [(32, 8, 1), (16, 16, 1), (32, 16, 2), (32, 32, 4)],
         (1, 1): [(32, 8, 1), (16, 16, 1), (32, 16, 2)],
         (1, 2): [(32, 8, 1), (16, 16, 1), (32, 16, 2)],
         (0, 0): [(16, 8, 1), (16, 4, 1)], (0, 1): [(16, 8, 1), (16, 4, 1)],
         (0, 2): [(16, 8, 1), (16, 4, 1)]}


@pytest.mark.parametrize("precision,order", sorted(TILES))
@pytest.mark.parametrize("limiter", [0, 1])
def test_tiles_agree(wb, precision, order, limiter):
    """Results do not depend on the tile shape or the cells per thread (fixed and CFL
    steps, so the wave-speed reduction too).  Shapes of one cells-per-thread count run the
    same instructions per cell and agree bit for bit, and so do all FP64 shapes and the
    degree-0 ones; between counts the compiler may contract a product and a sum into one
    FMA differently, which in FP32 is a rounding-level difference, well inside the FP32
    form's 1e-6 bar."""
    c = base_cfg(nx=37, ny=23, order=order, basis=1, limiter=limiter)
    d = random_delta(c, amp=5e-3, seed=21, smooth=not limiter)
    outs = []
    for tx, ty, cpt in TILES[(precision, order)]:
        with solver(wb, c, precision, tile_x=tx, tile_y=ty, cells_per_thread=cpt) as s:
            s.upload(d)
            s.step(3, 1e-3)
            s.step(3)
            outs.append((cpt, s.download(), s.time()))
    cpt0, ref, tref = outs[0]
    for cpt, o, t in outs[1:]:
        if precision == 0 or order == 0 or cpt == cpt0:
            np.testing.assert_array_equal(o, ref)
            assert t == tref
        else:
            assert np.max(np.abs(o - ref)) <= 1e-5 * np.max(np.abs(ref))
            assert np.all(rel_l1_full(c, o, ref) < 1e-6)  # the FP32 form's bar
            assert abs(t[0] - tref[0]) <= 1e-6 * tref[0] and t[1] == tref[1]


def test_cells_per_thread_on_interior_tiles(wb, orc):
    """Two cells per thread on a grid with TMA-staged interior tiles, against the oracle."""
    c = base_cfg(nx=128, ny=72, order=2, basis=1, eq_kind=1, gx=0.0, gy=1.0, bc_x=0, bc_y=1,
                 limiter=1)
    d = random_delta(c, amp=1e-2, seed=9)
    ref, _ = orc.run_rk2(orc_cfg(c), d, 4, 1e-3)
    with solver(wb, c, 1, tile_x=32, tile_y=16, cells_per_thread=2) as s:
        s.upload(d)
        s.step(4, 1e-3)
        got = s.download()
    assert np.all(rel_l1_full(c, got, ref) < 1e-6)


# Grids with interior tiles: those tiles are staged by one TMA copy (block inside the grid,
# 16-byte aligned rows); 130 cells per row are not a multiple of 16 bytes in FP32, so that
# grid runs the cp.async staging everywhere.
LARGE = [(128, 72), (130, 70), (132, 66)]


@pytest.mark.parametrize("nx,ny", LARGE)
@pytest.mark.parametrize("order,basis", [(2, 1), (1, 0), (2, 0)])
@pytest.mark.parametrize("precision", [0, 1])
def test_rhs_parity_interior_tiles(wb, orc, nx, ny, order, basis, precision):
    c = base_cfg(nx=nx, ny=ny, order=order, basis=basis, eq_kind=1, gx=0.3, gy=1.0, bc_x=0,
                 bc_y=1)
    d = random_delta(c, amp=1e-2, seed=nx + order)
    ref = orc.rhs(orc_cfg(c), d)
    with solver(wb, c, precision) as s:
        got = s.compute_update(d)
    scale = np.max(np.abs(ref))
    tol = 1e-12 if precision == 0 else 2e-5
    assert np.max(np.abs(got - ref)) <= tol * scale


@pytest.mark.parametrize("nx,ny", LARGE)
@pytest.mark.parametrize("limiter", [0, 1, 2])
@pytest.mark.parametrize("precision", [0, 1])
def test_steps_parity_interior_tiles(wb, orc, nx, ny, limiter, precision):
    c = base_cfg(nx=nx, ny=ny, order=2, basis=1, eq_kind=1, gx=0.0, gy=1.0, bc_x=0, bc_y=1,
                 limiter=limiter)
    # rough data only where minmod tames it (unlimited rough P2 data amplifies FP32
    # round-off past the bar; the positivity limiter leaves this state alone)
    d = random_delta(c, amp=1e-2, seed=5, smooth=limiter != 1)
    ref, tref = orc.run_rk2(orc_cfg(c), d, 6, 1e-3)
    with solver(wb, c, precision) as s:
        s.upload(d)
        s.step(6, 1e-3)
        got = s.download()
    bar = 1e-12 if precision == 0 else 1e-6
    assert np.all(rel_l1_full(c, got, ref) < bar)


def test_fp64_tiles_agree_on_interior_tiles(wb, orc):
    """The two FP64 tiles (16x8, 16x4) on a grid with TMA-staged tiles, against the oracle."""
    c = base_cfg(nx=128, ny=72, order=2, basis=1, eq_kind=1, gx=0.0, gy=1.0, bc_x=0, bc_y=1,
                 limiter=1)
    d = random_delta(c, amp=1e-2, seed=9)
    ref, _ = orc.run_rk2(orc_cfg(c), d, 4, 1e-3)
    outs = []
    for tx, ty in [(16, 8), (16, 4)]:
        with solver(wb, c, 0, tile_x=tx, tile_y=ty) as s:
            s.upload(d)
            s.step(4, 1e-3)
            outs.append(s.download())
    np.testing.assert_array_equal(outs[0], outs[1])
    assert np.all(rel_l1_full(c, outs[1], ref) < 1e-12)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("riemann,integrator", [(1, 0), (0, 1), (1, 1)])
def test_variants_on_interior_tiles(wb, orc, precision, riemann, integrator):
    """HLLC and SSP-RK(5,4) on a grid with TMA-staged tiles (the variant kernels run the
    default tile of the precision)."""
    c = base_cfg(nx=128, ny=72, order=2, basis=1, eq_kind=2, gx=0.0, gy=1.0, bc_x=0, bc_y=1,
                 riemann=riemann, limiter=1)
    d = random_delta(c, amp=1e-2, seed=17)
    run = orc.run_rk2 if integrator == 0 else orc.run_rk54
    ref, _ = run(orc_cfg(c), d, 4, 1e-3)
    with solver(wb, c, precision, integrator) as s:
        s.upload(d)
        s.step(4, 1e-3)
        got = s.download()
    bar = 1e-12 if precision == 0 else 1e-6
    assert np.all(rel_l1_full(c, got, ref) < bar)
