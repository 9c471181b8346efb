"""Properties of the oracle's scheme (CPU): exact well-balance, agreement with the
literal restatements of the reference operators, conservation, limiter behaviour and
the 1D finite-volume path."""
import numpy as np
import pytest

from helpers import base_cfg, orc_cfg, random_delta


@pytest.mark.parametrize("order,basis", [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1)])
@pytest.mark.parametrize("eq_kind", [1, 2])
@pytest.mark.parametrize("riemann", [0, 1])
def test_zero_perturbation_exact(orc, order, basis, eq_kind, riemann):
    c = base_cfg(order=order, basis=basis, eq_kind=eq_kind, gx=0.4, gy=1.0, limiter=1,
                 riemann=riemann)
    oc = orc_cfg(c)
    z = np.zeros((4, orc.nb(oc), c["ny"], c["nx"]))
    assert np.all(orc.rhs(oc, z) == 0.0)
    d, _ = orc.run_rk2(oc, z, 50, -1.0)
    assert np.all(d == 0.0)


@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("bc", [1, 2])
def test_matches_literal_reference_2d_operator(orc, order, bc):
    """Zero equilibrium, no gravity: the composed operator is the reference's
    2d/benchmark_2d_dg.f90 compute_update (with its 'llf1' flux branch taken)."""
    nx = ny = 6
    m = order + 1
    c = base_cfg(nx=nx, ny=ny, order=order, basis=0, eq_kind=0, gx=0.0, gy=0.0,
                 bc_x=0 if bc == 1 else 1, bc_y=0 if bc == 1 else 1, llf_speed=1)
    oc = orc_cfg(c)
    rng = np.random.default_rng(order)
    d = random_delta(c, amp=1e-1, seed=order)
    d[0, 0] += 1.0
    d[3, 0] += 2.5
    a, b = orc.modes(order, 0)
    f = np.zeros((4, nx, ny, m, m), order="F")
    for k in range(len(a)):
        f[:, :, :, a[k], b[k]] = d[:, k].transpose(0, 2, 1)
    ref = orc.ref2d_compute_update(f, nx, ny, m, bc=bc)
    got = orc.rhs(oc, d)
    for k in range(len(a)):
        np.testing.assert_allclose(got[:, k].transpose(0, 2, 1), ref[:, :, :, a[k], b[k]],
                                   rtol=0, atol=1e-13)


def test_reference_flux_type_defect_reproduced(orc):
    """flux_type='llf' never matches 'llf1' (2d/benchmark_2d_dg.f90:999): faces stay zero."""
    nx = ny = 4
    u = np.zeros((4, nx, ny, 2, 2), order="F")
    u[0] = 1.0
    u[3] = 2.5
    u[1, :, :, 1, 0] = 0.1
    r_bug = orc.ref2d_compute_update(u, nx, ny, 2, flux_bug=1)
    r_ok = orc.ref2d_compute_update(u, nx, ny, 2, flux_bug=0)
    assert not np.allclose(r_bug, r_ok)


@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("riemann", [0, 1])
def test_matches_literal_reference_1d_wb_operator(orc, order, riemann):
    """y-uniform data reduce the 2D well-balanced operator to the 1D
    compute_update_exact_delta of dg_with_source.f90:1749-2031 (interior cells)."""
    n, nx = order + 1, 10
    c = base_cfg(nx=nx, ny=1, order=order, basis=0, eq_kind=1, gx=1.0, gy=0.0, bc_x=0, bc_y=0,
                 riemann=riemann)
    oc = orc_cfg(c)
    a, b = orc.modes(order, 0)
    rng = np.random.default_rng(1)
    d = np.zeros((4, len(a), 1, nx))
    d1 = np.zeros((3, n, nx), order="F")
    for k in range(n):
        mm = [i for i in range(len(a)) if a[i] == k and b[i] == 0][0]
        vals = 1e-2 * rng.standard_normal((3, nx))
        d[0, mm, 0], d[1, mm, 0], d[3, mm, 0] = vals
        d1[:, k, :] = vals
    r2 = orc.rhs(oc, d)
    r1 = orc.dg1d_update_exact_delta(d1, nx, n, riemann=riemann + 1)
    for k in range(n):
        mm = [i for i in range(len(a)) if a[i] == k and b[i] == 0][0]
        for v2, v1 in ((0, 0), (1, 1), (3, 2)):
            np.testing.assert_allclose(r2[v2, mm, 0, 1:-1], r1[v1, k, 1:-1], rtol=0, atol=5e-14)
        assert np.max(np.abs(r2[2])) < 1e-16


def test_conservation_periodic(orc):
    c = base_cfg(nx=10, ny=8, order=2, basis=1, bc_x=0, bc_y=0, eq_kind=1, gx=0.0, gy=0.0)
    oc = orc_cfg(c)
    d = random_delta(c, seed=4)
    r = orc.rhs(oc, d)
    # mode 0 carries the cell mean: its domain sum changes only by boundary fluxes (none)
    assert np.all(np.abs(r[:, 0].sum(axis=(1, 2))) < 1e-13)


def test_limiter_idempotent_and_selective(orc):
    c = base_cfg(nx=16, ny=16, order=2, basis=1, limiter=1)
    oc = orc_cfg(c)
    d = random_delta(c, amp=1e-1, seed=8, smooth=False)
    l1 = orc.limit(oc, d)
    assert np.array_equal(orc.limit(oc, l1), l1)
    assert np.array_equal(l1[:, 0], d[:, 0])  # means untouched
    # a linear perturbation is not limited
    x = (np.arange(16) + 0.5) / 16
    lin = np.zeros_like(d)
    lin[0, 0] = 1e-3 * x[None, :]
    lin[0, 1] = 1e-3 / 16 / 2 / np.sqrt(3)  # exact slope mode of the linear function
    np.testing.assert_array_equal(orc.limit(oc, lin)[:, :, :, 1:-1], lin[:, :, :, 1:-1])


def test_rk54_consistent_with_rk2(orc):
    c = base_cfg(nx=16, ny=16, order=1, basis=1, eq_kind=1, bc_x=0, bc_y=1)
    oc = orc_cfg(c)
    d = random_delta(c, amp=1e-3, seed=6)
    a, _ = orc.run_rk2(oc, d, 40, 5e-4)
    b, _ = orc.run_rk54(oc, d, 20, 1e-3)
    l1, _, _ = orc.norms(oc, a, b)
    ref, _, _ = orc.norms(oc, d, np.zeros_like(d))
    assert np.all(l1[[0, 1, 3]] < 1e-3 * ref[[0, 1, 3]])


def test_fv1d_equilibrium_and_perturbation(orc):
    """Config 1: 1D well-balanced FV (benchmark_1d.f90 'EQL') with minmod MUSCL."""
    c = orc.make_fv1d(nx=256, bc=1, limiter=1, cfl=0.4)
    z = np.zeros((256, 3))
    assert np.all(orc.fv1d_rhs(c, z) == 0.0)
    zz, t, n = orc.fv1d_run(c, z, 0.25)
    assert t == pytest.approx(0.25, abs=1e-15) and np.all(zz == 0.0)
    d0 = orc.fv1d_ic(c)
    d, t, n = orc.fv1d_run(c, d0, 0.25)
    assert n > 50
    # the pressure pulse splits and travels; its energy perturbation stays O(amp)
    assert 1e-5 < np.max(np.abs(d[:, 2])) < 3e-3


def _state2d(rho, vx, vy, p, gamma=1.4):
    return np.array([rho, rho * vx, rho * vy, p / (gamma - 1) + 0.5 * rho * (vx * vx + vy * vy)])


@pytest.mark.parametrize("case", range(6))
@pytest.mark.parametrize("direction", [0, 1])
def test_hllc_matches_reference_riemann_hllc(orc, case, direction):
    """The composed scheme's HLLC in one direction, no transverse velocity, equals
    riemann_hllc of dg_with_source.f90 on the 1D states: subsonic both ways,
    supersonic both ways, strong pressure jump."""
    left, right = [((1.0, 0.1, 1.0), (0.8, -0.2, 0.7)), ((1.0, -0.3, 1.0), (0.9, -0.4, 1.2)),
                   ((1.0, 3.0, 1.0), (0.5, 2.5, 0.4)), ((0.7, -3.0, 0.6), (1.0, -2.8, 1.0)),
                   ((1.0, 0.0, 1000.0), (1.0, 0.0, 0.01)), ((0.125, 0.0, 0.1), (1.0, 0.0, 1.0))][case]
    oc = orc_cfg(base_cfg(riemann=1))
    g = 1.4
    vl = (left[1], 0.0) if direction == 0 else (0.0, left[1])
    vr = (right[1], 0.0) if direction == 0 else (0.0, right[1])
    f2 = orc.num_flux(oc, _state2d(left[0], *vl, left[2]), _state2d(right[0], *vr, right[2]),
                      direction)
    u1l = np.array([left[0], left[0] * left[1], left[2] / (g - 1) + 0.5 * left[0] * left[1] ** 2])
    u1r = np.array([right[0], right[0] * right[1], right[2] / (g - 1) + 0.5 * right[0] * right[1] ** 2])
    f1 = orc.ref_riemann_hllc(u1l, u1r)
    n = 1 + direction
    got = np.array([f2[0], f2[n], f2[3]])
    np.testing.assert_allclose(got, f1, rtol=1e-13, atol=1e-13 * np.max(np.abs(f1)))
    assert f2[3 - n] == 0.0  # no transverse velocity, no transverse momentum flux


@pytest.mark.parametrize("riemann", [0, 1])
def test_numerical_flux_consistent(orc, riemann):
    """F_hat(u, u) = F(u): bit for bit at rest, to round-off when moving."""
    oc = orc_cfg(base_cfg(riemann=riemann))
    g = 1.4
    rest = _state2d(0.9, 0.0, 0.0, 0.7)
    for d in (0, 1):
        f = orc.num_flux(oc, rest, rest, d)
        exp = np.zeros(4)
        exp[1 + d] = 0.7
        np.testing.assert_array_equal(f, exp)
    mov = _state2d(0.9, 0.3, -0.2, 0.7)
    for d in (0, 1):
        f = orc.num_flux(oc, mov, mov, d)
        v = mov[1 + d] / mov[0]
        p = 0.7
        exp = np.array([mov[1 + d], mov[1] * v, mov[2] * v, v * (mov[3] + p)])
        exp[1 + d] += p
        np.testing.assert_allclose(f, exp, rtol=1e-14, atol=1e-15)


def _wb1_numpy(c, d, orc):
    """compute_update_sr (benchmark_1d.f90:553-747) written out independently with numpy,
    on u = u_eq(x_i) + delta_i."""
    g, nx = c.gamma, c.nx
    dx = c.lx / nx
    re, pe = orc.fv1d_eq_cells(c)
    u = np.stack([re + d[:, 0], d[:, 1], pe / (g - 1) + d[:, 2]])
    rho, v = u[0], u[1] / u[0]
    p = (g - 1) * (u[2] - 0.5 * rho * v * v)
    fl = float(np.float32(1e-5))
    h = np.maximum(p, fl) / np.maximum(fl, rho) * (1 + 1.0 / (g - 1))
    x = (np.arange(nx) + 0.5) * dx
    xf = np.arange(nx + 1) * dx
    h0l = h + c.g * x - c.g * xf[:-1]
    h0r = h + c.g * x - c.g * xf[1:]
    K = np.maximum(fl, p) / np.maximum(fl, rho) ** g

    def state(h0):
        r = ((1.0 / K) * (g - 1) / g * h0) ** (1 / (g - 1))
        pp = (1.0 / K) ** (1 / (g - 1)) * ((g - 1) / g * h0) ** (g / (g - 1))
        return np.stack([r, r * v, pp / (g - 1) + 0.5 * r * v * v]), pp

    uL, pL = state(h0l)
    uR, pR = state(h0r)

    def flux(uu):
        vv = uu[1] / uu[0]
        pp = (g - 1) * (uu[2] - 0.5 * uu[0] * vv * vv)
        return np.stack([vv * uu[0], vv * uu[1] + pp, vv * uu[2] + pp * vv]), np.abs(vv) + np.sqrt(
            g * np.maximum(pp, 1e-10) / np.maximum(uu[0], 1e-10))

    fa, sa = flux(uR[:, :-1])   # left cell's right face state, faces 1..nx-1
    fb, sb = flux(uL[:, 1:])    # right cell's left face state
    cm = np.maximum(sa, sb)
    fh = 0.5 * (fb + fa) - 0.5 * cm * (uL[:, 1:] - uR[:, :-1])
    out = np.zeros((nx, 3))
    for i in range(1, nx - 1):
        s = np.array([0.0, (pR[i] - pL[i]) / dx, -rho[i] * v[i] * c.g * (x[i + 1] - x[i - 1]) / (2 * dx)])
        out[i] = -(fh[:, i] - fh[:, i - 1]) / dx + s
    out[0], out[-1] = out[1], out[-2]
    return out


@pytest.mark.parametrize("eq_kind", [1, 2])
def test_wb1_matches_independent_restatement(orc, eq_kind):
    c = orc.make_fv1d(nx=64, bc=1, limiter=0, eq_kind=eq_kind, scheme=1, cfl=0.8 / 3)
    rng = np.random.default_rng(eq_kind)
    d = 1e-3 * rng.standard_normal((64, 3))
    got = orc.fv1d_rhs(c, d)
    np.testing.assert_allclose(got, _wb1_numpy(c, d, orc), rtol=0, atol=1e-12)


def test_wb1_polytrope_equilibrium_balanced(orc):
    """'WB1' keeps the isentropic (polytropic) atmosphere to round-off; it is not exact for
    the isothermal one (K varies from cell to cell), as in the reference."""
    cp = orc.make_fv1d(nx=128, bc=1, limiter=0, eq_kind=2, scheme=1, cfl=0.8 / 3)
    z = np.zeros((128, 3))
    assert np.max(np.abs(orc.fv1d_rhs(cp, z))) < 1e-12
    d, t, n = orc.fv1d_run(cp, z, 0.2)
    assert n > 10 and np.max(np.abs(d)) < 1e-11
    ci = orc.make_fv1d(nx=128, bc=1, limiter=0, eq_kind=1, scheme=1, cfl=0.8 / 3)
    r = np.max(np.abs(orc.fv1d_rhs(ci, z)))
    assert 0.0 < r < 1e-2


def test_wb1_pressure_pulse(orc):
    """The reference's WB1 configuration (nx = 128, pressure bump on the isothermal
    atmosphere, zero-gradient ends, t_end = 0.2, CFL 0.8/3): stays finite, the pulse splits."""
    c = orc.make_fv1d(nx=128, bc=1, limiter=0, eq_kind=1, scheme=1, cfl=0.8 / 3)
    d0 = orc.fv1d_ic(c, amp=1e-3)
    d, t, n = orc.fv1d_run(c, d0, 0.2)
    assert abs(t - 0.2) < 1e-15 and np.all(np.isfinite(d))
    assert np.max(np.abs(d[:, 2])) < np.max(np.abs(d0[:, 2]))
