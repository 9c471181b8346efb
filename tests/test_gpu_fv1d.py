"""1D well-balanced finite volume on the GPU (the fvm.f90 / benchmark_1d.f90 path) against
the oracle: N = 256, gamma = 1.4, Phi = x, rho = p = exp(-x), pressure pulse 1e-3,
equilibrium-extrapolated boundaries, minmod MUSCL, SSP-RK2, CFL 0.4, t_end = 0.25."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bc,limiter,eq", [(1, 1, 1), (0, 1, 1), (1, 0, 1), (1, 1, 2)])
def test_fv1d_run_parity(wb, orc, bc, limiter, eq):
    c = orc.make_fv1d(nx=256, bc=bc, limiter=limiter, eq_kind=eq, cfl=0.4)
    d0 = orc.fv1d_ic(c)
    ref, tref, nref = orc.fv1d_run(c, d0, 0.25)
    with wb.Solver1D(nx=256, bc=bc, limiter=limiter, eq_kind=eq, cfl=0.4) as s:
        r = s.compute_update(d0)
        # dudt is a difference of O(1) face fluxes over dx: FMA vs unfused rounding
        # differences of 1e-16 grow to ~3e-14 there
        np.testing.assert_allclose(r, orc.fv1d_rhs(c, d0), rtol=0, atol=1e-12)
        s.upload(d0)
        n, t = s.evolve(0.25)
        got = s.download()
    assert n == nref and abs(t - tref) <= 1e-14
    for v in range(3):
        assert np.sum(np.abs(got[:, v] - ref[:, v])) <= 1e-10 * (np.sum(np.abs(ref[:, v])) + 1e-30)


def test_fv1d_equilibrium_exact(wb):
    with wb.Solver1D(nx=256) as s:
        z = np.zeros((256, 3))
        assert np.all(s.compute_update(z) == 0.0)
        s.upload(z)
        n, t = s.evolve(0.25)
        assert n > 10 and abs(t - 0.25) < 1e-15
        assert np.all(s.download() == 0.0)


@pytest.mark.parametrize("eq,bc", [(1, 1), (2, 1), (1, 0)])
def test_wb1_run_parity(wb, orc, eq, bc):
    """'WB1' (compute_update_sr, benchmark_1d.f90:553-747): the reference's configuration
    nx = 128, pressure pulse on the atmosphere, t_end = 0.2, CFL 0.8/3."""
    cfl = 0.8 / 3.0
    c = orc.make_fv1d(nx=128, bc=bc, limiter=0, eq_kind=eq, cfl=cfl, scheme=1)
    d0 = orc.fv1d_ic(c)
    ref, tref, nref = orc.fv1d_run(c, d0, 0.2)
    with wb.Solver1D(nx=128, bc=bc, limiter=0, eq_kind=eq, cfl=cfl, scheme=wb.SCHEME_WB1) as s:
        np.testing.assert_allclose(s.compute_update(d0), orc.fv1d_rhs(c, d0), rtol=0, atol=1e-11)
        s.upload(d0)
        n, t = s.evolve(0.2)
        got = s.download()
    assert n == nref and abs(t - tref) <= 1e-14
    for v in range(3):
        assert np.sum(np.abs(got[:, v] - ref[:, v])) <= 1e-9 * (np.sum(np.abs(ref[:, v])) + 1e-30)


def test_wb1_polytrope_balanced(wb):
    with wb.Solver1D(nx=128, limiter=0, eq_kind=2, cfl=0.8 / 3.0, scheme=wb.SCHEME_WB1) as s:
        z = np.zeros((128, 3))
        assert np.max(np.abs(s.compute_update(z))) < 1e-12
        s.upload(z)
        n, t = s.evolve(0.2)
        assert n > 10 and np.max(np.abs(s.download())) < 1e-11
