"""GPU parity of the Zhang-Shu positivity limiter (limiter 2: compute_positivity of
2d/limiters.f90:478-654 in delta form) against the oracle, through the C ABI.

Bars: FP64 matches the oracle to 1e-12 on the limited modes; FP32 to 2e-5 absolute
(the limiter's factors come from FP32 point values of the full state); a zero
perturbation stays exactly zero (the equilibrium itself is never limited)."""
import numpy as np
import pytest

from helpers import base_cfg, orc_cfg, random_delta, rel_l1_full, solver, violating_delta

pytestmark = pytest.mark.gpu

BASES = [(1, 0), (1, 1), (2, 0), (2, 1)]


@pytest.mark.parametrize("order,basis", BASES)
@pytest.mark.parametrize("eq_kind", [1, 2])
@pytest.mark.parametrize("precision", [0, 1])
def test_limiter_parity(wb, orc, order, basis, eq_kind, precision):
    c = base_cfg(nx=12, ny=10, order=order, basis=basis, eq_kind=eq_kind, gx=0.3, gy=1.0,
                 limiter=2)
    d = violating_delta(c, seed=order + 2 * basis + 5 * eq_kind)
    oc = orc_cfg(c)
    ref = orc.positivity(oc, d)
    assert np.any(ref != d)
    with solver(wb, c, precision) as s:
        s.upload(d)
        got = s.download()          # the limited view of the resident state
        s.apply_limiter()           # in place
        s.upload(s.download())
    tol = 1e-12 if precision == 0 else 2e-5
    np.testing.assert_allclose(got, ref, rtol=0, atol=tol)
    # means never change (an FP32 context holds the FP32-rounded upload)
    d0 = d[:, 0] if precision == 0 else d[:, 0].astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(got[:, 0], d0)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("order,basis", [(1, 1), (2, 1), (2, 0)])
def test_zero_perturbation_stays_zero(wb, order, basis, precision):
    c = base_cfg(order=order, basis=basis, eq_kind=2, gx=0.0, gy=1.0, limiter=2)
    with solver(wb, c, precision) as s:
        z = np.zeros(s.shape)
        s.upload(z)
        s.step(10)
        assert np.all(s.download() == 0.0)


@pytest.mark.parametrize("order,basis", [(1, 0), (2, 1), (2, 0)])
@pytest.mark.parametrize("integrator", [0, 1])
def test_steps_parity_fp64(wb, orc, order, basis, integrator):
    c = base_cfg(nx=16, ny=12, order=order, basis=basis, eq_kind=1, gx=0.0, gy=1.0, bc_x=0,
                 bc_y=1, limiter=2)
    d = violating_delta(c, seed=9, ncells=8, depth=1.2)
    dt, n = 2e-4, 4
    run = orc.run_rk2 if integrator == 0 else orc.run_rk54
    ref, _ = run(orc_cfg(c), d, n, dt)
    with solver(wb, c, 0, integrator) as s:
        s.upload(d)
        s.step(n, dt)
        got = s.download()
    assert np.all(np.isfinite(got))
    assert np.all(rel_l1_full(c, got, ref) < 1e-11)


@pytest.mark.parametrize("order,basis", [(2, 1), (1, 0)])
def test_steps_fp32_against_fp64(wb, orc, order, basis):
    c = base_cfg(nx=16, ny=12, order=order, basis=basis, eq_kind=1, gx=0.0, gy=1.0, bc_x=0,
                 bc_y=1, limiter=2)
    d = violating_delta(c, seed=4, ncells=8, depth=1.2)
    ref, _ = orc.run_rk2(orc_cfg(c), d, 4, 2e-4)
    with solver(wb, c, 1) as s:
        s.upload(d)
        s.step(4, 2e-4)
        got = s.download()
    assert np.all(rel_l1_full(c, got, ref) < 1e-5)


def test_smooth_state_matches_unlimited(wb):
    """A state positive on the whole set is left bit for bit alone by limiter 2."""
    c = base_cfg(order=2, basis=1, eq_kind=1, limiter=2)
    d = random_delta(c, amp=1e-2, seed=8)
    with solver(wb, c, 0) as s2, solver(wb, dict(c, limiter=0), 0) as s0:
        s2.upload(d)
        s0.upload(d)
        s2.step(3, 1e-3)
        s0.step(3, 1e-3)
        np.testing.assert_array_equal(s2.download(), s0.download())
