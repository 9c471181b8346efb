"""The oracle's Zhang-Shu positivity limiter (compute_positivity, 2d/limiters.f90:478-654):
known answers of solve_for_t, the delta form against the literal limiter on the full
state, and the limiter's invariants (means kept, positive states untouched, the limited
polynomial non-negative on the positivity set)."""
import numpy as np
import pytest

import pyoracle as O
from helpers import base_cfg, orc_cfg, random_delta, violating_delta

GAMMA = 1.4


def test_solve_for_t_known_root():
    """rho(t) = 1 + t, E(t) = 2.5 - 5t, m = 0: p(t) = 1 - 2t, so p = eps at t = (1 - eps)/2
    (the other root of 2 rho (E - eps/(gamma-1)) is t = -1, outside [0, 1])."""
    oc = orc_cfg(base_cfg())
    eps = oc.pos_eps
    t = O.solve_for_t(oc, np.array([2.0, 0.0, 0.0, -2.5]), np.array([1.0, 0.0, 0.0, 2.5]))
    assert abs(t - 0.5 * (1.0 - eps)) < 1e-15


def test_solve_for_t_with_momentum():
    """Moving state: check p(u_avg + t (u - u_avg)) = eps at the returned t."""
    oc = orc_cfg(base_cfg())
    ua = np.array([1.0, 0.3, -0.2, 2.0])
    u = np.array([0.8, 0.9, 0.4, 0.1])
    t = O.solve_for_t(oc, u, ua)
    s = ua + t * (u - ua)
    p = (GAMMA - 1) * (s[3] - 0.5 * (s[1] ** 2 + s[2] ** 2) / s[0])
    assert 0.0 < t < 1.0
    assert abs(p - oc.pos_eps) < 1e-13


def test_solve_for_t_degenerate_quadratic_gives_zero():
    """a = 0 (density and momentum constant along the segment): the reference divides by a,
    finds no root in range and returns t = 0."""
    oc = orc_cfg(base_cfg())
    t = O.solve_for_t(oc, np.array([1.0, 0.0, 0.0, -1.0]), np.array([1.0, 0.0, 0.0, 2.5]))
    assert t == 0.0


def _set_points(order, lobatto=True):
    x, _ = O.gl(order + 1)
    g = {1: [-1.0, 1.0 if lobatto else 0.0], 2: [-1.0, 0.0, 1.0]}[order]
    pts = [(gg, xq) for xq in x for gg in g] + [(xq, gg) for xq in x for gg in g]
    return pts


def _eval(order, basis, full, pts):
    a, b = O.modes(order, basis)
    out = np.zeros((4, len(pts)) + full.shape[2:])
    for k, (xi, eta) in enumerate(pts):
        for m in range(len(a)):
            out[:, k] += full[:, m] * O.legendre(xi, int(a[m])) * O.legendre(eta, int(b[m]))
    return out


@pytest.mark.parametrize("order,basis", [(1, 0), (1, 1), (2, 0), (2, 1)])
@pytest.mark.parametrize("eq_kind", [1, 2])
def test_delta_form_is_literal_limiter_on_full_state(order, basis, eq_kind):
    c = base_cfg(nx=10, ny=8, order=order, basis=basis, eq_kind=eq_kind, gx=0.3, gy=1.0,
                 limiter=2)
    oc = orc_cfg(c)
    d = violating_delta(c, seed=order + 3 * basis)
    e = O.eq_modes_full(oc)
    ref, theta, t = O.ref_positivity(oc, e + d)
    got = O.positivity(oc, d)
    assert np.sum((theta < 1) | (t < 1)) >= 2  # the case exercises the limiter
    touched = (theta < 1) | (t < 1)
    # limited cells: delta' = u' - e; untouched cells: bit for bit
    assert np.allclose(got, ref - e, rtol=0, atol=1e-13)
    assert np.array_equal(got[:, :, ~touched], d[:, :, ~touched])
    # means never change
    assert np.array_equal(got[:, 0], d[:, 0])


@pytest.mark.parametrize("order,basis", [(1, 1), (2, 0), (2, 1)])
def test_limited_state_positive_on_the_set(order, basis):
    c = base_cfg(nx=10, ny=8, order=order, basis=basis, eq_kind=1, limiter=2)
    oc = orc_cfg(c)
    d = violating_delta(c, seed=11)
    e = O.eq_modes_full(oc)
    pts = _set_points(order)
    before = _eval(order, basis, e + d, pts)
    assert before[0].min() < 0 or ((GAMMA - 1) * (before[3] - 0.5 * (before[1] ** 2 + before[2] ** 2) / np.maximum(before[0], 1e-9))).min() < 0
    after = _eval(order, basis, e + O.positivity(oc, d), pts)
    rho = after[0]
    p = (GAMMA - 1) * (after[3] - 0.5 * (after[1] ** 2 + after[2] ** 2) / np.maximum(rho, 1e-9))
    assert rho.min() > -1e-12
    assert p.min() > -1e-12


@pytest.mark.parametrize("order,basis", [(1, 1), (2, 0), (2, 1)])
def test_positive_state_untouched(order, basis):
    c = base_cfg(nx=9, ny=7, order=order, basis=basis, eq_kind=2, gx=0.0, gy=1.0, limiter=2)
    oc = orc_cfg(c)
    d = random_delta(c, amp=1e-2, seed=4)
    assert np.array_equal(O.positivity(oc, d), d)
    assert np.array_equal(O.limit(oc, d), d)


def test_reference_two_point_gll_nodes():
    """The reference's two-point GLL list is {-1, 0} (2d/legendre.f90:122-126); the composed
    scheme uses {-1, +1}.  Both limit the same violating cell; the factors differ."""
    c = base_cfg(nx=8, ny=8, order=1, basis=0, eq_kind=1, limiter=2)
    oc = orc_cfg(c)
    d = violating_delta(c, seed=2)
    e = O.eq_modes_full(oc)
    _, th_l, t_l = O.ref_positivity(oc, e + d, ref_gll_nodes=False)
    _, th_r, t_r = O.ref_positivity(oc, e + d, ref_gll_nodes=True)
    assert np.any(th_l * t_l < 1) and np.any(th_r * t_r < 1)
    assert not np.array_equal(th_l * t_l, th_r * t_r)


def test_order0_no_limiting():
    c = base_cfg(order=0, basis=0, limiter=2)
    oc = orc_cfg(c)
    d = random_delta(c, amp=0.5, seed=1)
    assert np.array_equal(O.positivity(oc, d), d)


def test_rk2_with_positivity_keeps_set_positive():
    """A strong rarefaction-like cell pattern: with the positivity limiter every stage
    output is non-negative on the set (checked on the final state)."""
    c = base_cfg(nx=16, ny=16, order=2, basis=1, eq_kind=1, gx=0.0, gy=1.0, limiter=2,
                 bc_x=0, bc_y=1)
    oc = orc_cfg(c)
    d = violating_delta(c, seed=5, ncells=10, depth=1.2)
    out, _ = O.run_rk2(oc, d, 3, 2e-4)
    e = O.eq_modes_full(oc)
    v = _eval(2, 1, e + out, _set_points(2))
    p = (GAMMA - 1) * (v[3] - 0.5 * (v[1] ** 2 + v[2] ** 2) / np.maximum(v[0], 1e-9))
    assert v[0].min() > -1e-12 and p.min() > -1e-12
    assert np.all(np.isfinite(out))
