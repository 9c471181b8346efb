"""The oracle against the known answers the reference offers for this path:
closed-form Legendre basis values (2d/legendre.f90:1-50), Gauss-Legendre nodes and
weights (2d/legendre.f90:77-108) and the modes<->nodes round trip of 2d/test2d.f90:77-84.
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_legendre_values(orc):
    L = orc.lib()
    for e in json.load(open(os.path.join(GOLD, "legendre_kat.json"))):
        assert abs(L.orc_legendre(e["x"], e["n"]) - e["phi"]) <= 4e-15 * max(1.0, abs(e["phi"]))
        assert abs(L.orc_legendre_prime(e["x"], e["n"]) - e["dphi"]) <= 4e-14 * max(1.0, abs(e["dphi"]))


def test_legendre_endpoints(orc):
    L = orc.lib()
    for n in range(7):
        assert L.orc_legendre(1.0, n) == pytest.approx(np.sqrt(2 * n + 1), abs=1e-15)
        assert L.orc_legendre(-1.0, n) == pytest.approx((-1) ** n * np.sqrt(2 * n + 1), abs=1e-15)
        # the reference clamps the argument to [-1, 1]
        assert L.orc_legendre(1.5, n) == L.orc_legendre(1.0, n)


def test_gauss_legendre(orc):
    gold = json.load(open(os.path.join(GOLD, "gl_kat.json")))
    for n in range(1, 7):
        x, w = orc.gl(n)
        # Newton (500 steps) settles within a few ulps of the exact root
        np.testing.assert_allclose(x, gold[str(n)]["x"], rtol=0, atol=5e-16)
        np.testing.assert_allclose(w, gold[str(n)]["w"], rtol=0, atol=1e-15)
        assert abs(np.sum(w) - 2.0) < 1e-15


def test_gauss_legendre_closed_forms(orc):
    x, w = orc.gl(2)
    assert x[1] == pytest.approx(1 / np.sqrt(3), abs=3e-16)
    x, w = orc.gl(3)
    assert x[2] == pytest.approx(np.sqrt(3 / 5), abs=3e-16)
    assert w[1] == pytest.approx(8 / 9, abs=3e-16)


@pytest.mark.parametrize("order", [0, 1, 2])
def test_roundtrip_test2d(orc, order):
    """2d/test2d.f90: project exp(-x+y), then 1000 modes->nodes->modes round trips."""
    c = orc.make_cfg(nx=8, ny=8, order=order, basis=orc.BASIS_Q)
    nq = order + 1
    xq, _ = orc.gl(nq)
    dx = 1.0 / 8
    nodes = np.zeros((1, nq * nq, 8, 8))
    for qa in range(nq):
        for qb in range(nq):
            x = (np.arange(8) + 0.5) * dx + dx / 2 * xq[qa]
            y = (np.arange(8) + 0.5) * dx + dx / 2 * xq[qb]
            nodes[0, qa * nq + qb] = np.exp(-x[None, :] + y[:, None])
    u = nodes.copy()
    for _ in range(1000):
        m = orc.modes_from_nodes(c, nodes, nvar=1)
        nodes = orc.nodes_from_modes(c, m, nvar=1)
    # 1000 round trips accumulate round-off: the reference prints the max difference
    assert np.max(np.abs(u - nodes)) < 2e-12


def test_oracle_regression_vectors(orc):
    """Pins the oracle against its own committed outputs (not reference-pinned)."""
    from helpers import orc_cfg
    for case in json.load(open(os.path.join(GOLD, "oracle_regression.json"))):
        c = case["cfg"]
        oc = orc_cfg(c)
        shape = (4, orc.nb(oc), c["ny"], c["nx"])
        d = np.array(case["delta"]).reshape(shape)
        np.testing.assert_allclose(orc.rhs(oc, d), np.array(case["dudt"]).reshape(shape),
                                   rtol=0, atol=1e-15)


def test_splitmix_matches_product_draws(orc, wb):
    import ctypes
    st = ctypes.c_uint64(12345)
    r = wb.SplitMix64(12345)
    for _ in range(20):
        assert orc.lib().orc_uniform(ctypes.byref(st)) == r.uniform()
