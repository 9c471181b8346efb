"""Generates the known-answer fixtures in this folder (run here, committed; the GPU machine
only reads the JSON).

* legendre_kat.json -- phi_n(x) = sqrt(2n+1) P_n(x) and its derivative for n <= 6 at
  exact rational points, from sympy's exact Legendre polynomials (the basis of
  2d/legendre.f90:1-50).
* gl_kat.json -- Gauss-Legendre nodes/weights for n = 1..6 from sympy's exact root
  isolation at 30 digits (what 2d/legendre.f90:77-108 computes by Newton iteration).
* oracle_regression.json -- oracle outputs on tiny seeded cases.  These are produced by
  the oracle itself: they pin it against accidental change, not against the reference.
"""
import json
import os
import sys

import numpy as np
import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
sys.path.insert(0, os.path.join(HERE, ".."))


def legendre_kat():
    x = sp.Symbol("x")
    pts = [sp.Rational(-1), sp.Rational(-3, 4), sp.Rational(-1, 3), sp.Rational(0),
           sp.Rational(1, 7), sp.Rational(1, 2), sp.Rational(9, 10), sp.Rational(1)]
    out = []
    for n in range(7):
        P = sp.legendre(n, x)
        dP = sp.diff(P, x)
        s = sp.sqrt(2 * n + 1)
        for p in pts:
            out.append({"n": n, "x": float(p), "phi": float(sp.N(s * P.subs(x, p), 30)),
                        "dphi": float(sp.N(s * dP.subs(x, p), 30))})
    return out


def gl_kat():
    x = sp.Symbol("x")
    out = {}
    for n in range(1, 7):
        P = sp.Poly(sp.legendre(n, x), x)
        roots = sorted(float(r) for r in sp.Poly(P).nroots(n=30))
        dP = sp.diff(sp.legendre(n, x), x)
        ws = [float(sp.N(2 / ((1 - sp.Float(r, 30) ** 2) * dP.subs(x, sp.Float(r, 30)) ** 2), 30))
              for r in roots]
        out[str(n)] = {"x": roots, "w": ws}
    return out


def regression():
    import pyoracle as O
    from helpers import base_cfg, orc_cfg, random_delta
    cases = []
    for order, basis, eq in [(1, 1, 1), (2, 1, 2), (1, 0, 1), (2, 0, 1), (0, 0, 2)]:
        c = base_cfg(nx=4, ny=3, order=order, basis=basis, eq_kind=eq, gx=0.5, gy=1.0)
        d = random_delta(c, amp=1e-2, seed=100 + order)
        r = O.rhs(orc_cfg(c), d)
        cases.append({"cfg": c, "delta": d.ravel().tolist(), "dudt": r.ravel().tolist()})
    return cases


if __name__ == "__main__":
    with open(os.path.join(HERE, "legendre_kat.json"), "w") as f:
        json.dump(legendre_kat(), f, indent=0)
    with open(os.path.join(HERE, "gl_kat.json"), "w") as f:
        json.dump(gl_kat(), f, indent=1)
    with open(os.path.join(HERE, "oracle_regression.json"), "w") as f:
        json.dump(regression(), f)
    print("written")
