"""Writes wb_ctab.h: compile-time Gauss-Legendre / scaled-Legendre tables for degrees 0..2.

Values are computed exactly (sympy) and rounded to double: nodes xi_q (ascending) and
weights w_q of the (k+1)-point rule, phi_a = sqrt(2a+1) P_a at the nodes and at +-1,
phi_a' at the nodes, and phi_a at the Gauss-Lobatto nodes of the positivity limiter's set
(-1, +1 for k = 1; -1, 0, +1 for k = 2).  Run: python gen_ctab.py > wb_ctab.h
"""
import sympy as sp

x = sp.Symbol("x")


def lit(v):
    f = float(sp.N(v, 40))
    r = repr(f)
    if "e" not in r and "." not in r:
        r += ".0"
    return r


def sel(idx, vals):
    """nested conditional on idx returning the literal vals[idx]"""
    e = lit(vals[-1])
    for i in range(len(vals) - 2, -1, -1):
        e = "(%s == %d ? %s : %s)" % (idx, i, lit(vals[i]), e)
    return e


def main():
    out = ["// wb_ctab.h -- compile-time Gauss-Legendre / scaled-Legendre tables (generated by",
           "// gen_ctab.py; exact values rounded to double).  The stage kernels use these so that",
           "// the structural zeros and ones of the basis (phi_0 = 1, phi_1(0) = 0, ...) fold away",
           "// once the quadrature loops are unrolled.",
           "#pragma once", "", "namespace wb {", "", "template <int K>", "struct CTab;", ""]
    fn = "  static __host__ __device__ __forceinline__ constexpr double"
    for k in range(3):
        n = k + 1
        P = sp.legendre(n, x)
        roots = sorted(sp.solve(P, x), key=lambda r: float(r))
        dP = sp.diff(P, x)
        ws = [sp.simplify(2 / ((1 - r ** 2) * dP.subs(x, r) ** 2)) for r in roots]
        phi = [sp.sqrt(2 * a + 1) * sp.legendre(a, x) for a in range(n)]
        dphi = [sp.diff(f, x) for f in phi]
        def two(tab):
            rows = [sel("q", tab[a]) for a in range(n)]
            e = rows[-1]
            for a in range(n - 2, -1, -1):
                e = "(a == %d ? %s : %s)" % (a, rows[a], e)
            return e
        B = [[phi[a].subs(x, r) for r in roots] for a in range(n)]
        D = [[dphi[a].subs(x, r) for r in roots] for a in range(n)]
        BW = [[phi[a].subs(x, r) * w for r, w in zip(roots, ws)] for a in range(n)]
        DW = [[dphi[a].subs(x, r) * w for r, w in zip(roots, ws)] for a in range(n)]
        out.append("template <>")
        out.append("struct CTab<%d> {" % k)
        out.append("%s xq(int q) { return %s; }" % (fn, sel("q", roots)))
        out.append("%s wq(int q) { return %s; }" % (fn, sel("q", ws)))
        for name, tab in (("B", B), ("D", D), ("BW", BW), ("DW", DW)):
            out.append("%s %s(int a, int q) { return %s; }" % (fn, name, two(tab)))
        out.append("%s Ep(int a) { return %s; }" % (fn, sel("a", [f.subs(x, 1) for f in phi])))
        out.append("%s Em(int a) { return %s; }" % (fn, sel("a", [f.subs(x, -1) for f in phi])))
        gll = {0: [0], 1: [-1, 1], 2: [-1, 0, 1]}[k]
        out.append("  static constexpr int NG = %d;" % len(gll))
        out.append("%s xg(int g) { return %s; }" % (fn, sel("g", gll)))
        G = [[phi[a].subs(x, r) for r in gll] for a in range(n)]
        rows = [sel("g", G[a]) for a in range(n)]
        e = rows[-1]
        for a in range(n - 2, -1, -1):
            e = "(a == %d ? %s : %s)" % (a, rows[a], e)
        out.append("%s Gl(int a, int g) { return %s; }" % (fn, e))
        out.append("};")
        out.append("")
    out.append("}  // namespace wb")
    print("\n".join(out))


if __name__ == "__main__":
    main()
