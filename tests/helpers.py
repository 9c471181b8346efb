"""Helpers shared by the tests: one configuration dict drives both the product context
and the oracle, and seeded random perturbation states."""
import numpy as np

import pyoracle as O

_CFG_KEYS = ("nx", "ny", "order", "basis", "bc_x", "bc_y", "eq_kind", "llf_speed", "limiter",
             "gamma", "gx", "gy", "rho0", "p0", "kpoly", "lx", "ly", "lim_norm", "lim_M",
             "lim_tol", "cfl", "pos_eps", "riemann")


def base_cfg(**kw):
    c = dict(nx=12, ny=10, order=1, basis=1, bc_x=1, bc_y=1, eq_kind=1, llf_speed=0, limiter=0,
             gamma=1.4, gx=1.0, gy=1.0, rho0=1.0, p0=1.0, kpoly=1.0, lx=1.0, ly=1.0,
             lim_norm=3.0, lim_M=0.0, lim_tol=1e-6, cfl=0.3, pos_eps=1e-10, riemann=0)
    c.update(kw)
    return c


def orc_cfg(c):
    return O.make_cfg(**{k: c[k] for k in _CFG_KEYS if k in c})


def solver(wb, c, precision=0, integrator=0, **extra):
    kw = {k: c[k] for k in _CFG_KEYS if k in c}
    kw.update(precision=precision, integrator=integrator)
    kw.update(extra)
    return wb.Solver(**kw)


def random_delta(c, amp=1e-2, seed=0, smooth=True):
    """Seeded perturbation modes with decaying higher-mode amplitudes."""
    rng = np.random.default_rng(seed)
    a, b = O.modes(c["order"], c["basis"])
    nb = len(a)
    d = np.zeros((4, nb, c["ny"], c["nx"]))
    for m in range(nb):
        scale = amp / (1.0 + 2.0 * (a[m] + b[m])) if smooth else amp
        d[:, m] = scale * rng.standard_normal((4, c["ny"], c["nx"]))
    return d


def full_l1(c, delta):
    """L1 per conserved variable of the full state u_eq + delta at the GL nodes."""
    oc = orc_cfg(c)
    nq = c["order"] + 1
    x, w = O.gl(nq)
    nodes = O.nodes_from_modes(oc, delta)
    dx, dy = c["lx"] / c["nx"], c["ly"] / c["ny"]
    out = np.zeros(4)
    gam = c["gamma"]
    for qa in range(nq):
        for qb in range(nq):
            xs = (np.arange(c["nx"]) + 0.5) * dx + dx / 2.0 * x[qa]
            ys = (np.arange(c["ny"]) + 0.5) * dy + dy / 2.0 * x[qb]
            re = np.zeros((c["ny"], c["nx"]))
            pe = np.zeros((c["ny"], c["nx"]))
            for j in range(c["ny"]):
                for i in range(c["nx"]):
                    re[j, i], pe[j, i] = O.eq_at(oc, xs[i], ys[j])
            ueq = [re, 0 * re, 0 * re, pe / (gam - 1.0)]
            for v in range(4):
                u = ueq[v] + nodes[v, qa * nq + qb]
                out[v] += np.sum(np.abs(u)) * w[qa] * w[qb] * dx * dy * 0.25
    return out


def rel_l1_full(c, a, b):
    """||u_a - u_b||_1 / ||u_b||_1 per conserved variable (u = u_eq + delta)."""
    l1, _, _ = O.norms(orc_cfg(c), a, b)
    return l1 / np.maximum(full_l1(c, b), 1e-300)


def rel_l1_delta(c, a, b):
    """||d_a - d_b||_1 / ||d_b||_1 per variable (perturbation-relative, stricter)."""
    oc = orc_cfg(c)
    l1, _, _ = O.norms(oc, a, b)
    ref, _, _ = O.norms(oc, b, np.zeros_like(b))
    return l1 / np.maximum(ref, 1e-300)


def violating_delta(c, seed=0, ncells=6, depth=1.6):
    """Smooth perturbation plus a few cells whose density and energy slopes are steep
    enough that the full state goes negative at some points of the positivity set."""
    rng = np.random.default_rng(seed)
    d = random_delta(c, amp=1e-3, seed=seed)
    a, b = O.modes(c["order"], c["basis"])
    m10 = [m for m in range(len(a)) if a[m] == 1 and b[m] == 0][0]
    m01 = [m for m in range(len(a)) if a[m] == 0 and b[m] == 1][0]
    idx = rng.choice(c["nx"] * c["ny"], ncells, replace=False)
    for k, cell in enumerate(idx):
        j, i = divmod(int(cell), c["nx"])
        s = depth * (1.0 if k % 2 == 0 else -1.0)
        d[0, m10, j, i] = s * 0.6 * (0.9 if k % 3 else 0.5)
        d[3, m01, j, i] = -s * 1.5
        d[1, m10, j, i] = 0.3 * s
    return d
