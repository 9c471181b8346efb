"""ctypes binding of the CPU oracle (oracle/wb_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py's CPU-baseline / reference arm.  The product library never
imports this module.  Parity status of the oracle: basis/quadrature pinned by KATs,
operator parity unpinned (the Fortran reference cannot be compiled on these machines).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

BASIS_Q, BASIS_P = 0, 1
BC_PERIODIC, BC_COPY = 0, 1
EQ_NONE, EQ_ISOTHERMAL, EQ_POLYTROPE = 0, 1, 2
LLF_MAXABS, LLF_REF2D = 0, 1


class OrcCfg(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("order", ctypes.c_int),
        ("basis", ctypes.c_int), ("bc_x", ctypes.c_int), ("bc_y", ctypes.c_int),
        ("eq_kind", ctypes.c_int), ("llf_speed", ctypes.c_int), ("limiter", ctypes.c_int),
        ("riemann", ctypes.c_int),
        ("gamma", ctypes.c_double), ("gx", ctypes.c_double), ("gy", ctypes.c_double),
        ("rho0", ctypes.c_double), ("p0", ctypes.c_double), ("kpoly", ctypes.c_double),
        ("lx", ctypes.c_double), ("ly", ctypes.c_double),
        ("lim_norm", ctypes.c_double), ("lim_M", ctypes.c_double), ("lim_tol", ctypes.c_double),
        ("cfl", ctypes.c_double), ("pos_eps", ctypes.c_double),
    ]


class OrcIC(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int), ("nmodes", ctypes.c_int),
        ("amp", ctypes.c_double), ("xc", ctypes.c_double), ("yc", ctypes.c_double),
        ("sigma", ctypes.c_double),
        ("kx", ctypes.c_double * 32), ("ky", ctypes.c_double * 32),
        ("phase_u", ctypes.c_double * 32), ("phase_v", ctypes.c_double * 32),
        ("weight", ctypes.c_double * 32),
    ]


class OrcFV1D(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("bc", ctypes.c_int), ("limiter", ctypes.c_int),
        ("eq_kind", ctypes.c_int), ("scheme", ctypes.c_int), ("pad0", ctypes.c_int),
        ("gamma", ctypes.c_double), ("g", ctypes.c_double), ("rho0", ctypes.c_double),
        ("p0", ctypes.c_double), ("kpoly", ctypes.c_double), ("lx", ctypes.c_double),
        ("cfl", ctypes.c_double),
    ]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        d, i, p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
        L.orc_legendre.restype = d
        L.orc_legendre.argtypes = [d, i]
        L.orc_legendre_prime.restype = d
        L.orc_legendre_prime.argtypes = [d, i]
        L.orc_gl_quadrature.argtypes = [i, p, p]
        L.orc_nb.restype = i
        L.orc_nb.argtypes = [i, i]
        L.orc_modes.restype = i
        L.orc_modes.argtypes = [i, i, p, p]
        for name in ("orc_rhs", "orc_limit", "orc_positivity"):
            getattr(L, name).argtypes = [p, p, p]
        L.orc_project_ic.argtypes = [p, p, p]
        L.orc_ref_positivity.argtypes = [p, p, p, i, p, p]
        L.orc_solve_for_t.restype = d
        L.orc_solve_for_t.argtypes = [p, p, p]
        L.orc_eq_modes.argtypes = [p, i, i, p, p]
        L.orc_nodes_from_modes.argtypes = [p, i, p, p]
        L.orc_modes_from_nodes.argtypes = [p, i, p, p]
        L.orc_max_speed.argtypes = [p, p, p, p]
        L.orc_cfl_dt.restype = d
        L.orc_cfl_dt.argtypes = [p, d, d]
        L.orc_run_rk2.restype = d
        L.orc_run_rk2.argtypes = [p, p, i, d]
        L.orc_run_rk54.restype = d
        L.orc_run_rk54.argtypes = [p, p, i, d]
        L.orc_norms.argtypes = [p, p, p, p, p, p]
        L.orc_set_threads.argtypes = [i]
        L.orc_get_threads.restype = i
        L.orc_eq_at.argtypes = [p, d, d, p, p]
        L.orc_splitmix64.restype = ctypes.c_uint64
        L.orc_splitmix64.argtypes = [p]
        L.orc_uniform.restype = d
        L.orc_uniform.argtypes = [p]
        L.orc_ref2d_compute_update.argtypes = [i, i, i, d, d, d, i, i, i, d, d, i, p, p]
        L.orc_dg1d_update_exact_delta.argtypes = [i, i, d, d, i, i, p, p]
        L.orc_ref_riemann_hllc.argtypes = [d, p, p, p]
        L.orc_num_flux.argtypes = [p, p, p, i, p]
        L.orc_fv1d_rhs.argtypes = [p, p, p]
        L.orc_fv1d_run.restype = d
        L.orc_fv1d_run.argtypes = [p, p, d, i, p]
        L.orc_fv1d_eq_cells.argtypes = [p, p, p]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_cfg(nx=16, ny=16, order=1, basis=BASIS_P, bc_x=BC_COPY, bc_y=BC_COPY,
             eq_kind=EQ_ISOTHERMAL, llf_speed=LLF_MAXABS, limiter=0, gamma=1.4, gx=1.0, gy=1.0,
             rho0=1.0, p0=1.0, kpoly=1.0, lx=1.0, ly=1.0, lim_norm=3.0, lim_M=0.0,
             lim_tol=1e-6, cfl=0.3, pos_eps=1e-10, riemann=0):
    c = OrcCfg()
    c.nx, c.ny, c.order, c.basis = nx, ny, order, basis
    c.bc_x, c.bc_y, c.eq_kind, c.llf_speed, c.limiter = bc_x, bc_y, eq_kind, llf_speed, limiter
    c.gamma, c.gx, c.gy, c.rho0, c.p0, c.kpoly = gamma, gx, gy, rho0, p0, kpoly
    c.lx, c.ly, c.lim_norm, c.lim_M, c.lim_tol, c.cfl = lx, ly, lim_norm, lim_M, lim_tol, cfl
    c.pos_eps = pos_eps
    c.riemann = riemann
    return c


def cfg_from_dict(d):
    return make_cfg(**d)


def nb(cfg):
    return lib().orc_nb(cfg.order, cfg.basis)


def modes(order, basis):
    n = lib().orc_nb(order, basis)
    a = np.zeros(n, dtype=np.int32)
    b = np.zeros(n, dtype=np.int32)
    lib().orc_modes(order, basis, _ptr(a), _ptr(b))
    return a, b


def state_shape(cfg):
    return (4, nb(cfg), cfg.ny, cfg.nx)


def zeros(cfg):
    return np.zeros(state_shape(cfg), dtype=np.float64)


def legendre(x, n):
    """phi_n(x) = sqrt(2n+1) P_n(x) (2d/legendre.f90:1-25)"""
    return lib().orc_legendre(float(x), int(n))


def gl(n):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().orc_gl_quadrature(n, _ptr(x), _ptr(w))
    return x, w


def make_ic(kind=0, amp=0.0, xc=0.5, yc=0.5, sigma=0.05, nmodes=0, kx=(), ky=(), phase_u=(),
            phase_v=(), weight=()):
    ic = OrcIC()
    ic.kind, ic.nmodes, ic.amp, ic.xc, ic.yc, ic.sigma = kind, nmodes, amp, xc, yc, sigma
    for k in range(nmodes):
        ic.kx[k], ic.ky[k] = kx[k], ky[k]
        ic.phase_u[k], ic.phase_v[k], ic.weight[k] = phase_u[k], phase_v[k], weight[k]
    return ic


def project_ic(cfg, ic):
    out = zeros(cfg)
    lib().orc_project_ic(ctypes.byref(cfg), ctypes.byref(ic), _ptr(out))
    return out


def rhs(cfg, delta):
    delta = np.ascontiguousarray(delta, dtype=np.float64)
    out = np.empty_like(delta)
    lib().orc_rhs(ctypes.byref(cfg), _ptr(delta), _ptr(out))
    return out


def positivity(cfg, delta):
    """Zhang-Shu positivity limiter in delta form (whatever cfg.limiter says)."""
    delta = np.ascontiguousarray(delta, dtype=np.float64)
    out = np.empty_like(delta)
    lib().orc_positivity(ctypes.byref(cfg), _ptr(delta), _ptr(out))
    return out


def ref_positivity(cfg, u_full, ref_gll_nodes=False):
    """Literal compute_positivity on full-state modes; returns (u, theta, t) per cell."""
    u_full = np.ascontiguousarray(u_full, dtype=np.float64)
    out = np.empty_like(u_full)
    nc = cfg.nx * cfg.ny
    th = np.ones(nc)
    tt = np.ones(nc)
    lib().orc_ref_positivity(ctypes.byref(cfg), _ptr(u_full), _ptr(out), int(ref_gll_nodes),
                             _ptr(th), _ptr(tt))
    return out, th.reshape(cfg.ny, cfg.nx), tt.reshape(cfg.ny, cfg.nx)


def solve_for_t(cfg, u, u_avg):
    u = np.ascontiguousarray(u, dtype=np.float64)
    ua = np.ascontiguousarray(u_avg, dtype=np.float64)
    return lib().orc_solve_for_t(ctypes.byref(cfg), _ptr(u), _ptr(ua))


def eq_modes_full(cfg):
    """Projected equilibrium as a full state (4, nb, ny, nx): rho and E modes, zero momentum."""
    n = nb(cfg)
    out = np.zeros((4, n, cfg.ny, cfg.nx))
    er = np.zeros(n)
    ee = np.zeros(n)
    for j in range(cfg.ny):
        for i in range(cfg.nx):
            lib().orc_eq_modes(ctypes.byref(cfg), i, j, _ptr(er), _ptr(ee))
            out[0, :, j, i] = er
            out[3, :, j, i] = ee
    return out


def limit(cfg, delta):
    delta = np.ascontiguousarray(delta, dtype=np.float64)
    out = np.empty_like(delta)
    lib().orc_limit(ctypes.byref(cfg), _ptr(delta), _ptr(out))
    return out


def max_speed(cfg, delta):
    delta = np.ascontiguousarray(delta, dtype=np.float64)
    sx = ctypes.c_double()
    sy = ctypes.c_double()
    lib().orc_max_speed(ctypes.byref(cfg), _ptr(delta), ctypes.byref(sx), ctypes.byref(sy))
    return sx.value, sy.value


def cfl_dt(cfg, sx, sy):
    return lib().orc_cfl_dt(ctypes.byref(cfg), sx, sy)


def run_rk2(cfg, delta, nsteps, dt=-1.0):
    d = np.array(delta, dtype=np.float64, order="C", copy=True)
    t = lib().orc_run_rk2(ctypes.byref(cfg), _ptr(d), nsteps, dt)
    return d, t


def run_rk54(cfg, delta, nsteps, dt=-1.0):
    d = np.array(delta, dtype=np.float64, order="C", copy=True)
    t = lib().orc_run_rk54(ctypes.byref(cfg), _ptr(d), nsteps, dt)
    return d, t


def norms(cfg, a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    l1, linf, l2 = np.zeros(4), np.zeros(4), np.zeros(4)
    lib().orc_norms(ctypes.byref(cfg), _ptr(a), _ptr(b), _ptr(l1), _ptr(linf), _ptr(l2))
    return l1, linf, l2


def nodes_from_modes(cfg, m, nvar=4):
    m = np.ascontiguousarray(m, dtype=np.float64)
    nq = cfg.order + 1
    out = np.zeros((nvar, nq * nq, cfg.ny, cfg.nx))
    lib().orc_nodes_from_modes(ctypes.byref(cfg), nvar, _ptr(m), _ptr(out))
    return out


def modes_from_nodes(cfg, n, nvar=4):
    n = np.ascontiguousarray(n, dtype=np.float64)
    out = np.zeros((nvar, nb(cfg), cfg.ny, cfg.nx))
    lib().orc_modes_from_nodes(ctypes.byref(cfg), nvar, _ptr(n), _ptr(out))
    return out


def set_threads(n):
    lib().orc_set_threads(int(n))


def eq_at(cfg, x, y):
    r = ctypes.c_double()
    p = ctypes.c_double()
    lib().orc_eq_at(ctypes.byref(cfg), x, y, ctypes.byref(r), ctypes.byref(p))
    return r.value, p.value


def ref2d_compute_update(u_f, nx, ny, m, gamma=1.4, lx=1.0, ly=1.0, flux_bug=0, source=1,
                         grad_phi_bug=0, gx=0.0, gy=0.0, bc=1):
    """u_f: Fortran-ordered array (4, nx, ny, m, m)."""
    u_f = np.asfortranarray(u_f, dtype=np.float64)
    out = np.zeros_like(u_f, order="F")
    lib().orc_ref2d_compute_update(nx, ny, m, gamma, lx, ly, flux_bug, source, grad_phi_bug,
                                   gx, gy, bc, _ptr(u_f), _ptr(out))
    return out


def dg1d_update_exact_delta(du_f, nx, n, gamma=1.4, lx=1.0, half_source=1, riemann=1):
    """du_f: Fortran-ordered array (3, n, nx); riemann: 1 riemann_llf, 2 riemann_hllc."""
    du_f = np.asfortranarray(du_f, dtype=np.float64)
    out = np.zeros_like(du_f, order="F")
    lib().orc_dg1d_update_exact_delta(nx, n, gamma, lx, half_source, riemann, _ptr(du_f),
                                      _ptr(out))
    return out


def ref_riemann_hllc(ul, ur, gamma=1.4):
    """riemann_hllc of dg_with_source.f90 (1D states rho, rho u, E)."""
    ul = np.ascontiguousarray(ul, dtype=np.float64)
    ur = np.ascontiguousarray(ur, dtype=np.float64)
    f = np.zeros(3)
    lib().orc_ref_riemann_hllc(gamma, _ptr(ul), _ptr(ur), _ptr(f))
    return f


def num_flux(cfg, uL, uR, direction):
    """The composed scheme's numerical flux (cfg.riemann) of two 2D states."""
    uL = np.ascontiguousarray(uL, dtype=np.float64)
    uR = np.ascontiguousarray(uR, dtype=np.float64)
    f = np.zeros(4)
    lib().orc_num_flux(ctypes.byref(cfg), _ptr(uL), _ptr(uR), int(direction), _ptr(f))
    return f


def make_fv1d(nx=256, bc=1, limiter=1, eq_kind=EQ_ISOTHERMAL, gamma=1.4, g=1.0, rho0=1.0,
              p0=1.0, kpoly=1.0, lx=1.0, cfl=0.4, scheme=0):
    c = OrcFV1D()
    c.nx, c.bc, c.limiter, c.eq_kind, c.scheme = nx, bc, limiter, eq_kind, scheme
    c.gamma, c.g, c.rho0, c.p0, c.kpoly, c.lx, c.cfl = gamma, g, rho0, p0, kpoly, lx, cfl
    return c


def fv1d_rhs(c, d):
    d = np.ascontiguousarray(d, dtype=np.float64)
    out = np.zeros_like(d)
    lib().orc_fv1d_rhs(ctypes.byref(c), _ptr(d), _ptr(out))
    return out


def fv1d_run(c, d, tend, max_steps=10**9):
    d = np.array(d, dtype=np.float64, copy=True)
    steps = ctypes.c_int()
    t = lib().orc_fv1d_run(ctypes.byref(c), _ptr(d), tend, max_steps, ctypes.byref(steps))
    return d, t, steps.value


def fv1d_eq_cells(c):
    r = np.zeros(c.nx)
    p = np.zeros(c.nx)
    lib().orc_fv1d_eq_cells(ctypes.byref(c), _ptr(r), _ptr(p))
    return r, p


def fv1d_ic(c, amp=1e-3, width=100.0, centre=0.5):
    """Config-1 initial perturbation (benchmark_1d.f90:54-57): p += amp exp(-width (x-c)^2),
    sampled at cell centres, in conservative delta variables (0, 0, dp/(gamma-1))."""
    dx = c.lx / c.nx
    x = (np.arange(c.nx) + 0.5) * dx
    d = np.zeros((c.nx, 3))
    d[:, 2] = amp * np.exp(-width * (x - centre) ** 2) * (1.0 / (c.gamma - 1.0))
    return d
