"""GB300-native well-balanced Euler-with-gravity step (host-side mirror of the reference
interface of hanveiga/fvm-source-wb over the C ABI in include/wb_capi.h).

The reference's step routines are Fortran subroutines -- compute_update, apply_limiter,
compute_max_speed, evolve, compute_error (2d/benchmark_2d_dg.f90) -- driven by module
parameters.  `Solver` exposes the same operations on a context created from a
configuration; every call goes through libwbgb300.so (CUDA, sm_103a).  There is no CPU
fallback: if the library is missing or no GPU is present the calls raise.
"""
import ctypes
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwbgb300.so")

WB_OK, WB_ERR_CONFIG, WB_ERR_CUDA, WB_ERR_NONPHYSICAL = 0, -1, -2, -3
WB_ERR_TIMEOUT, WB_ERR_ARG, WB_ERR_NOMEM, WB_ERR_STATE = -4, -5, -6, -7
BASIS_Q, BASIS_P = 0, 1
BC_PERIODIC, BC_COPY = 0, 1
EQ_NONE, EQ_ISOTHERMAL, EQ_POLYTROPE = 0, 1, 2
LLF_MAXABS, LLF_REF2D = 0, 1
PREC_FP64, PREC_FP32 = 0, 1
RK2, RK54 = 0, 1
LIMITER_NONE, LIMITER_MINMOD, LIMITER_POSITIVITY = 0, 1, 2
RIEMANN_LLF, RIEMANN_HLLC = 0, 1
SCHEME_EQL, SCHEME_WB1 = 0, 1
LAYOUT_SOA, LAYOUT_FORTRAN = 0, 1


class WbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


class WbConfig(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "nx", "ny", "order", "basis", "bc_x", "bc_y", "eq_kind", "llf_speed", "limiter",
        "precision", "integrator", "tile_x", "tile_y", "device", "riemann", "cells_per_thread")] + [
        (n, ctypes.c_double) for n in (
            "gamma", "gx", "gy", "rho0", "p0", "kpoly", "lx", "ly", "lim_norm", "lim_M",
            "lim_tol", "cfl", "pos_eps")]


class WbPerturbation(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("nmodes", ctypes.c_int32), ("amp", ctypes.c_double),
                ("xc", ctypes.c_double), ("yc", ctypes.c_double), ("sigma", ctypes.c_double),
                ("kx", ctypes.c_double * 32), ("ky", ctypes.c_double * 32),
                ("phase_u", ctypes.c_double * 32), ("phase_v", ctypes.c_double * 32),
                ("weight", ctypes.c_double * 32)]


class Wb1dConfig(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("nx", "bc", "limiter", "eq_kind", "device", "scheme")] + [
        (n, ctypes.c_double) for n in ("gamma", "g", "rho0", "p0", "kpoly", "lx", "cfl")]


_lib = None


def lib():
    """Load libwbgb300.so (built by build.py / __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libwbgb300.so not built: run fvm-source-wb_gb300/build.py "
                               "(no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        p, i32, d = ctypes.c_void_p, ctypes.c_int32, ctypes.c_double
        sig = {
            "wb_config_default": ([p], i32), "wb_create": ([p, p], i32), "wb_destroy": ([p], i32),
            "wb_last_error": ([p], ctypes.c_char_p), "wb_status_string": ([i32], ctypes.c_char_p),
            "wb_num_modes": ([i32, i32], i32), "wb_mode_list": ([i32, i32, p, p], i32),
            "wb_upload_state": ([p, p, i32], i32), "wb_download_state": ([p, p, i32], i32),
            "wb_upload_state_f32": ([p, p], i32), "wb_download_state_f32": ([p, p], i32),
            "wb_step_io_f32": ([p, p, p, i32, ctypes.c_double], i32),
            "wb_selftest_wait_timeout": ([p, i32], i32),
            "wb_set_equilibrium": ([p, i32, ctypes.c_double, ctypes.c_double, p], i32),
            "wb_download_state_raw": ([p, p], i32),
            "wb_init_perturbation": ([p, p], i32), "wb_device_state": ([p, p, p], i32),
            "wb_compute_update": ([p, p, p, i32], i32), "wb_apply_limiter": ([p], i32),
            "wb_max_speed": ([p, p, p], i32), "wb_step": ([p, i32, d], i32),
            "wb_evolve": ([p, d, i32, p, p], i32), "wb_sync": ([p], i32),
            "wb_get_time": ([p, p, p], i32), "wb_set_time": ([p, d, ctypes.c_int64], i32),
            "wb_norms": ([p, p, p, p, p], i32), "wb_write_dat": ([p, ctypes.c_char_p, i32], i32),
            "wb_conserved_sums": ([p, p], i32), "wb_get_stream": ([p, p], i32),
            "wb_profile_stages": ([p, i32], i32), "wb_stage_stats": ([p, p, p], i32),
            "wb_autotune": ([p, i32, p, p, p], i32),
            "wb_batch_create": ([p, i32, p], i32), "wb_batch_destroy": ([p], i32),
            "wb_batch_last_error": ([p], ctypes.c_char_p),
            "wb_batch_init_perturbation": ([p, p], i32), "wb_batch_step": ([p, i32, d], i32),
            "wb_batch_sync": ([p], i32), "wb_batch_download": ([p, i32, p], i32),
            "wb_batch_total_dofs": ([p, p], i32), "wb_batch_autotune": ([p, i32, p], i32),
            "wb1d_create": ([p, p], i32), "wb1d_destroy": ([p], i32),
            "wb1d_last_error": ([p], ctypes.c_char_p), "wb1d_upload": ([p, p], i32),
            "wb1d_download": ([p, p], i32), "wb1d_compute_update": ([p, p, p], i32),
            "wb1d_evolve": ([p, d, i32, p, p], i32),
            "wb1d_write_dat": ([p, ctypes.c_char_p, i32], i32),
            "wb_read_dat": ([ctypes.c_char_p, i32, p, ctypes.c_int64, p], i32),
            "wb_norms_device_noalloc": ([i32, i32, i32, i32, d, d, p, p, ctypes.c_size_t, p,
                                         p, p, p], i32),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def num_modes(order, basis):
    return lib().wb_num_modes(order, basis)


def mode_list(order, basis):
    n = num_modes(order, basis)
    a = np.zeros(n, np.int32)
    b = np.zeros(n, np.int32)
    lib().wb_mode_list(order, basis, _ptr(a), _ptr(b))
    return a, b


def read_dat(path, ncols):
    """Records of a text snapshot in the reference's '(7(1PE12.5,1X))' format as an
    (nrows, ncols) array (wb_read_dat; a host-only call, no GPU needed)."""
    cap = os.path.getsize(path) // (13 * ncols) + 1  # every value takes 13 columns
    out = np.zeros((cap, ncols))
    n = ctypes.c_int64()
    rc = lib().wb_read_dat(os.fsencode(path), int(ncols), _ptr(out), cap, ctypes.byref(n))
    if rc != WB_OK:
        raise WbError(rc, "cannot read %s as %d-column records" % (path, ncols))
    return out[:n.value].copy()


def read_output_file(path, nx, ny, var=1):
    """A 2D snapshot of output_file read back as get_image does (post_processing2d.py:55-64):
    x, y and the fields w - w_eq of variables var..4, each shaped (nx, ny)."""
    data = read_dat(path, 2 + 5 - var)
    if data.shape[0] != nx * ny:
        raise WbError(WB_ERR_ARG, "%s holds %d records, not %d" % (path, data.shape[0], nx * ny))
    cols = [data[:, k].reshape(nx, ny) for k in range(data.shape[1])]
    return cols[0], cols[1], cols[2:]


def default_config(**kw):
    c = WbConfig()
    lib().wb_config_default(ctypes.byref(c))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c


# ---------------------------------------------------------------- seeded inputs

_M64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014) -> uniform doubles in [0,1)."""

    def __init__(self, seed):
        self.s = seed & _M64

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & _M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self):
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)


def gaussian_bump(amp, xc=0.5, yc=0.5, sigma=0.05):
    ic = WbPerturbation()
    ic.kind, ic.amp, ic.xc, ic.yc, ic.sigma = 1, amp, xc, yc, sigma
    return ic


def seeded_gaussian_bump(seed, amp, sigma=0.05):
    """Gaussian pressure bump with centre U(0.2,0.8)^2 drawn from splitmix64(seed)."""
    r = SplitMix64(seed)
    xc = 0.2 + 0.6 * r.uniform()
    yc = 0.2 + 0.6 * r.uniform()
    return gaussian_bump(amp, xc, yc, sigma)


def seeded_multimode(seed, nmodes=16, amp=1e-2, kmax=8):
    """Velocity field amp * sum_m (1/nmodes) sin(2 pi (kx x + ky y) + phase), integer
    (kx, ky) in [1,kmax]^2 and phases U(0, 2 pi) drawn from splitmix64(seed)."""
    r = SplitMix64(seed)
    ic = WbPerturbation()
    ic.kind, ic.nmodes, ic.amp = 2, nmodes, amp
    tpi = 2.0 * math.pi
    for m in range(nmodes):
        ic.kx[m] = 1 + int(kmax * r.uniform())
        ic.ky[m] = 1 + int(kmax * r.uniform())
        ic.phase_u[m] = tpi * r.uniform()
        ic.phase_v[m] = tpi * r.uniform()
        ic.weight[m] = 1.0 / nmodes
    return ic


# ---------------------------------------------------------------- workloads

def workload(name, precision=PREC_FP32, **over):
    """Configurations of the published workloads (2D ones).

    cfg2: 256^2 P1, isothermal Phi = x + y, pressure bump 1e-3 (sigma 0.05) at the centre,
          minmod limiter, SSP-RK2, CFL 0.3.
    cfg3: 2048^2 P2, polytrope K = 1, Phi = y, seeded pressure bump (sigma 0.05).
    cfg5: 8192^2 P2, isothermal Phi = 0.1 y, 16-mode seeded velocity field, amp 1e-2.
    """
    if name == "cfg2":
        c = dict(nx=256, ny=256, order=1, basis=BASIS_P, bc_x=BC_COPY, bc_y=BC_COPY,
                 eq_kind=EQ_ISOTHERMAL, gx=1.0, gy=1.0, rho0=1.0, p0=1.0, limiter=1, cfl=0.3)
    elif name == "cfg3":
        c = dict(nx=2048, ny=2048, order=2, basis=BASIS_P, bc_x=BC_COPY, bc_y=BC_COPY,
                 eq_kind=EQ_POLYTROPE, gx=0.0, gy=1.0, kpoly=1.0, limiter=0, cfl=0.3)
    elif name == "cfg5":
        c = dict(nx=8192, ny=8192, order=2, basis=BASIS_P, bc_x=BC_PERIODIC, bc_y=BC_COPY,
                 eq_kind=EQ_ISOTHERMAL, gx=0.0, gy=0.1, rho0=1.0, p0=1.0, limiter=0, cfl=0.3)
    else:
        raise KeyError(name)
    c.update(precision=precision, integrator=RK2, gamma=1.4, lx=1.0, ly=1.0)
    c.update(over)
    return c


def workload_ic(name, amp=None):
    if name == "cfg2":
        return gaussian_bump(1e-3 if amp is None else amp, 0.5, 0.5, 0.05)
    if name == "cfg3":
        return seeded_gaussian_bump(3, 1e-3 if amp is None else amp, 0.05)
    if name == "cfg5":
        return seeded_multimode(5, 16, 1e-2 if amp is None else amp, 8)
    raise KeyError(name)


# ---------------------------------------------------------------- the solver

class Solver:
    """One context: the state of compute_update / evolve for one grid."""

    def __init__(self, config=None, **kw):
        L = lib()
        c = config if config is not None else default_config()
        for k, v in kw.items():
            setattr(c, k, v)
        self.cfg = c
        self._ctx = ctypes.c_void_p()
        rc = L.wb_create(ctypes.byref(c), ctypes.byref(self._ctx))
        if rc != WB_OK:
            msg = L.wb_last_error(self._ctx).decode() if self._ctx else "wb_create failed"
            if self._ctx:
                L.wb_destroy(self._ctx)
            self._ctx = None
            raise WbError(rc, msg)
        self.nb = num_modes(c.order, c.basis)
        self.dtype = np.float32 if c.precision == PREC_FP32 else np.float64

    # -- plumbing
    def _check(self, rc):
        if rc != WB_OK:
            raise WbError(rc, lib().wb_last_error(self._ctx).decode())

    def close(self):
        if self._ctx:
            lib().wb_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def shape(self):
        return (4, self.nb, self.cfg.ny, self.cfg.nx)

    @property
    def dofs(self):
        return 4 * self.nb * self.cfg.nx * self.cfg.ny

    def fortran_shape(self):
        k = self.cfg.order + 1
        return (4, self.cfg.nx, self.cfg.ny, k, k)

    # -- state
    def upload(self, delta, layout=LAYOUT_SOA):
        if layout == LAYOUT_FORTRAN:
            a = np.asfortranarray(delta, dtype=np.float64)
        else:
            a = np.ascontiguousarray(delta, dtype=np.float64).reshape(self.shape)
        self._check(lib().wb_upload_state(self._ctx, _ptr(a), layout))

    def download(self, layout=LAYOUT_SOA):
        if layout == LAYOUT_FORTRAN:
            out = np.zeros(self.fortran_shape(), dtype=np.float64, order="F")
        else:
            out = np.zeros(self.shape, dtype=np.float64)
        self._check(lib().wb_download_state(self._ctx, _ptr(out), layout))
        return out

    def download_raw(self):
        """The resident state as stored (before the limit-on-load), in the context's precision."""
        out = np.zeros(self.shape, dtype=self.dtype)
        self._check(lib().wb_download_state_raw(self._ctx, _ptr(out)))
        return out

    def upload_f32(self, delta):
        a = np.ascontiguousarray(delta, dtype=np.float32).reshape(self.shape)
        self._check(lib().wb_upload_state_f32(self._ctx, _ptr(a)))

    def download_f32(self):
        out = np.zeros(self.shape, dtype=np.float32)
        self._check(lib().wb_download_state_f32(self._ctx, _ptr(out)))
        return out

    def init_perturbation(self, ic):
        self._check(lib().wb_init_perturbation(self._ctx, ctypes.byref(ic)))

    def device_state(self):
        p = ctypes.c_void_p()
        s = ctypes.c_size_t()
        self._check(lib().wb_device_state(self._ctx, ctypes.byref(p), ctypes.byref(s)))
        return p.value, s.value

    # -- the reference's step routines
    def compute_update(self, delta_u, layout=LAYOUT_SOA):
        """dudt for a perturbation state: compute_update(delta_u, x, y, u_eq, dudt)."""
        if layout == LAYOUT_FORTRAN:
            a = np.asfortranarray(delta_u, dtype=np.float64)
            out = np.zeros(self.fortran_shape(), dtype=np.float64, order="F")
        else:
            a = np.ascontiguousarray(delta_u, dtype=np.float64).reshape(self.shape)
            out = np.zeros(self.shape, dtype=np.float64)
        self._check(lib().wb_compute_update(self._ctx, _ptr(a), _ptr(out), layout))
        return out

    def apply_limiter(self):
        self._check(lib().wb_apply_limiter(self._ctx))

    def compute_max_speed(self):
        sx = ctypes.c_double()
        sy = ctypes.c_double()
        self._check(lib().wb_max_speed(self._ctx, ctypes.byref(sx), ctypes.byref(sy)))
        return sx.value, sy.value

    def step(self, nsteps=1, dt=-1.0):
        self._check(lib().wb_step(self._ctx, int(nsteps), float(dt)))

    def sync(self):
        self._check(lib().wb_sync(self._ctx))

    def time(self):
        t = ctypes.c_double()
        n = ctypes.c_int64()
        self._check(lib().wb_get_time(self._ctx, ctypes.byref(t), ctypes.byref(n)))
        return t.value, n.value

    def output_file(self, path, var=1):
        """Text snapshot in the reference's output_file format ('(7(1PE12.5,1X))')."""
        self._check(lib().wb_write_dat(self._ctx, os.fsencode(path), int(var)))

    def set_time(self, t, steps):
        self._check(lib().wb_set_time(self._ctx, float(t), int(steps)))

    # -- checkpoint / restart (binary: magic, JSON header, raw SoA state)
    _MAGIC = b"WBGB300\x00"

    def save_checkpoint(self, path):
        """Writes config, t, step count and the resident state as stored (before the
        limit-on-load); a restart from it continues bit for bit."""
        t, n = self.time()
        state = self.download_raw()
        hdr = {"config": {k: getattr(self.cfg, k) for k, _ in WbConfig._fields_},
               "t": t, "steps": n, "dtype": str(state.dtype), "shape": list(state.shape)}
        h = json.dumps(hdr).encode()
        with open(path, "wb") as f:
            f.write(self._MAGIC)
            f.write(np.uint32(len(h)).tobytes())
            f.write(h)
            f.write(np.ascontiguousarray(state).tobytes())

    @classmethod
    def read_checkpoint(cls, path):
        with open(path, "rb") as f:
            if f.read(8) != cls._MAGIC:
                raise ValueError("not a checkpoint: %s" % path)
            n = int(np.frombuffer(f.read(4), np.uint32)[0])
            hdr = json.loads(f.read(n).decode())
            state = np.frombuffer(f.read(), dtype=hdr["dtype"]).reshape(hdr["shape"])
        return hdr, state

    def load_checkpoint(self, path):
        hdr, state = self.read_checkpoint(path)
        c = hdr["config"]
        for k in ("nx", "ny", "order", "basis", "precision"):
            if c[k] != getattr(self.cfg, k):
                raise ValueError("checkpoint %s=%s does not match the solver's %s"
                                 % (k, c[k], getattr(self.cfg, k)))
        if state.dtype == np.float32:
            self.upload_f32(state)
        else:
            self.upload(state)
        self.set_time(hdr["t"], hdr["steps"])

    @classmethod
    def from_checkpoint(cls, path, device=0):
        hdr, _ = cls.read_checkpoint(path)
        c = default_config(**dict(hdr["config"], device=device))
        s = cls(config=c)
        s.load_checkpoint(path)
        return s

    def evolve(self, tend, max_steps=2**31 - 1):
        steps = ctypes.c_int32()
        t = ctypes.c_double()
        self._check(lib().wb_evolve(self._ctx, float(tend), int(max_steps), ctypes.byref(steps),
                                    ctypes.byref(t)))
        return steps.value, t.value

    def compute_error(self, other=None):
        """(L1, Linf, L2) per conserved variable of self - other (compute_error)."""
        l1, linf, l2 = np.zeros(4), np.zeros(4), np.zeros(4)
        o = other._ctx if other is not None else None
        self._check(lib().wb_norms(self._ctx, o, _ptr(l1), _ptr(linf), _ptr(l2)))
        return l1, linf, l2

    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        p = ctypes.c_void_p()
        self._check(lib().wb_get_stream(self._ctx, ctypes.byref(p)))
        return p.value or 0

    def autotune(self, steps=3):
        """Pick the fastest compiled tile shape and cells per thread for this grid (state
        is preserved); returns (tile_x, tile_y, cells_per_thread)."""
        tx = ctypes.c_int32()
        ty = ctypes.c_int32()
        cpt = ctypes.c_int32()
        self._check(lib().wb_autotune(self._ctx, int(steps), ctypes.byref(tx), ctypes.byref(ty),
                                      ctypes.byref(cpt)))
        return tx.value, ty.value, cpt.value

    def profile_stages(self, on=True):
        self._check(lib().wb_profile_stages(self._ctx, 1 if on else 0))

    def stage_stats(self):
        """(summed stage-kernel milliseconds, launches) since the last call."""
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        self._check(lib().wb_stage_stats(self._ctx, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def upload_f32_ptr(self, host_ptr):
        """Upload from a raw host address holding a dense float32 SoA state."""
        self._check(lib().wb_upload_state_f32(self._ctx, ctypes.c_void_p(host_ptr)))

    def set_equilibrium(self, eq_kind, gx, gy, rho0=None, p0=None, kpoly=None):
        """Replace the hydrostatic equilibrium; the perturbation state is kept."""
        params = None
        if rho0 is not None or p0 is not None or kpoly is not None:
            params = np.array([self.cfg.rho0 if rho0 is None else rho0,
                               self.cfg.p0 if p0 is None else p0,
                               self.cfg.kpoly if kpoly is None else kpoly], dtype=np.float64)
        self._check(lib().wb_set_equilibrium(self._ctx, int(eq_kind), float(gx), float(gy),
                                             _ptr(params) if params is not None else None))
        self.cfg.eq_kind, self.cfg.gx, self.cfg.gy = eq_kind, gx, gy
        if params is not None:
            self.cfg.rho0, self.cfg.p0, self.cfg.kpoly = params

    def selftest_wait_timeout(self, polls=4096):
        """Status of the bounded-wait self-test (WB_ERR_TIMEOUT expected)."""
        return lib().wb_selftest_wait_timeout(self._ctx, int(polls))

    def step_io_f32_ptr(self, in_ptr, out_ptr, nsteps=1, dt=-1.0):
        """Pipelined: upload from in_ptr, step, download into out_ptr; returns at once.
        Both host buffers belong to the library until sync()."""
        self._check(lib().wb_step_io_f32(self._ctx, ctypes.c_void_p(in_ptr),
                                         ctypes.c_void_p(out_ptr), int(nsteps), float(dt)))

    def download_f32_ptr(self, host_ptr):
        self._check(lib().wb_download_state_f32(self._ctx, ctypes.c_void_p(host_ptr)))

    def conserved_sums(self):
        s = np.zeros(4)
        self._check(lib().wb_conserved_sums(self._ctx, _ptr(s)))
        return s


# ---------------------------------------------------------------- batched form

def batch_workload(n=512, seed_base=1000, nmin=32, nmax=512, device=0):
    """Independent instances of the batched workload: instance i draws from
    splitmix64(seed_base + i) its side N = round(exp(U(ln nmin, ln nmax))), degree in
    {0,1,2}, isothermal or polytropic atmosphere (Phi = y), and a Gaussian pressure bump
    of amplitude 10^U(-6,-2), centre U(0.2,0.8)^2, width U(0.02,0.1)."""
    cfgs, ics = [], []
    for i in range(n):
        r = SplitMix64(seed_base + i)
        side = int(round(math.exp(math.log(nmin) + (math.log(nmax) - math.log(nmin)) * r.uniform())))
        order = min(2, int(3 * r.uniform()))
        eq = EQ_ISOTHERMAL if r.uniform() < 0.5 else EQ_POLYTROPE
        amp = 10.0 ** (-6.0 + 4.0 * r.uniform())
        xc = 0.2 + 0.6 * r.uniform()
        yc = 0.2 + 0.6 * r.uniform()
        sigma = 0.02 + 0.08 * r.uniform()
        c = default_config(nx=side, ny=side, order=order, basis=BASIS_P, bc_x=BC_COPY,
                           bc_y=BC_COPY, eq_kind=eq, gx=0.0, gy=1.0, rho0=1.0, p0=1.0,
                           kpoly=1.0, limiter=0, precision=PREC_FP32, integrator=RK2, cfl=0.3,
                           device=device)
        cfgs.append(c)
        ics.append(gaussian_bump(amp, xc, yc, sigma))
    return cfgs, ics


class Batch:
    """Many independent instances advanced by one persistent launch per RK stage."""

    def __init__(self, cfgs):
        L = lib()
        arr = (WbConfig * len(cfgs))(*cfgs)
        self._b = ctypes.c_void_p()
        rc = L.wb_batch_create(arr, len(cfgs), ctypes.byref(self._b))
        if rc != WB_OK:
            msg = L.wb_batch_last_error(self._b).decode() if self._b else "wb_batch_create failed"
            if self._b:
                L.wb_batch_destroy(self._b)
            self._b = None
            raise WbError(rc, msg)
        self.cfgs = list(cfgs)

    def _check(self, rc):
        if rc != WB_OK:
            raise WbError(rc, lib().wb_batch_last_error(self._b).decode())

    def close(self):
        if self._b:
            lib().wb_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def init_perturbation(self, ics):
        arr = (WbPerturbation * len(ics))(*ics)
        self._check(lib().wb_batch_init_perturbation(self._b, arr))

    def step(self, nsteps=1, dt=-1.0):
        self._check(lib().wb_batch_step(self._b, int(nsteps), float(dt)))

    def autotune(self, reps=3):
        """Pick the tile shape and cells per thread of every (degree, size class) group by
        timing; returns {(degree, size_class): (TX, TY, CPT)} (size class 0: max(nx, ny) <
        128)."""
        t = np.zeros(18, dtype=np.int32)
        self._check(lib().wb_batch_autotune(self._b, int(reps), _ptr(t)))
        return {(k, c): tuple(int(v) for v in t[(2 * k + c) * 3:(2 * k + c) * 3 + 3])
                for k in range(3) for c in range(2)}

    def sync(self):
        self._check(lib().wb_batch_sync(self._b))

    def download(self, index):
        c = self.cfgs[index]
        out = np.zeros((4, num_modes(c.order, c.basis), c.ny, c.nx))
        self._check(lib().wb_batch_download(self._b, int(index), _ptr(out)))
        return out

    @property
    def dofs(self):
        n = ctypes.c_int64()
        self._check(lib().wb_batch_total_dofs(self._b, ctypes.byref(n)))
        return n.value


# ---------------------------------------------------------------- 1D finite volume

class Solver1D:
    """compute_update / evolve of benchmark_1d.f90 (the fvm.f90 path) on the device, FP64.

    State layout: delta[i, v], v = 0..2 is the (rho, rho*u, E) perturbation of cell i.
    """

    def __init__(self, nx=256, bc=BC_COPY, limiter=1, eq_kind=EQ_ISOTHERMAL, gamma=1.4, g=1.0,
                 rho0=1.0, p0=1.0, kpoly=1.0, lx=1.0, cfl=0.4, device=0, scheme=0):
        """scheme: SCHEME_EQL ('EQL', equilibrium + perturbation faces) or SCHEME_WB1
        ('WB1', hydrostatic reconstruction of compute_update_sr)."""
        L = lib()
        c = Wb1dConfig()
        c.nx, c.bc, c.limiter, c.eq_kind, c.device = nx, bc, limiter, eq_kind, device
        c.scheme = scheme
        c.gamma, c.g, c.rho0, c.p0, c.kpoly, c.lx, c.cfl = gamma, g, rho0, p0, kpoly, lx, cfl
        self.cfg = c
        self._c = ctypes.c_void_p()
        rc = L.wb1d_create(ctypes.byref(c), ctypes.byref(self._c))
        if rc != WB_OK:
            msg = L.wb1d_last_error(self._c).decode() if self._c else "wb1d_create failed"
            if self._c:
                L.wb1d_destroy(self._c)
            self._c = None
            raise WbError(rc, msg)

    def _check(self, rc):
        if rc != WB_OK:
            raise WbError(rc, lib().wb1d_last_error(self._c).decode())

    def close(self):
        if self._c:
            lib().wb1d_destroy(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, delta):
        a = np.ascontiguousarray(delta, dtype=np.float64).reshape(self.cfg.nx, 3)
        self._check(lib().wb1d_upload(self._c, _ptr(a)))

    def download(self):
        out = np.zeros((self.cfg.nx, 3))
        self._check(lib().wb1d_download(self._c, _ptr(out)))
        return out

    def compute_update(self, delta):
        a = np.ascontiguousarray(delta, dtype=np.float64).reshape(self.cfg.nx, 3)
        out = np.zeros((self.cfg.nx, 3))
        self._check(lib().wb1d_compute_update(self._c, _ptr(a), _ptr(out)))
        return out

    def evolve(self, tend, max_steps=10**8):
        n = ctypes.c_int32()
        t = ctypes.c_double()
        self._check(lib().wb1d_evolve(self._c, float(tend), int(max_steps), ctypes.byref(n),
                                      ctypes.byref(t)))
        return n.value, t.value

    def output_file(self, path, var=3):
        """Text snapshot in benchmark_1d.f90's output_file format: x and w - w_eq of the
        primitive variables var..3 at the cell centres (the reference writes var = 3)."""
        self._check(lib().wb1d_write_dat(self._c, os.fsencode(path), int(var)))

    @staticmethod
    def read_output_file(path, var=3):
        """(x, [w - w_eq for variables var..3]) of a 1D snapshot."""
        data = read_dat(path, 1 + 4 - var)
        return data[:, 0], [data[:, k] for k in range(1, data.shape[1])]
