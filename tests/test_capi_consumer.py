"""A compiled C consumer of include/wb_capi.h (tests/capi_consumer.c), built with gcc and
linked to libwbgb300.so: the struct layouts the header gives a C or Fortran bind(C)
caller must equal the ctypes mirrors of the Python package (CPU), and the ABI driven
from C through the Fortran state layout must reproduce the oracle's evolve (GPU)."""
import ctypes
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import base_cfg, orc_cfg, random_delta, rel_l1_full

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def consumer(tmp_path_factory, wb):
    wb.lib()  # the library is built
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(wb.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("capi") / "capi_consumer")
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "capi_consumer.c"),
           "-o", exe, "-L", libdir, "-lwbgb300", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _mirror_layout(struct):
    out = {struct.__name__: ctypes.sizeof(struct)}
    for name, _ in struct._fields_:
        out["%s.%s" % (struct.__name__, name)] = getattr(struct, name).offset
    return out


def test_struct_layouts_match_the_ctypes_mirrors(wb, consumer):
    r = subprocess.run([consumer, "layout"], capture_output=True, text=True, check=True)
    got = json.loads(r.stdout)
    want = {}
    for struct, cname in ((wb.WbConfig, "wb_config"), (wb.WbPerturbation, "wb_perturbation"),
                          (wb.Wb1dConfig, "wb1d_config")):
        for k, v in _mirror_layout(struct).items():
            want[k.replace(struct.__name__, cname)] = v
    assert got == want


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_c_driver_evolve_matches_oracle(wb, orc, consumer, tmp_path, order):
    """wb_create, wb_upload_state(WB_LAYOUT_FORTRAN), wb_max_speed, wb_evolve,
    wb_download_state(WB_LAYOUT_FORTRAN), wb_norms, wb_step + wb_sync -- called from C --
    against the oracle: tensor basis, isothermal Phi = x + y, minmod, SSP-RK2, CFL 0.3."""
    nx, ny, tend = 20, 14, 0.02
    c = base_cfg(nx=nx, ny=ny, order=order, basis=0, bc_x=1, bc_y=1, eq_kind=1, gx=1.0, gy=1.0,
                 limiter=1, cfl=0.3, lim_tol=1e-6)
    d = random_delta(c, amp=1e-2, seed=40 + order)
    a, b = orc.modes(order, 0)
    k = order + 1
    f = np.zeros((4, nx, ny, k, k), order="F")  # u(nvar, nx, ny, mx, my)
    for m in range(len(a)):
        f[:, :, :, a[m], b[m]] = d[:, m].transpose(0, 2, 1)
    fin, fout, fout2 = (str(tmp_path / n) for n in ("in.bin", "out.bin", "out2.bin"))
    f.ravel(order="F").tofile(fin)
    r = subprocess.run([consumer, "evolve", fin, fout, fout2, str(nx), str(ny), str(order),
                        repr(tend)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    res = json.loads(r.stdout)

    def soa(path):
        g = np.fromfile(path).reshape((4, nx, ny, k, k), order="F")
        return np.stack([g[:, :, :, a[m], b[m]].transpose(0, 2, 1) for m in range(len(a))], 1)

    oc = orc_cfg(c)
    sx, sy = orc.max_speed(oc, d)
    assert abs(res["smax"][0] - sx) <= 1e-14 * sx and abs(res["smax"][1] - sy) <= 1e-14 * sy
    n = res["steps"]
    assert n > 3 and abs(res["t"] - tend) < 1e-15
    ref, tref = orc.run_rk2(oc, d, n - 1, -1.0)
    ref, _ = orc.run_rk2(oc, ref, 1, tend - tref)   # evolve's last step is clipped at tend
    got = soa(fout)
    assert np.all(rel_l1_full(c, got, ref) < 1e-12)
    l1, linf, _ = orc.norms(oc, ref, np.zeros_like(ref))
    np.testing.assert_allclose(res["l1"], l1, rtol=1e-11)
    np.testing.assert_allclose(res["linf"], linf, rtol=1e-11)
    ref2, _ = orc.run_rk2(oc, ref, 2, 1e-4)
    assert np.all(rel_l1_full(c, soa(fout2), ref2) < 1e-12)
    assert res["steps2"] == n + 2 and abs(res["t2"] - (tend + 2e-4)) < 1e-15
