"""The TMA tile staging and the cp.async staging (WB_NO_TMA=1) stage the same bytes, so
they give bit-identical results.  The switch is read once per process, so each path runs
in its own subprocess."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import importlib.util, json, sys
import numpy as np
sys.path.insert(0, %(tests)r)
sys.path.insert(0, %(oracle)r)
spec = importlib.util.spec_from_file_location("wbt", %(pkg)r)
wb = importlib.util.module_from_spec(spec); sys.modules["wbt"] = wb; spec.loader.exec_module(wb)
from helpers import base_cfg, random_delta, solver
out = {}
for precision in (0, 1):
    for limiter in (0, 1):
        c = base_cfg(nx=128, ny=72, order=2, basis=1, eq_kind=1, gx=0.0, gy=1.0, bc_x=0,
                     bc_y=1, limiter=limiter)
        d = random_delta(c, amp=1e-2, seed=31 + limiter)
        with solver(wb, c, precision) as s:
            s.upload(d)
            s.step(5)
            out["%%d_%%d" %% (precision, limiter)] = s.download().tolist()
json.dump(out, open(sys.argv[1], "w"))
'''


def _run(tmp_path, name, no_tma):
    script = SCRIPT % {"tests": os.path.join(ROOT, "tests"), "oracle": os.path.join(ROOT, "oracle"),
                       "pkg": os.path.join(ROOT, "fvm-source-wb_gb300", "__init__.py")}
    env = dict(os.environ)
    env.pop("WB_NO_TMA", None)
    if no_tma:
        env["WB_NO_TMA"] = "1"
    path = str(tmp_path / (name + ".json"))
    subprocess.run([sys.executable, "-c", script, path], check=True, env=env, timeout=600)
    return json.load(open(path))


def test_tma_and_cp_async_staging_agree_bitwise(tmp_path):
    a = _run(tmp_path, "tma", False)
    b = _run(tmp_path, "cpasync", True)
    assert a.keys() == b.keys()
    for k in a:
        np.testing.assert_array_equal(np.array(a[k]), np.array(b[k]), err_msg=k)
