"""In-tree build of libwbgb300.so for sm_103a (nvcc, translation units in parallel).

    python fvm-source-wb_gb300/build.py [--force]
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libwbgb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
SOURCES = ["wb_stage_f32_k2p.cu", "wb_stage_f32_k2q.cu", "wb_stage_f64_k2p.cu",
           "wb_stage_f64_k2q.cu", "wb_kernels_f64.cu", "wb_kernels_f32.cu", "wb_stage_f32_k1p.cu",
           "wb_stage_f32_k1q.cu", "wb_stage_f64_k1p.cu", "wb_stage_f64_k1q.cu", "wb_stage_f32_k0.cu",
           "wb_stage_f64_k0.cu", "wb_capi.cu", "wb_batch.cu", "wb_fv1d.cu", "wb_noalloc.cu", "wb_tables.cpp"]


def _deps():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "wb_capi.h"))
    return hs


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps if os.path.exists(p))


def _compile(src, force):
    s = os.path.join(CSRC, src)
    o = os.path.join(OUT, src.rsplit(".", 1)[0] + ".o")
    if not force and not _stale(o, s, _deps()):
        return o, None
    cmd = [NVCC] + ARCH + FLAGS + ["-c", s, "-o", o]
    if src.endswith(".cpp"):
        cmd = [NVCC] + FLAGS + ["-x", "c++", "-c", s, "-o", o]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return o, "compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr)
    return o, None


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("\n".join(errs))
    objs = [o for o, _ in results]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
