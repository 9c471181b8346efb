"""In-tree build of libwbgb300.so for sm_103a (nvcc, translation units in parallel).

    python fvm-source-wb_gb300/build.py [--force]
"""
import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libwbgb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
SOURCES = ["wb_kernels_f64.cu", "wb_kernels_f32.cu", "wb_capi.cu", "wb_batch.cu", "wb_fv1d.cu",
           "wb_noalloc.cu", "wb_stage_dispatch.cu", "wb_tables.cpp", "wb_dat.cpp"]
GEN = os.path.join(OUT, "gen")


def stage_instances():
    """The lines of WB_STAGE_INSTANCES (csrc/wb_stage_instances.h):
    (P, R, K, BT, B, TX, TY, VAR, CPT)."""
    txt = open(os.path.join(CSRC, "wb_stage_instances.h")).read()
    pat = r"X\((f\d+), (\w+), (\d), (\w), (\d), (\d+), (\d+), (\d), (\d)\)"
    return re.findall(pat, txt)


def batch_instances():
    """The lines of WB_BATCH_INSTANCES: (K, TX, TY, POS, CPT)."""
    txt = open(os.path.join(CSRC, "wb_stage_instances.h")).read()
    return re.findall(r"X\((\d), (\d+), (\d+), (\d), (\d)\)", txt)


def _write_unit(name, body):
    path = os.path.join(GEN, name)
    if not os.path.exists(path) or open(path).read() != body:
        with open(path, "w") as f:
            f.write(body)
    return path


def generate_stage_units():
    """One translation unit per compiled stage kernel and per batched stage kernel (so
    nvcc runs them in parallel)."""
    os.makedirs(GEN, exist_ok=True)
    names = []
    for inst in stage_instances():
        P, R, K, BT, B, TX, TY, VAR, CPT = inst
        name = "stage_%s_k%s%s_%sx%s_%s_c%s.cu" % (P, K, BT, TX, TY, VAR, CPT)
        names.append(_write_unit(name, '// generated by build.py from wb_stage_instances.h\n'
                                       '#include "wb_stage_launch.cuh"\n'
                                       'WB_STAGE_INSTANCE(%s)\n' % ", ".join(inst)))
    for inst in batch_instances():
        K, TX, TY, POS, CPT = inst
        name = "batch_k%s_%sx%s_%s_c%s.cu" % (K, TX, TY, POS, CPT)
        names.append(_write_unit(name, '// generated by build.py from wb_stage_instances.h\n'
                                       '#include "wb_batch_launch.cuh"\n'
                                       'WB_BATCH_INSTANCE(%s)\n' % ", ".join(inst)))
    # units of instances no longer listed are not linked
    keep = {os.path.basename(n) for n in names}
    for f in os.listdir(GEN):
        if f.endswith(".cu") and f not in keep:
            os.remove(os.path.join(GEN, f))
    return names


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
    s = src if os.path.isabs(src) else os.path.join(CSRC, src)
    o = os.path.join(OUT, os.path.basename(src).rsplit(".", 1)[0] + ".o")
    if not force and not _stale(o, s, _deps()):
        return o, None
    cmd = [NVCC] + ARCH + FLAGS + ["-I", CSRC, "-c", s, "-o", o]
    if src.endswith(".cpp"):
        cmd = [NVCC] + FLAGS + ["-x", "c++", "-c", s, "-o", o]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return o, "compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr)
    return o, None


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    # slowest units first: the generated stage kernels, then the rest
    srcs = generate_stage_units() + SOURCES
    srcs.sort(key=lambda p: 0 if "_k2" in p else 1)
    keep = {os.path.basename(p).rsplit(".", 1)[0] + ".o" for p in srcs}
    for f in os.listdir(OUT):  # objects of units no longer built are not linked
        if f.endswith(".o") and f not in keep:
            os.remove(os.path.join(OUT, f))
    jobs = max(2, min(len(srcs), os.cpu_count() or 8))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
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
