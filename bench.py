"""Benchmark of the well-balanced Euler-with-gravity step (DOF-updates/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (N=1): the 8192x8192 P2 bandwidth-stress configuration -- isothermal
atmosphere Phi = 0.1 y, rho = p = exp(-0.1 y), 16-mode seeded velocity perturbation of
amplitude 1e-2 -- advanced by SSP-RK2 with device-computed CFL steps (CFL 0.3) in the
FP32-perturbation form.  One step = one full time step (two fused RK stages + CFL
reduction) over the whole grid.  Inputs (6.4 GB of FP32 state) are far larger than L2.
Beside it: the FP64 plain method on the same grid (DOF-updates/s and the L1 error of the
FP32 form against it), the end-to-end rate through the C ABI with pinned host buffers,
and the CPU oracle on a bounded sample.  For N > 1 (torchrun) every rank advances its own
independent replica ("replicas only": the path has no data exchange on one GPU each).
"""
import argparse
import csv
import importlib.util
import io
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
METRIC = "DOF-updates/s on 1 GB300: FP32-perturbation vs FP64 plain at L1 err<=1e-6"
UNIT = "DOF-updates/s"
BYTES_PER_DOF_UPDATE = {"fp32": 20.0, "fp64": 40.0}  # SSP-RK2: 5 state accesses per DOF


def load_package():
    name = "fvm_source_wb_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(
        name, os.path.join(ROOT, "fvm-source-wb_gb300", "__init__.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(workload):
    """Per-launch DRAM bytes of the stage kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "k_stage_%s_traffic.json" % workload)
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = tempfile.TemporaryFile(mode="w+")

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.f.read())) if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[5 + k]
                          and "Not" not in r[5 + k]})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    import torch.distributed as dist
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(lr)
    dist.init_process_group(backend=backend)
    return dist, dist.get_rank(), dist.get_world_size(), lr


def reduce_max(dist, x, device):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda:%d" % device if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---------------------------------------------------------------- CPU baseline

def cpu_sample(wb, seconds=12.0, n=512, min_steps=2, warm=1, threads=None):
    """The FP64 CPU oracle (OpenMP, all host threads) on an n x n grid with the cfg5
    physics; returns (DOF-updates/s, threads, sample description)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    threads = threads or os.cpu_count() or 1
    O.set_threads(threads)
    w = wb.workload("cfg5", nx=n, ny=n)
    oc = O.make_cfg(nx=n, ny=n, order=w["order"], basis=w["basis"], bc_x=w["bc_x"],
                    bc_y=w["bc_y"], eq_kind=w["eq_kind"], gx=w["gx"], gy=w["gy"],
                    rho0=w["rho0"], p0=w["p0"], limiter=w["limiter"], cfl=w["cfl"])
    ic = wb.workload_ic("cfg5")
    oic = O.make_ic(kind=2, amp=ic.amp, nmodes=ic.nmodes, kx=list(ic.kx), ky=list(ic.ky),
                    phase_u=list(ic.phase_u), phase_v=list(ic.phase_v), weight=list(ic.weight))
    d = O.project_ic(oc, oic)
    dof = d.size
    if warm:
        d, _ = O.run_rk2(oc, d, warm, -1.0)
    steps, t0 = 0, time.perf_counter()
    while steps < min_steps or time.perf_counter() - t0 < seconds:
        d, _ = O.run_rk2(oc, d, 1, -1.0)
        steps += 1
    el = time.perf_counter() - t0
    desc = ("FP64 oracle port (C, OpenMP, %d thread%s) on %dx%d cells of the cfg5 physics "
            "(P2, isothermal Phi=0.1y, 16-mode velocity field), %d SSP-RK2 CFL steps, %.1f s"
            % (threads, "" if threads == 1 else "s", n, n, steps, el))
    return dof * steps / el, threads, desc


def run_reference(args):
    # rank 0 alone runs the CPU reference; the other ranks exit at once (no process
    # group: nothing to rendezvous on)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    wb = load_package()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    n = args.ref_n
    w = wb.workload("cfg5", nx=n, ny=n)
    oc = O.make_cfg(nx=n, ny=n, order=w["order"], basis=w["basis"], bc_x=w["bc_x"],
                    bc_y=w["bc_y"], eq_kind=w["eq_kind"], gx=w["gx"], gy=w["gy"],
                    rho0=w["rho0"], p0=w["p0"], limiter=w["limiter"], cfl=w["cfl"])
    ic = wb.workload_ic("cfg5")
    oic = O.make_ic(kind=2, amp=ic.amp, nmodes=ic.nmodes, kx=list(ic.kx), ky=list(ic.ky),
                    phase_u=list(ic.phase_u), phase_v=list(ic.phase_v), weight=list(ic.weight))
    d = O.project_ic(oc, oic)
    dof = d.size
    d, _ = O.run_rk2(oc, d, args.warmup, -1.0)
    t0 = time.perf_counter()
    d, _ = O.run_rk2(oc, d, args.steps, -1.0)
    el = time.perf_counter() - t0
    value = dof * args.steps / el
    sample = ("each step: one SSP-RK2 CFL step of the FP64 oracle port (the reference's "
              "Fortran cannot be compiled here) on %dx%d cells of the cfg5 physics" % (n, n))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "cfg5: 8192^2 P2 isothermal Phi=0.1y, 16-mode velocity field "
                               "(CPU sample %dx%d)" % (n, n), "order": 2, "basis": "P",
                   "dofs_per_step": dof, "l2_policy": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- our arm

def parse_batch_tiles(spec):
    """'0:32x16/2,1:32x16/2,2:32x8/1' -> {degree: (TX, TY, CPT)}."""
    out = {}
    for part in filter(None, spec.split(",")):
        k, shape = part.split(":")
        dims, _, cpt = shape.lower().partition("/")
        tx, ty = (int(v) for v in dims.split("x"))
        out[int(k)] = (tx, ty, int(cpt or 1))
    return out


def batch_leg(wb, n, dev, steps=24, warmup=6, pinned=None, instances=None, label=None):
    """The batched form on n instances: DOF-updates/s over `steps` CFL steps (host clock
    around graph launches + sync, after `warmup` steps that include the graph capture), and
    its HBM roofline fraction (20 B per DOF-update per SSP-RK2 step, all stage launches).
    pinned: {degree: (TX, TY, CPT)} pins those degrees' tiles (profiling); the rest are
    autotuned.  instances: (configs, initial conditions) instead of the cfg4 draw, named by
    label."""
    cfgs, ics = instances if instances else wb.batch_workload(n=n, device=dev)
    for c in cfgs:
        if pinned and c.order in pinned:
            c.tile_x, c.tile_y, c.cells_per_thread = pinned[c.order]
    with wb.Batch(cfgs) as bt:
        bt.init_perturbation(ics)
        tiles = bt.autotune(3)
        if pinned:
            tiles.update({(k, c): pinned[k] for k in pinned for c in range(2)})
        bt.step(warmup)
        bt.sync()
        t0 = time.perf_counter()
        bt.step(steps)
        bt.sync()
        el = time.perf_counter() - t0
        dofs = bt.dofs
    peak, peak_kind = measured_hbm_peak()
    achieved = BYTES_PER_DOF_UPDATE["fp32"] * dofs * steps / el / 1e9
    return {"value": dofs * steps / el, "unit": UNIT, "instances": len(cfgs), "dofs": dofs,
            "steps": steps, "ms_per_step": el / steps * 1e3,
            "tiles": {"K%d_%s" % (k, "small" if c == 0 else "large"): "%dx%d/%d" % t
                      for (k, c), t in sorted(tiles.items())},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "kernel": "k_batch_stage<float>", "note": "whole step, host clock"},
            "workload": label or (
                "%d instances: N = exp(U(ln 32, ln 512)), degree 0..2 (P basis), "
                "isothermal or polytrope, Gaussian bump 10^U(-6,-2); FP32, SSP-RK2, "
                "CFL steps" % len(cfgs))}


def batch_accuracy(wb, n, dev, steps=20):
    """The batched form's FP32 instances against FP64 plain contexts of the same instances
    (same seeded workload), after `steps` fixed steps of one dt that satisfies every
    instance's CFL condition: L1 / Linf per conserved variable of the difference, maximum
    over the instances (norms in FP64 on the device, wb_norms)."""
    cfgs, ics = wb.batch_workload(n=n, device=dev)
    # one dt for all: the smallest instance CFL step (FP64 wave speeds of the initial state)
    dts = []
    for c, ic in zip(cfgs, ics):
        c64 = wb.default_config(**{k: getattr(c, k) for k, _ in wb.WbConfig._fields_})
        c64.precision = wb.PREC_FP64
        with wb.Solver(config=c64) as s:
            s.init_perturbation(ic)
            sx, sy = s.compute_max_speed()
            dts.append(c.cfl / (2 * c.order + 1) / (sx * c.nx / c.lx + sy * c.ny / c.ly))
    dt = 0.9 * min(dts)
    t0 = time.perf_counter()
    with wb.Batch(cfgs) as bt:
        bt.init_perturbation(ics)
        bt.step(steps, dt)
        bt.sync()
        worst_l1, worst_linf, worst_rel = np.zeros(4), np.zeros(4), 0.0
        for i, (c, ic) in enumerate(zip(cfgs, ics)):
            c64 = wb.default_config(**{k: getattr(c, k) for k, _ in wb.WbConfig._fields_})
            c64.precision = wb.PREC_FP64
            with wb.Solver(config=c64) as ref, wb.Solver(config=c64) as got:
                ref.init_perturbation(ic)
                ref.step(steps, dt)
                got.upload(bt.download(i))
                l1, linf, _ = got.compute_error(ref)
                p1, _, _ = ref.compute_error(None)
            worst_l1 = np.maximum(worst_l1, l1)
            worst_linf = np.maximum(worst_linf, linf)
            worst_rel = max(worst_rel, float(np.max(l1 / np.maximum(p1, 1e-300))))
    return {"instances": len(cfgs), "steps": steps, "dt": dt,
            "l1_fp32_vs_fp64_max": worst_l1.tolist(), "linf_fp32_vs_fp64_max": worst_linf.tolist(),
            "l1_relative_to_perturbation_max": worst_rel, "l1_bar": 1e-6,
            "pass": bool(np.all(worst_l1 <= 1e-6)), "seconds": time.perf_counter() - t0,
            "reference": "FP64 plain context of each instance, same dt and steps"}


def limited_leg(wb, name, dev, steps=6, warmup=3):
    """The headline grid with the minmod limiter on the perturbation (limit-on-load inside
    the stage kernel: the means halo is staged too): DOF-updates/s by CUDA events."""
    import torch
    w = wb.workload(name, wb.PREC_FP32, limiter=1, device=dev)
    with wb.Solver(**w) as s:
        s.init_perturbation(wb.workload_ic(name))
        s.step(warmup)
        s.sync()
        st = torch.cuda.ExternalStream(s.stream(), device=dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        s.step(steps)
        e1.record(st)
        e1.synchronize()
        s.sync()
        ms = e0.elapsed_time(e1)
        dof = s.dofs
    return {"value": dof * steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
            "steps": steps, "limiter": "minmod (compute_limiter on the perturbation)",
            "workload": "%s with the minmod limiter" % name}


def run_batch_only(args):
    wb = load_package()
    line = {"metric": "batched form: " + UNIT, "impl": "batch"}
    instances, label = None, None
    if args.batch_grid:
        # one instance: the workload's grid (at --nx), to set the batch kernel beside
        # k_stage on the same cells
        n = args.nx or wb.workload(args.workload)["nx"]
        c = wb.default_config(**wb.workload(args.workload, nx=n, ny=n))
        instances = ([c], [wb.workload_ic(args.workload)])
        label = "one instance: the %s grid at %dx%d (FP32, SSP-RK2, CFL steps)" % (
            args.workload, n, n)
    line.update(batch_leg(wb, args.batch, 0, steps=args.steps, warmup=max(args.warmup, 6),
                          pinned=parse_batch_tiles(args.batch_tiles), instances=instances,
                          label=label))
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    dist, rank, world, lr = dist_init()
    wb = load_package()
    wb.lib()  # raises if the CUDA library is missing: there is no CPU fallback
    dev = lr
    torch.cuda.set_device(dev)
    name = args.workload
    size = {} if args.nx <= 0 else {"nx": args.nx, "ny": args.nx}
    fixed = {}
    if args.tile:  # TXxTY or TXxTY/CPT
        shape, _, cpt = args.tile.lower().partition("/")
        tx, ty = (int(v) for v in shape.split("x"))
        fixed = {"tile_x": tx, "tile_y": ty, "cells_per_thread": int(cpt or 1)}
    w32 = wb.workload(name, wb.PREC_FP32, **size, **fixed)
    ic = wb.workload_ic(name)
    s32 = wb.Solver(device=dev, **w32)
    dof = s32.dofs
    s32.init_perturbation(ic)
    # fastest compiled tile shape for this grid (state preserved), unless one is given
    tile = (fixed["tile_x"], fixed["tile_y"], fixed["cells_per_thread"]) if fixed else s32.autotune(2)
    s32.step(args.warmup)
    s32.sync()
    stream = torch.cuda.ExternalStream(s32.stream(), device=dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(dev) if rank == 0 else None
    barrier(dist)
    torch.cuda.synchronize()
    if sampler:
        sampler.start()
    s32.profile_stages(True)
    e0.record(stream)
    s32.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    s32.sync()
    torch.cuda.synchronize()
    barrier(dist)
    clocks = sampler.stop() if sampler else None
    ms = e0.elapsed_time(e1)
    stage_ms, launches = s32.stage_stats()
    s32.profile_stages(False)
    ms_max = reduce_max(dist, ms, dev)
    value = world * dof * args.steps / (ms_max / 1e3)

    # roofline of the dominant kernel (the fused stage kernel: every launch in the region)
    peak, peak_kind = measured_hbm_peak()
    per_launch_bytes = BYTES_PER_DOF_UPDATE["fp32"] * dof / 2.0
    avg_launch_s = stage_ms / max(launches, 1) / 1e3
    achieved = per_launch_bytes / avg_launch_s / 1e9
    traffic = ncu_traffic(name)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": traffic.get("bytes_per_launch") if traffic else None,
                "kernel": "k_stage<float,2,P>", "algorithmic_bytes_per_launch": per_launch_bytes,
                "avg_launch_ms": avg_launch_s * 1e3}

    extra = {}
    if rank == 0 and not args.quick:
        # FP64 plain on the same grid
        w64 = wb.workload(name, wb.PREC_FP64, **size)
        s64 = wb.Solver(device=dev, **w64)
        s64.init_perturbation(ic)
        tile64 = s64.autotune(1)
        s64.step(1)
        s64.sync()
        st64 = torch.cuda.ExternalStream(s64.stream(), device=dev)
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(st64)
        s64.step(args.plain_steps)
        a1.record(st64)
        a1.synchronize()
        s64.sync()
        v64 = dof * args.plain_steps / (a0.elapsed_time(a1) / 1e3)
        # L1 of the FP32 form against the FP64 plain method, same fixed steps
        s64.init_perturbation(ic)
        s32b = wb.Solver(device=dev, **w32)
        s32b.init_perturbation(ic)
        sx, sy = s64.compute_max_speed()
        dx = 1.0 / w64["nx"]
        dt = w64["cfl"] / (2 * w64["order"] + 1) / (sx / dx + sy / dx)
        s64.step(args.check_steps, dt)
        s32b.step(args.check_steps, dt)
        l1, linf, _ = s32b.compute_error(s64)
        ref1, _, _ = s64.compute_error(None)
        s32b.close()
        s64.close()
        extra["fp64_plain"] = {"value": v64, "unit": UNIT, "steps": args.plain_steps,
                               "tile": list(tile64),
                               "speedup_fp32_over_fp64": value / world / v64}
        extra["accuracy"] = {"l1_fp32_vs_fp64": l1.tolist(), "linf_fp32_vs_fp64": linf.tolist(),
                             "l1_perturbation_fp64": ref1.tolist(), "steps": args.check_steps,
                             "dt": dt, "l1_bar": 1e-6, "pass": bool(np.all(l1 <= 1e-6))}

    # end to end through the C ABI: every step copies its whole input state from pinned
    # host memory and its whole (limited) result back
    e2e = None
    if not args.no_e2e:
        host_in = torch.empty(dof, dtype=torch.float32, pin_memory=True)
        host_out = torch.empty(dof, dtype=torch.float32, pin_memory=True)
        s32.download_f32_ptr(host_out.data_ptr())
        host_in.copy_(host_out)
        nE = args.e2e_steps
        # (a) synchronous calls: upload, step, download
        s32.upload_f32_ptr(host_in.data_ptr())  # one untimed round trip (first-use costs)
        s32.step(1)
        s32.download_f32_ptr(host_out.data_ptr())
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(nE):
            s32.upload_f32_ptr(host_in.data_ptr())
            s32.step(1)
            s32.download_f32_ptr(host_out.data_ptr())
        el_sync = reduce_max(dist, time.perf_counter() - t0, dev)
        # (b) pipelined host I/O: the upload of step k+1 and the download of step k-1
        #     overlap step k
        s32.step_io_f32_ptr(host_in.data_ptr(), host_out.data_ptr(), 1)  # untimed warm-up
        s32.sync()
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(nE):
            s32.step_io_f32_ptr(host_in.data_ptr(), host_out.data_ptr(), 1)
        s32.sync()
        el = reduce_max(dist, time.perf_counter() - t0, dev)
        e2e = {"value": world * dof * nE / el, "unit": UNIT, "h2d_bytes_per_step": dof * 4,
               "d2h_bytes_per_step": dof * 4, "steps": nE,
               "path": "wb_step_io_f32 per step (pipelined host I/O), pinned host",
               "sync_api": {"value": world * dof * nE / el_sync, "unit": UNIT,
                            "path": "wb_upload_state_f32 + wb_step + wb_download_state_f32"}}
    s32.close()

    # beside the headline, not part of it: the grid with the minmod limiter on; the
    # batched form (512 independent instances, CUDA graph of six steps) and its accuracy
    # against FP64 instances; the cfg3 accuracy study (FP32 form vs FP64 plain, 500 steps)
    if rank == 0 and not args.quick:
        extra["limited"] = limited_leg(wb, name, dev)
        extra["batch"] = batch_leg(wb, 512, dev)
        extra["batch"]["accuracy"] = batch_accuracy(wb, 512, dev)
        if args.accuracy_steps > 0:
            extra["accuracy_cfg3"] = accuracy_cfg3(wb, args.accuracy_steps, dev)

    cpu = None
    if rank == 0 and not args.quick:
        v, cores, desc = cpu_sample(wb, seconds=args.cpu_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
        # the reference is serial: the same port on one core, on a smaller sample
        v1, _, desc1 = cpu_sample(wb, seconds=args.cpu_seconds, n=128, threads=1)
        cpu["one_core"] = {"value": v1, "unit": UNIT, "cores": 1, "kind": "port",
                           "sample": desc1}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 16-mode velocity field on the isothermal atmosphere)",
            "config": {"workload": "cfg5: %d^2 P2 isothermal Phi=0.1y, 16-mode velocity field, "
                                   "FP32-perturbation, SSP-RK2, CFL 0.3" % w32["nx"],
                       "nx": w32["nx"], "ny": w32["ny"], "order": 2, "basis": "P",
                       "dofs": dof, "tile": list(tile),
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2_policy": "inputs larger than L2 (6.4 GB state per buffer)"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clocks,
        }
        line.update(extra)
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def accuracy_cfg3(wb, n, dev=0):
    """The accuracy configuration (cfg3): 2048^2 P2 polytrope K = 1, Phi = y, seeded Gaussian
    pressure bump (sigma 0.05) of amplitude 1e-1, 1e-3 and 1e-6; the FP32 perturbation form
    against the FP64 plain method over the same n fixed time steps (dt from the initial CFL
    speed of the FP64 run): L1 / Linf per conserved variable of the difference (unit-area
    domain, so L1 is a mean absolute error) and of the perturbation."""
    results = []
    for amp in (1e-1, 1e-3, 1e-6):
        w64 = wb.workload("cfg3", wb.PREC_FP64, device=dev)
        w32 = wb.workload("cfg3", wb.PREC_FP32, device=dev)
        ic = wb.workload_ic("cfg3", amp)
        with wb.Solver(**w64) as s64, wb.Solver(**w32) as s32:
            s64.init_perturbation(ic)
            s32.init_perturbation(ic)
            sx, sy = s64.compute_max_speed()
            dx, dy = w64["lx"] / w64["nx"], w64["ly"] / w64["ny"]
            dt = w64["cfl"] / (2 * w64["order"] + 1) / (sx / dx + sy / dy)
            t0 = time.perf_counter()
            s64.step(n, dt)
            s32.step(n, dt)
            s64.sync()
            s32.sync()
            el = time.perf_counter() - t0
            l1, linf, _ = s32.compute_error(s64)
            p1, pinf, _ = s64.compute_error(None)
        results.append({"amplitude": amp, "l1_fp32_vs_fp64": l1.tolist(),
                        "linf_fp32_vs_fp64": linf.tolist(), "l1_perturbation": p1.tolist(),
                        "linf_perturbation": pinf.tolist(), "dt": dt, "seconds": el,
                        "pass": bool(np.all(l1 <= 1e-6))})
    return {"workload": "cfg3: 2048^2 P2 polytrope K=1, Phi=y, Gaussian pressure bump "
                        "(sigma 0.05, seed 3), FP32 perturbation vs FP64 plain, fixed dt",
            "steps": n, "l1_bar": 1e-6, "pass": all(r["pass"] for r in results),
            "results": results}


def run_accuracy(args):
    """The cfg3 accuracy study alone (one JSON line)."""
    import torch
    wb = load_package()
    wb.lib()
    torch.cuda.set_device(0)
    line = {"mode": "accuracy"}
    line.update(accuracy_cfg3(wb, args.accuracy_steps))
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg5")
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--check-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-n", type=int, default=512)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--nx", type=int, default=0,
                    help="cells per side instead of the workload's (small cases for profiling)")
    ap.add_argument("--tile", default="",
                    help="fixed stage tile TXxTY[/cells per thread] (default: autotune)")
    ap.add_argument("--quick", action="store_true", help="skip FP64, accuracy and CPU legs")
    ap.add_argument("--accuracy", action="store_true",
                    help="run the cfg3 accuracy study instead of the benchmark")
    ap.add_argument("--accuracy-steps", type=int, default=500)
    ap.add_argument("--batch", type=int, default=0,
                    help="run only the batched form with this many instances (profiling)")
    ap.add_argument("--batch-grid", action="store_true",
                    help="with --batch 1: the one instance is the workload's grid (at --nx)")
    ap.add_argument("--batch-tiles", default="",
                    help="with --batch: pin tiles per degree, e.g. 0:32x16/2,1:32x16/2,2:32x8/1")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.accuracy:
        return run_accuracy(args)
    if args.batch > 0:
        return run_batch_only(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
