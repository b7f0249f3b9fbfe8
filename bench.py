#!/usr/bin/env python3
"""Benchmark of the cell-update hot path (one JSON line on stdout).

Workload (default): Jacobi-7 heat diffusion on a 512^3 grid of FP64 cells,
constant zero boundary, U[0,1) initial values (seeded SplitMix64) - the
grid the Jacobi3D GLUPS target is quoted on.  A "step" is one time step of
the whole grid (134,217,728 lattice-site updates).  The grid (1 GiB per
buffer) is larger than L2, so consecutive steps read from HBM.

  value  GLUPS with the grid resident in HBM, timed with CUDA events on the
         library's stream over exactly --steps launches.
  e2e    GLUPS through the C ABI with host buffers: upload from pinned host
         memory, 100 time steps (the run length of the configuration), and
         download of the result, per e2e step.

--impl reference times the reference's CPU algorithm on this machine's host
cores instead: the C restatement in oracle/ (the reference itself cannot be
built here), OpenMP over all cores, on whole time steps of the same grid.

Under torchrun (--gpus N > 1) every rank advances its own replica (the
workload is replicated, not sharded: weak scaling with no collective on the
data path); rank 0 prints the line with the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOADS = {
    # name: (cell, shape, periodic, steps per e2e run, bytes per LUP)
    "jacobi7_f64_512": ("fix", (512, 512, 512), 0, 100, 16),
    "jacobi7_f64_ieee_512": ("ieee", (512, 512, 512), 0, 100, 16),
    "gol_u8_8192": ("gol", (8192, 8192), 3, 1000, 2),
}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(kernel_key: str):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary (profiles/ncu_traffic.txt: lines 'key bytes_per_launch')."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 2 and parts[0] == kernel_key:
                    return float(parts[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100", "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax.append(float(p[2]))
                except ValueError:
                    continue
                for n, v in zip(names, p[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_gpu(args, world, rank, local, dist):
    import torch
    torch.cuda.set_device(local)
    from libgeodecomp_gb300 import lgd, workloads

    kind, shape, periodic, run_steps, bpl = WORKLOADS[args.workload]
    cell = {"fix": lgd.CELL_JACOBI7_F64_FIX, "ieee": lgd.CELL_JACOBI7_F64, "gol": lgd.CELL_GOL_U8}[kind]
    cells = int(np.prod(shape))
    g = lgd.Grid(cell, shape, periodic=periodic)
    if kind == "gol":
        g.fill_bernoulli(0.3, seed=42, stream=workloads.STREAM_GRID)
    else:
        g.fill_uniform(0, seed=42, stream=workloads.STREAM_GRID)
    stream_ptr = lgd.ctypes.c_void_p()
    lgd.check(lgd.lib().lgd_gpu_stream(g._h, lgd.ctypes.byref(stream_ptr)))
    stream = torch.cuda.ExternalStream(stream_ptr.value)

    for _ in range(args.warmup):
        g.step(1)
    g.synchronize()
    launches0 = g.launch_count()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    barrier(dist)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record(stream)
        for _ in range(args.steps):
            g.step(1)
        end.record(stream)
        end.synchronize()
    torch.cuda.synchronize()
    barrier(dist)
    ms = start.elapsed_time(end)
    launches = g.launch_count() - launches0
    ms = max_over_ranks(dist, ms)
    clocks = clk.summary()
    ms_per_step = ms / args.steps
    glups = cells * args.steps * world / (ms * 1e-3) / 1e9

    # roofline of the dominant kernel (one launch per step)
    peak, peak_kind = load_peaks()
    achieved = cells * bpl / (ms_per_step * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": cells * bpl,
                "traffic": profile_traffic(args.workload)}

    # end to end through the C ABI: pinned host in, run_steps steps, host out
    e2e = None
    if not args.no_e2e:
        host_dtype = np.uint8 if kind == "gol" else np.float64
        hin = torch.empty(cells * np.dtype(host_dtype).itemsize, dtype=torch.uint8, pin_memory=True).numpy()
        hout = torch.empty(cells * np.dtype(host_dtype).itemsize, dtype=torch.uint8, pin_memory=True).numpy()
        hin_v = hin.view(host_dtype).reshape(shape)
        hout_v = hout.view(host_dtype).reshape(shape)
        g.download(0, out=hin_v)
        e2e_runs = max(1, args.e2e_runs)
        # warm-up run
        g.upload(0, hin_v)
        g.step(run_steps)
        g.download(0, out=hout_v)
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(e2e_runs):
            g.upload(0, hin_v)
            g.step(run_steps)
            g.download(0, out=hout_v)
        t1 = time.perf_counter()
        barrier(dist)
        e2e_s = max_over_ranks(dist, t1 - t0)
        e2e = {"value": round(cells * run_steps * e2e_runs * world / e2e_s / 1e9, 3), "unit": "GLUPS",
               "h2d_bytes_per_step": cells * np.dtype(host_dtype).itemsize,
               "d2h_bytes_per_step": cells * np.dtype(host_dtype).itemsize,
               "step": "upload + %d time steps + download via the C ABI" % run_steps,
               "ms_per_step": round(e2e_s * 1e3 / e2e_runs, 3)}

    extra = {}
    if args.workload == "jacobi7_f64_512" and not args.no_ieee:
        # the bit-exact IEEE FP64 kernel on the same grid, for comparison
        gi = lgd.Grid(lgd.CELL_JACOBI7_F64, shape, periodic=periodic)
        gi.fill_uniform(0, seed=42, stream=workloads.STREAM_GRID)
        sp = lgd.ctypes.c_void_p()
        lgd.check(lgd.lib().lgd_gpu_stream(gi._h, lgd.ctypes.byref(sp)))
        st = torch.cuda.ExternalStream(sp.value)
        for _ in range(3):
            gi.step(1)
        gi.synchronize()
        k = max(3, args.steps // 4)
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(st)
        for _ in range(k):
            gi.step(1)
        s1.record(st)
        s1.synchronize()
        ims = s0.elapsed_time(s1) / k
        extra["ieee_fp64_kernel"] = {"glups": round(cells / (ims * 1e-3) / 1e9, 2), "ms_per_step": round(ims, 4),
                                     "hbm_frac": round(cells * 16 / (ims * 1e-3) / 1e9 / peak, 4),
                                     "note": "bit-identical to the reference; bound by the FP64 pipe"}
        gi.close()
    g.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.workload, budget_s=args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": "Jacobi3D GLUPS & HBM GB/s vs 8 TB/s" if kind != "gol" else "Game of Life GLUPS",
            "value": round(glups, 3), "unit": "GLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fix": "f64 (64-bit fixed-point arithmetic)", "ieee": "f64", "gol": "u8"}[kind],
            "data": "synthetic (seeded SplitMix64 U[0,1), generated on device)",
            "config": {"workload": args.workload, "grid": list(shape), "boundary": "constant 0" if periodic == 0 else "torus",
                       "cells": cells, "l2": "grid (%d MiB per buffer) larger than L2" % (cells * bpl // 2 >> 20),
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "gpu_launches": launches, "roofline": roofline, "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def cpu_baseline(workload: str, budget_s: float = 15.0):
    """The oracle (C restatement of the reference algorithm) on all host
    cores, timed on whole time steps of the same grid until about budget_s
    seconds of work."""
    import oracle
    from libgeodecomp_gb300 import workloads
    kind, shape, periodic, _, _ = WORKLOADS[workload]
    threads = oracle.max_threads()
    cells = int(np.prod(shape))
    if kind == "gol":
        u = workloads.gol_initial(shape[1], shape[0], seed=42)
        fn = lambda a, s: oracle.gol(a, s)  # noqa: E731
    else:
        u = workloads.jacobi_initial(shape[2], shape[1], shape[0], seed=42)
        fn = lambda a, s: oracle.jacobi7(a, s)  # noqa: E731
    fn(u, 1)
    t0 = time.perf_counter()
    fn(u, 1)
    one = time.perf_counter() - t0
    steps = max(1, int(budget_s / max(one, 1e-6)))
    t0 = time.perf_counter()
    fn(u, steps)
    dt = time.perf_counter() - t0
    return {"value": round(cells * steps / dt / 1e9, 4), "unit": "GLUPS", "cores": threads, "kind": "port",
            "sample": "%d time steps of the %s grid (%.1f s)" % (steps, "x".join(map(str, shape)), dt)}


def run_reference(args, world, rank):
    if rank != 0:
        return
    from libgeodecomp_gb300 import workloads  # noqa: F401
    import oracle
    kind, shape, periodic, _, _ = WORKLOADS[args.workload]
    cells = int(np.prod(shape))
    if kind == "gol":
        u = workloads.gol_initial(shape[1], shape[0], seed=42)
        fn = lambda a, s: oracle.gol(a, s)  # noqa: E731
    else:
        u = workloads.jacobi_initial(shape[2], shape[1], shape[0], seed=42)
        fn = lambda a, s: oracle.jacobi7(a, s)  # noqa: E731
    for _ in range(args.warmup):
        u = fn(u, 1)
    t0 = time.perf_counter()
    u = fn(u, args.steps)
    dt = time.perf_counter() - t0
    glups = cells * args.steps / dt / 1e9
    threads = oracle.max_threads()
    line = {
        "metric": "Jacobi3D GLUPS & HBM GB/s vs 8 TB/s" if kind != "gol" else "Game of Life GLUPS",
        "value": round(glups, 4), "unit": "GLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3 / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if kind != "gol" else "u8", "data": "synthetic (seeded SplitMix64)",
        "config": {"workload": args.workload, "grid": list(shape), "cells": cells},
        "impl": "reference",
        "cpu_baseline": {"value": round(glups, 4), "unit": "GLUPS", "cores": threads, "kind": "port",
                         "sample": "%d whole time steps of the %s grid" % (args.steps, "x".join(map(str, shape)))},
        "e2e": {"value": round(glups, 4), "unit": "GLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="jacobi7_f64_512")
    ap.add_argument("--e2e-runs", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-ieee", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    world, rank, local, dist = dist_setup(args.gpus)
    run_gpu(args, world, rank, local, dist)


if __name__ == "__main__":
    main()
