#!/usr/bin/env python3
"""Benchmark of the cell-update hot path (one JSON line on stdout).

Default workload: Jacobi-7 heat diffusion on a 512^3 grid of FP64 cells,
constant zero boundary, U[0,1) initial values (seeded SplitMix64) - the
grid the Jacobi3D GLUPS target is quoted on.  A "step" is one time step of
the whole grid (134,217,728 lattice-site updates); the library fuses two
steps into one pass over memory by default (one kernel launch per pass).
The grid (1 GiB per buffer) is larger than L2, so every pass streams from
HBM.

  value     GLUPS with the grid resident in HBM, timed with CUDA events on
            the library's stream over exactly --steps time steps.
  roofline  per launch: achieved = the launch's algorithmic bytes (16 B
            per lattice-site update for FP64 Jacobi: one read and one write
            of every cell and time step, times the updates the launch
            performs) / the launch's average time, frac = achieved / the
            measured HBM copy bandwidth, traffic = DRAM bytes per launch
            from the committed ncu summaries.  Where a launch fuses several
            steps (temporal blocking) achieved can exceed the copy
            bandwidth; per_pass_gbs and frac_per_pass count one read and
            one write per cell and launch, which is what HBM sees.
  e2e       the same metric through the C ABI with host buffers: upload
            from pinned host memory, the configuration's run length of time
            steps, download of the result - per e2e step.
  secondary the other configurations, each measured the same way (value,
            roofline with traffic, e2e where the data fits a host round
            trip, the oracle on the host cores as cpu_baseline, clocks):
            Game of Life 8192^2, SELL-C-sigma diffusion on 4,194,304 nodes,
            the 512-cavity D3Q19 ensemble, variable-coefficient diffusion
            256^3 and Jacobi-7 512^3 in FP32.  --no-secondary skips them.

Other workloads as the headline (--workload): gol_u8_8192, sell_f64_4m,
jacobi7_f64_ieee_512 (the bit-exact IEEE FP64 kernel alone),
jacobi7_f32_512, lbm_d3q19_ensemble_512, varcoef_f32_256; --surrogate runs
the learned-surrogate time-to-solution benchmark.

--impl reference times the reference's CPU algorithm on this machine's host
cores: the C restatement in oracle/ (the reference's own sources are not on
this machine), OpenMP over all cores, on whole time steps of the same input,
with the same config block as the GPU arm.

Under torchrun (--gpus N > 1) the structured workloads are decomposed into
slabs, one per rank (weak scaling: every rank owns a 512^3 slab of a
512 x 512 x 512N grid, Game of Life 8192^2 cells of a y-cut torus), with a
ghost-zone exchange of R*T planes every T steps (libgeodecomp_gb300.slabs);
SELL-C-sigma runs its 4,194,304 nodes over row blocks with an all-gather
per step (strong scaling, libgeodecomp_gb300.sell_shards), the ensemble
one 512-cavity ensemble per rank; rank 0 prints the line with the max time
over ranks.
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

JACOBI_METRIC = "Jacobi3D GLUPS & HBM GB/s vs 8 TB/s"
METRICS = {"gol_u8_8192": "Game of Life GLUPS", "sell_f64_4m": "SELL-C-sigma diffusion GB/s and s/step",
           "lbm_d3q19_ensemble_512": "D3Q19 ensemble GLUPS (persistent launches, autotuned steps per launch)",
           "varcoef_f32_256": "variable-coefficient diffusion GLUPS"}
DTYPES = {"gol_u8_8192": "u8", "lbm_d3q19_ensemble_512": "f32", "varcoef_f32_256": "f32", "jacobi7_f32_512": "f32",
          "sell_f64_4m": "f64", "jacobi7_f64_ieee_512": "f64",
          "jacobi7_f64_512": "f64 (values on the device in 64-bit fixed point, integer arithmetic)"}
WORKLOAD_NAMES = ["jacobi7_f64_512", "jacobi7_f64_ieee_512", "jacobi7_f32_512", "gol_u8_8192", "sell_f64_4m",
                  "lbm_d3q19_ensemble_512", "varcoef_f32_256"]
# secondary configurations of the default run: (workload, timed steps, warm-up steps, e2e)
SECONDARY = [("gol_u8_8192", 1000, 32, True), ("sell_f64_4m", 200, 10, True),
             ("varcoef_f32_256", 1024, 8, True), ("jacobi7_f32_512", 102, 6, True),
             ("lbm_d3q19_ensemble_512", 10, 2, False)]


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(key: str):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary (profiles/ncu_traffic.txt, lines 'workload bytes_per_launch')."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.txt")) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 2 and parts[0] == key:
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
            time.sleep(0.3)
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


# ------------------------------------------------------ workload configs
def workload_config(name: str, args, world: int = 1) -> dict:
    """The configuration block of a workload: what runs, on which input.

    Both arms (the GPU library and the reference's CPU algorithm) print
    this same block, so their lines describe the same workload."""
    size = getattr(args, "size", 512)
    if name.startswith("jacobi7"):
        f32 = name.startswith("jacobi7_f32")
        ieee = "ieee" in name
        cfg = {"workload": name if size == 512 else name.replace("512", str(size)),
               "grid": [size, size, size], "boundary": "constant 0", "cells": size ** 3,
               "initial": "U[0,1) seed 42", "cell_update": "(c+n+s+e+w+t+b)*(1/7)",
               "cell": "FP32" if f32 else "FP64 IEEE" if ieee else "FP64, 64-bit fixed point on the device",
               "l2": "inputs larger than L2 (%d MiB per buffer)" % (size ** 3 * (4 if f32 else 8) >> 20)}
        if not ieee:
            tb = getattr(args, "time_block", 0)
            cfg["time_block"] = ("library default (%d steps per pass)" % (3 if f32 else 2)) if tb == 0 else tb
    elif name == "gol_u8_8192":
        cfg = {"workload": name, "grid": [8192, 8192], "boundary": "torus", "cells": 8192 * 8192,
               "initial": "Bernoulli(0.3) seed 42", "run_steps": 1000,
               "generations_per_pass": "library default (16, bit-sliced)",
               "l2": "both buffers (128 MiB) about L2-sized; no flush between steps"}
    elif name == "sell_f64_4m":
        cfg = {"workload": name, "nodes": 4194304, "C": 32, "sigma": 256, "degree": "power law alpha=2 on [4,64]",
               "weights": "U[0,1) row-normalised to 0.9", "update": "x' = 0.1 x + W x", "run_steps": 200,
               "l2": "matrix (547 MiB) larger than L2; x (32 MiB) L2-resident"}
    elif name == "varcoef_f32_256":
        cfg = {"workload": name, "grid": [256, 256, 256], "boundary": "torus", "cells": 256 ** 3,
               "kappa": "GRF length 16 mapped to [0.02, 0.15]", "initial": "GRF length 16 on [0, 1]",
               "run_steps": 4096, "l2": "u, k and u' (192 MiB) larger than L2; no flush between steps"}
    elif name == "lbm_d3q19_ensemble_512":
        n = getattr(args, "lbm_instances", 512)
        cfg = {"workload": name, "instances": n, "edges": "uniform {32..%d}" % getattr(args, "lbm_edge_max", 192),
               "omega": "uniform [1.0, 1.9)", "lid": 0.05, "precision": "FP32", "run_steps": 500,
               "l2": "populations far larger than L2"}
    else:
        raise ValueError(name)
    if world > 1:
        if name == "gol_u8_8192":
            cfg["parallelism"] = "y-slabs of 8192^2 cells, %d ranks" % world
        elif slab_capable(name):
            cfg["parallelism"] = "z-slabs, %d ranks" % world
        elif name == "sell_f64_4m":
            cfg["parallelism"] = "row blocks of whole chunks, an all-gather of the node values per step, %d ranks" % world
        elif name == "lbm_d3q19_ensemble_512":
            cfg["parallelism"] = "%d independent ensembles of %d cavities (seed 42 + rank), %d ranks" % (
                world, getattr(args, "lbm_instances", 512), world)
        else:
            cfg["parallelism"] = "replicas, %d ranks" % world
    else:
        cfg["parallelism"] = "single GPU"
    return cfg


def slab_capable(name: str) -> bool:
    return name.startswith("jacobi7") or name in ("varcoef_f32_256", "gol_u8_8192")


# ---------------------------------------------------------------- workloads
class JacobiWorkload:
    run_steps = 100
    bytes_per_unit = 16          # one FP64 read + one FP64 write per cell and step

    def __init__(self, ieee: bool, edge: int = 512, f32: bool = False):
        from libgeodecomp_gb300 import lgd, workloads
        self.shape = (edge, edge, edge)
        self.lgd = lgd
        self.ieee = ieee
        self.f32 = f32
        self.name = ("jacobi7_f32_%d" if f32 else "jacobi7_f64_ieee_%d" if ieee else "jacobi7_f64_%d") % edge
        self.metric = JACOBI_METRIC
        self.unit = "GLUPS"
        self.units = int(np.prod(self.shape))
        if f32:
            self.bytes_per_unit = 8
        cell = lgd.CELL_JACOBI7_F32 if f32 else lgd.CELL_JACOBI7_F64 if ieee else lgd.CELL_JACOBI7_F64_FIX
        self.g = lgd.Grid(cell, self.shape, periodic=0)
        self.g.fill_uniform(0, seed=42, stream=workloads.STREAM_GRID)
        self.time_block = 0
        self.setup = {}

    def stream(self):
        p = self.lgd.ctypes.c_void_p()
        self.lgd.check(self.lgd.lib().lgd_gpu_stream(self.g._h, self.lgd.ctypes.byref(p)))
        return p.value

    def step(self, n=1):
        self.g.step(n)

    def set_time_block(self, depth, shape=0):
        """Steps fused per pass (0 = the library's default for the cell)."""
        self.g.set_time_block(depth)
        self.g.set_time_block_shape(shape)
        self.time_block = depth

    def traffic_key(self):
        """Key of the committed ncu traffic line: the workload, plus _tb<d>
        when d > 1 steps are fused per pass (the library's default depth is
        3 for the FP32 cell, 2 for the fixed-point cell)."""
        if self.ieee:
            return self.name
        depth = self.time_block or (3 if self.f32 else 2)
        depth = depth if self.f32 else min(depth, 2)
        return self.name if depth <= 1 else "%s_tb%d" % (self.name, depth)

    def sync(self):
        self.g.synchronize()

    def launches(self):
        return self.g.launch_count()

    def host_buffers(self, torch):
        dt = np.float32 if self.f32 else np.float64
        nbytes = self.units * np.dtype(dt).itemsize
        hin = pinned(torch, nbytes).view(dt).reshape(self.shape)
        hout = pinned(torch, nbytes).view(dt).reshape(self.shape)
        self.g.download(0, out=hin)
        return hin, hout

    def e2e_run(self, hin, hout):
        self.g.upload(0, hin)
        self.g.step(self.run_steps)
        self.g.download(0, out=hout)
        return hin.nbytes, hout.nbytes

    def close(self):
        self.g.close()


class GoLWorkload:
    shape = (8192, 8192)
    run_steps = 1000
    bytes_per_unit = 2

    def __init__(self):
        from libgeodecomp_gb300 import lgd, workloads
        self.lgd = lgd
        self.name = "gol_u8_8192"
        self.metric = METRICS[self.name]
        self.unit = "GLUPS"
        self.units = int(np.prod(self.shape))
        self.g = lgd.Grid(lgd.CELL_GOL_U8, self.shape, periodic=3)
        self.g.fill_bernoulli(0.3, seed=42, stream=workloads.STREAM_GRID)
        self.setup = {}

    stream = JacobiWorkload.stream
    step = JacobiWorkload.step
    sync = JacobiWorkload.sync
    launches = JacobiWorkload.launches
    e2e_run = JacobiWorkload.e2e_run
    close = JacobiWorkload.close

    def traffic_key(self):
        return self.name

    def set_time_block(self, depth, shape=0):
        """Generations fused per pass (0 = the library's default, 16)."""
        self.g.set_time_block(depth)
        self.g.set_time_block_shape(shape)

    def host_buffers(self, torch):
        hin = pinned(torch, self.units).reshape(self.shape)
        hout = pinned(torch, self.units).reshape(self.shape)
        self.g.download(0, out=hin)
        return hin, hout


class SellWorkload:
    n = 4194304
    run_steps = 200

    def __init__(self):
        from libgeodecomp_gb300 import lgd, workloads
        self.lgd = lgd
        self.name = "sell_f64_4m"
        self.metric = METRICS[self.name]
        self.unit = "GLUPS"
        rp, col, w = workloads.powerlaw_graph(self.n, seed=42)
        self.nnz = int(col.size)
        # the matrix is built twice, by the host builder and on the GPU
        # (identical arrays); the timed grid is the GPU-built one
        t0 = time.perf_counter()
        self.s = lgd.sell_build(self.n, rp, col, w, 32, 256)
        host_build = time.perf_counter() - t0
        lgd.SellGrid.from_csr(4096, rp[:4097] - rp[0], col[:int(rp[4096])] % 4096, w[:int(rp[4096])], 32, 256).close()
        t0 = time.perf_counter()
        self.g = lgd.SellGrid.from_csr(self.n, rp, col, w, 32, 256)
        gpu_build = time.perf_counter() - t0
        self.x0 = workloads.sell_values(self.n, seed=42)
        self.g.upload(self.x0)
        self.units = self.n
        n_chunks = (self.n - 1) // 32 + 1
        # 12 B per stored entry (8 value + 4 column), 16 B per row (x own read
        # + x' write) + 4 B row length, 4 B per chunk offset
        self.bytes_per_step = 12 * self.nnz + 20 * self.n + 4 * n_chunks
        self.bytes_per_unit = self.bytes_per_step / self.n
        self.setup = {"nnz": self.nnz, "slots": int(self.s["values"].size),
                      "build_s": {"host_builder": round(host_build, 3),
                                  "gpu_builder_from_host_csr": round(gpu_build, 4)}}

    def traffic_key(self):
        return self.name

    def stream(self):
        return self.g.stream()

    def step(self, n=1):
        self.g.step(n)

    def sync(self):
        self.g.synchronize()

    def launches(self):
        return self.g.launch_count()

    def host_buffers(self, torch):
        hin = pinned(torch, self.n * 8).view(np.float64)
        hout = pinned(torch, self.n * 8).view(np.float64)
        hin[:] = self.x0
        return hin, hout

    def e2e_run(self, hin, hout):
        self.g.upload(hin)
        self.g.step(self.run_steps)
        self.g.download(out=hout)
        return hin.nbytes, hout.nbytes

    def close(self):
        self.g.close()


class VarcoefWorkload:
    """Variable-coefficient diffusion u' = u + sum_f 0.5 (k_c + k_n)(u_n - u_c)
    on a 256^3 FP32 torus: u0 a Gaussian random field on [0, 1], k a
    separate one on [0.02, 0.15] (length 16) - the plain stencil the learned
    surrogate is measured against, to t = 4096."""
    run_steps = 4096
    bytes_per_unit = 12      # u read, k read, u written (FP32)

    def __init__(self, edge: int = 256):
        from libgeodecomp_gb300 import lgd, workloads
        self.lgd = lgd
        self.shape = (edge, edge, edge)
        self.name = "varcoef_f32_%d" % edge
        self.metric = METRICS["varcoef_f32_256"]
        self.unit = "GLUPS"
        self.units = int(np.prod(self.shape))
        self.u0, kappa = workloads.varcoef_fields(edge, seed=42, length=16.0)
        self.g = lgd.Grid(lgd.CELL_VARCOEF_F32, self.shape, periodic=7)
        self.g.upload(0, self.u0)
        self.g.upload(1, kappa)
        self.setup = {}

    stream = JacobiWorkload.stream
    step = JacobiWorkload.step
    sync = JacobiWorkload.sync
    launches = JacobiWorkload.launches
    close = JacobiWorkload.close

    def traffic_key(self):
        return self.name

    def host_buffers(self, torch):
        hin = pinned(torch, self.units * 4).view(np.float32)
        hout = pinned(torch, self.units * 4).view(np.float32)
        hin[:] = self.u0.reshape(-1)
        return hin.reshape(self.shape), hout.reshape(self.shape)

    def e2e_run(self, hin, hout):
        self.g.upload(0, hin)
        self.g.step(self.run_steps)
        self.g.download(0, out=hout)
        return hin.nbytes, hout.nbytes


class LbmWorkload:
    """512 D3Q19 lid-driven cavities, edges uniform in {32..192}, omega
    uniform in [1.0, 1.9), lid 0.05, FP32; one persistent launch per step or
    one two-step launch per pair of steps, launch shape and steps per launch
    from the library's pattern-search tuner."""
    run_steps = 500
    bytes_per_unit = 152     # 19 FP32 reads + 19 FP32 writes per cell

    def __init__(self, instances=512, edge_max=192, tune=True, time_block=None, seed=42):
        from libgeodecomp_gb300 import lgd, workloads
        self.lgd = lgd
        self.name = "lbm_d3q19_ensemble_512"
        self.metric = METRICS[self.name]
        self.unit = "GLUPS"
        # the configuration is 512 instances with edges up to 192; smaller
        # ensembles serve profiling captures
        edges, omegas = workloads.lbm_ensemble(instances, seed=seed, edge_max=edge_max)
        self.e = lgd.LbmEnsemble(edges, omegas, lid=0.05, precision=4)
        self.units, self.items = self.e.info()
        t0 = time.perf_counter()
        if tune:
            (ty, th, ct), best = self.e.tune(trial_steps=2)
            self.e.reset()
        else:
            ty, th, ct = self.e.config()
        if time_block:
            self.e.set_time_block(*time_block)
        depth, shape, ctas = self.e.time_block()
        self.depth = depth
        self.setup = {"cells": self.units, "work_items": self.items, "tune_s": round(time.perf_counter() - t0, 2),
                      "tuned_launch": {"tile_rows": ty, "threads": th, "ctas_per_sm": ct},
                      "tuned_time_block": {"steps_per_launch": depth, "tile": ["32x8", "32x4"][shape],
                                           "ctas_per_sm": ctas}}

    def traffic_key(self):
        return self.name + ("_tb2" if self.depth == 2 else "")

    def stream(self):
        return self.e.stream()

    def step(self, n=1):
        self.e.step(n)

    def sync(self):
        self.e.synchronize()

    def launches(self):
        return self.e.launch_count()

    def looped_ms(self, torch, steps):
        st = torch.cuda.ExternalStream(self.e.stream())
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st)
        self.e.step_looped(steps)
        b.record(st)
        b.synchronize()
        return a.elapsed_time(b) / steps

    def close(self):
        self.e.close()


def make_workload(name, args):
    if name == "lbm_d3q19_ensemble_512":
        tb = tuple(int(v) for v in args.lbm_time_block.split(",")) if args.lbm_time_block else None
        # several GPUs: the ensemble's instances are independent, so every
        # rank advances its own 512 cavities (seed 42 + rank), no collective
        return LbmWorkload(instances=args.lbm_instances, edge_max=args.lbm_edge_max, tune=not args.lbm_no_tune,
                           time_block=tb, seed=42 + getattr(args, "rank", 0))
    if name == "jacobi7_f64_512":
        return JacobiWorkload(ieee=False, edge=args.size)
    if name == "jacobi7_f64_ieee_512":
        return JacobiWorkload(ieee=True, edge=args.size)
    if name == "jacobi7_f32_512":
        return JacobiWorkload(ieee=False, edge=args.size, f32=True)
    if name == "gol_u8_8192":
        return GoLWorkload()
    if name == "sell_f64_4m":
        return SellWorkload()
    if name == "varcoef_f32_256":
        return VarcoefWorkload(256)
    raise ValueError(name)


# ------------------------------------------------------------------ helpers
def dist_setup(backend: str = "gloo"):
    """torch.distributed from torchrun's environment: NCCL where ranks
    exchange device data (the slab decomposition), gloo otherwise."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def time_steps(torch, w, steps):
    """CUDA-event time (ms) of `steps` time steps issued as one call, on the
    library's stream: the library may fuse several steps into one pass
    (temporal blocking), exactly as a user's lgd_gpu_step(h, 0, steps)."""
    stream = torch.cuda.ExternalStream(w.stream())
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    w.step(steps)
    end.record(stream)
    end.synchronize()
    return start.elapsed_time(end)


def roofline_of(w, ms, steps, launches, peak, peak_kind):
    """Per launch, with the algorithmic bytes of a lattice-site update
    (bytes_per_unit: one read and one write of every cell and step) times
    the updates one launch performs: a launch that advances k time steps
    (temporal blocking) performs k updates per cell.  frac above 1 is what
    fusing steps buys: the pass moves each cell once for k updates, so the
    per-pass figures (one read and one write per cell and launch, what HBM
    actually sees) are reported beside it."""
    launch_ms = ms / max(1, launches)
    steps_per_launch = steps / max(1, launches)
    pass_bytes = w.units * w.bytes_per_unit
    algo_bytes = pass_bytes * steps_per_launch
    achieved = algo_bytes / (launch_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4),
                "peak_source": (peak_kind + " (MEASURED_PEAKS.json hbm_gbs)") if peak_kind == "measured"
                else "fallback 6800 GB/s",
                "algorithmic_bytes_per_launch": int(algo_bytes), "launch_ms": round(launch_ms, 4),
                "steps_per_launch": round(steps_per_launch, 3), "traffic": profile_traffic(w.traffic_key())}
    if launches and launches < steps:
        per_pass = pass_bytes / (launch_ms * 1e-3) / 1e9
        roofline["per_pass_gbs"] = round(per_pass, 1)
        roofline["frac_per_pass"] = round(per_pass / peak, 4)
        roofline["per_pass_bytes"] = int(pass_bytes)
        roofline["note"] = ("temporal blocking: %.3g time steps per launch; achieved counts the bytes of every "
                            "update, per_pass_gbs what HBM moves" % steps_per_launch)
    return roofline


_PLACEMENT = None


def host_placement(torch, sysfs: str = "/sys"):
    """The NUMA nodes this process may run on and the GPU's node (from the
    PCI function's sysfs entry; None where the system does not say).  Where
    there is more than one node, pinned buffers are allocated from a thread
    bound to the CPUs of the GPU's node, so that their pages sit next to the
    GPU's host link."""
    global _PLACEMENT
    if _PLACEMENT is None:
        allowed = os.sched_getaffinity(0)
        nodes = {}
        base = os.path.join(sysfs, "devices", "system", "node")
        for name in (os.listdir(base) if os.path.isdir(base) else []):
            if not (name.startswith("node") and name[4:].isdigit()):
                continue
            try:
                with open(os.path.join(base, name, "cpulist")) as f:
                    text = f.read().strip()
            except OSError:
                continue
            cpus = set()
            for part in filter(None, text.split(",")):
                a, _, b = part.partition("-")
                cpus.update(range(int(a), int(b or a) + 1))
            if cpus & allowed:
                nodes[int(name[4:])] = sorted(cpus & allowed)
        gpu = None
        try:
            p = torch.cuda.get_device_properties(torch.cuda.current_device())
            with open(os.path.join(sysfs, "bus", "pci", "devices", "%04x:%02x:%02x.0" % (
                    p.pci_domain_id, p.pci_bus_id, p.pci_device_id), "numa_node")) as f:
                gpu = int(f.read().strip())
        except Exception:           # no device properties or no sysfs entry: unknown
            gpu = None
        cpus = nodes.get(gpu) if gpu is not None and len(nodes) > 1 else None
        _PLACEMENT = {"numa_nodes": len(nodes), "gpu_node": gpu, "bound_to_gpu_node": cpus is not None,
                      "cpus": cpus}
    return _PLACEMENT


def pinned(torch, nbytes):
    """Page-locked host memory of nbytes (a numpy uint8 array that keeps the
    torch tensor alive), placed as host_placement says."""
    cpus = host_placement(torch)["cpus"]
    old = os.sched_getaffinity(0) if cpus else None
    if cpus:
        os.sched_setaffinity(0, cpus)
    try:
        return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy()
    finally:
        if old is not None:
            os.sched_setaffinity(0, old)


def host_link_gbs(torch, hin, hout):
    """One copy of the run's own host buffers each way, after its timed
    runs: what the host link gave these buffers (GB/s)."""
    a = torch.from_numpy(hin.reshape(-1).view(np.uint8))
    b = torch.from_numpy(hout.reshape(-1).view(np.uint8))
    d = torch.empty(a.numel(), dtype=torch.uint8, device="cuda")
    d.copy_(a, non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d.copy_(a, non_blocking=True)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    b.copy_(d[:b.numel()], non_blocking=True)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    del d
    return {"h2d": round(a.numel() / (t1 - t0) / 1e9, 1), "d2h": round(b.numel() / (t2 - t1) / 1e9, 1)}


def e2e_of(w, torch, runs, dist=None, world=1):
    """The workload's run through the C ABI with host buffers: upload from
    pinned memory, run_steps time steps, download - averaged over runs."""
    hin, hout = w.host_buffers(torch)
    w.e2e_run(hin, hout)     # warm-up
    runs = max(1, runs)
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(runs):
        bi, bo = w.e2e_run(hin, hout)
    t1 = time.perf_counter()
    barrier(dist)
    e2e_s = max_over_ranks(dist, t1 - t0)
    pl = host_placement(torch)
    return {"value": round(w.units * w.run_steps * runs * world / e2e_s / 1e9, 3), "unit": w.unit,
            "h2d_bytes_per_step": int(bi), "d2h_bytes_per_step": int(bo),
            "step": "upload from pinned host + %d time steps + download, through the C ABI" % w.run_steps,
            "ms_per_step": round(e2e_s * 1e3 / runs, 3),
            "host_link_gbs": host_link_gbs(torch, hin, hout),
            "host_numa": {k: pl[k] for k in ("numa_nodes", "gpu_node", "bound_to_gpu_node")}}


def measure(torch, w, steps, warmup, local, dist, world, peak, peak_kind):
    """Warm-up, then exactly `steps` time steps timed with CUDA events between
    barriers and device synchronisations; clocks sampled meanwhile."""
    w.step(warmup)
    w.sync()
    launches0 = w.launches()
    barrier(dist)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = time_steps(torch, w, steps)
    torch.cuda.synchronize()
    barrier(dist)
    launches = w.launches() - launches0
    ms = max_over_ranks(dist, ms)
    return {"ms": ms, "launches": launches, "clocks": clk.summary(),
            "value": w.units * steps * world / (ms * 1e-3) / 1e9,
            "roofline": roofline_of(w, ms, steps, launches, peak, peak_kind)}


def sell_renumbering(torch, w, steps=50):
    """ms per step of the SELL kernel with and without the reverse
    Cuthill-McKee numbering (LGD_SELL_RENUMBER; the node values agree to
    rounding: a renumbered row sums its entries in another order): the
    configuration's graph, whose targets are
    uniform at random, and a periodic 160^3 7-point mesh numbered at random,
    whose locality the numbering recovers."""
    from libgeodecomp_gb300 import lgd, workloads

    def timed(g):
        st = torch.cuda.ExternalStream(g.stream())
        g.step(3)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st)
        g.step(steps)
        b.record(st)
        b.synchronize()
        return a.elapsed_time(b) / steps

    out = {}
    rp, col, wt = workloads.powerlaw_graph(w.n, seed=42)
    with lgd.SellGrid.from_csr(w.n, rp, col, wt, 32, 256, renumber=True) as g:
        g.upload(w.x0)
        out["config_graph_ms_per_step"] = {"plain": round(timed(w.g), 4), "renumbered": round(timed(g), 4)}
    del rp, col, wt
    n1 = 160
    n = n1 ** 3
    idx = np.arange(n, dtype=np.int64).reshape(n1, n1, n1)
    perm = np.random.default_rng(7).permutation(n)
    rows = np.concatenate([perm[idx.ravel()]] * 6)
    cols = np.concatenate([perm[np.roll(idx, shift=d, axis=(0, 1, 2)).ravel()]
                           for d in ((0, 0, 1), (0, 0, -1), (0, 1, 0), (0, -1, 0), (1, 0, 0), (-1, 0, 0))])
    o = np.argsort(rows, kind="stable")
    cols = cols[o].astype(np.int32)
    rpm = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rpm, rows + 1, 1)
    rpm = np.cumsum(rpm)
    wm = np.full(cols.size, 0.15)
    x0 = workloads.sell_values(n, seed=3)
    mesh = {}
    for renumber in (False, True):
        with lgd.SellGrid.from_csr(n, rpm, cols, wm, 32, 256, renumber=renumber) as g:
            g.upload(x0)
            mesh["renumbered" if renumber else "random_numbering"] = round(timed(g), 4)
    out["mesh_160cubed_ms_per_step"] = mesh
    return out


def run_secondary(torch, args, local, peak, peak_kind):
    """The other configurations, one compact block each."""
    out = {}
    for name, steps, warmup, has_e2e in SECONDARY:
        t0 = time.perf_counter()
        try:
            w = make_workload(name, argparse.Namespace(**dict(vars(args), size=512, time_block=0)))
            m = measure(torch, w, steps, warmup, local, None, 1, peak, peak_kind)
            block = {"metric": w.metric, "value": round(m["value"], 3), "unit": w.unit, "steps": steps,
                     "warmup": warmup, "ms_per_step": round(m["ms"] / steps, 5), "gpu_launches": m["launches"],
                     "dtype": DTYPES[name], "config": workload_config(name, args), "roofline": m["roofline"],
                     "clocks": m["clocks"], "setup": w.setup}
            if name == "sell_f64_4m":
                block["s_per_step"] = round(m["ms"] / steps * 1e-3, 7)
                block["renumbering"] = sell_renumbering(torch, w)
            if name == "lbm_d3q19_ensemble_512":
                lms = w.looped_ms(torch, 4)
                block["looped_single_grid_launches"] = {"ms_per_step": round(lms, 3),
                                                        "glups": round(w.units / (lms * 1e-3) / 1e9, 2)}
                block["e2e"] = None
                block["e2e_note"] = ("no host round trip: the ensemble's populations are 83 GB per buffer, "
                                     "about 0.8 s per upload and download at the host link's rate")
            elif has_e2e and not args.no_e2e:
                block["e2e"] = e2e_of(w, torch, args.secondary_e2e_runs)
            w.close()
            del w
            torch.cuda.synchronize()
            block["wall_s"] = round(time.perf_counter() - t0, 1)
            out[name] = block
        except Exception as e:      # a failing secondary must not hide the headline
            out[name] = {"error": "%s: %s" % (type(e).__name__, e)}
    return out


def dropin_run(edge=512, steps=100):
    """GB300Simulator::run() of the C++ example program (a LibGeoDecomp-style
    application on the drop-in): wall time of run() - initializer, upload,
    the steps, a writer reading every cell - and of the steps alone."""
    from libgeodecomp_gb300 import build
    src = os.path.join(ROOT, "libgeodecomp_gb300", "examples", "jacobi3d_dropin.cpp")
    libdir = os.path.join(ROOT, "libgeodecomp_gb300")
    exe = os.path.join(tempfile.mkdtemp(), "jacobi3d_dropin")
    build.build()
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(libdir, "include"), src, "-L", libdir, "-llgd_gb300", "-Wl,-rpath," + libdir,
                    "-o", exe], check=True, capture_output=True, text=True)
    res = subprocess.run([exe, str(edge), str(steps)], check=True, capture_output=True, text=True, timeout=600)
    out = json.loads(res.stdout.strip().splitlines()[-1])
    out["program"] = "libgeodecomp_gb300/examples/jacobi3d_dropin.cpp (%d^3, %d steps)" % (edge, steps)
    return out


def run_gpu(args, world, rank, local, dist):
    import torch
    torch.cuda.set_device(local)
    peak, peak_kind = load_peaks()
    if world > 1 and slab_capable(args.workload):
        return run_slabs(args, world, rank, local, dist, peak, peak_kind)
    if world > 1 and args.workload == "sell_f64_4m":
        return run_sell_shards(args, world, rank, local, dist)
    args.rank = rank
    w = make_workload(args.workload, args)
    if hasattr(w, "set_time_block"):
        w.set_time_block(args.time_block, args.time_block_shape)
    m = measure(torch, w, args.steps, args.warmup, local, dist, world, peak, peak_kind)
    ms, launches = m["ms"], m["launches"]
    ms_per_step = ms / args.steps

    e2e = None
    if not args.no_e2e and args.workload != "lbm_d3q19_ensemble_512":
        e2e = e2e_of(w, torch, args.e2e_runs, dist, world)

    extra = {}
    if args.workload == "jacobi7_f64_512" and not args.no_ieee and world == 1:
        # the same grid at the other blocking depth (steps fused per pass)
        sweep = {}
        for depth in (1, 2):         # the fixed-point cell fuses at most two steps
            if depth == min(args.time_block or 2, 2):     # the depth the headline ran at
                continue
            w.set_time_block(depth)
            w.step(2 * depth)
            k = 4 * depth
            msd = time_steps(torch, w, k) / k
            sweep[str(depth)] = {"glups": round(w.units / (msd * 1e-3) / 1e9, 2), "ms_per_step": round(msd, 4),
                                 "hbm_frac_per_pass": round(w.units * 16 / (msd * depth * 1e-3) / 1e9 / peak, 4)}
        extra["time_block_sweep"] = sweep
        w.close()
        wi = make_workload("jacobi7_f64_ieee_512", args)
        for _ in range(3):
            wi.step(1)
        wi.sync()
        k = max(3, args.steps // 4)
        ims = time_steps(torch, wi, k) / k
        extra["ieee_fp64_kernel"] = {
            "glups": round(wi.units / (ims * 1e-3) / 1e9, 2), "ms_per_step": round(ims, 4),
            "hbm_frac": round(wi.units * 16 / (ims * 1e-3) / 1e9 / peak, 4),
            "note": "LGD_CELL_JACOBI7_F64: bit-identical to the reference; bound by the GPU's FP64 rate"}
        wi.close()
    else:
        if args.workload == "lbm_d3q19_ensemble_512":
            # the same steps with one launch per instance (512 launches per step)
            lms = w.looped_ms(torch, max(2, args.steps // 4))
            extra["looped_single_grid_launches"] = {"ms_per_step": round(lms, 3),
                                                    "glups": round(w.units / (lms * 1e-3) / 1e9, 2)}
            extra["e2e_note"] = "no host round trip: the 166 GB ensemble lives on the device"
        w.close()
    if args.workload == "sell_f64_4m":
        extra["s_per_step"] = round(ms_per_step * 1e-3, 7)
    if w.setup:
        extra["setup"] = w.setup

    secondary = None
    if rank == 0 and world == 1 and not args.no_secondary and args.workload == "jacobi7_f64_512":
        secondary = run_secondary(torch, args, local, peak, peak_kind)
        try:
            extra["dropin_run"] = dropin_run(args.size, 100)
        except Exception as e:      # the headline does not depend on it
            extra["dropin_run"] = {"error": "%s: %s" % (type(e).__name__, e)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.workload, budget_s=args.cpu_seconds)
        if secondary:
            for name, block in secondary.items():
                if "error" not in block:
                    try:
                        block["cpu_baseline"] = cpu_baseline(name, budget_s=args.secondary_cpu_seconds)
                    except Exception as e:
                        block["cpu_baseline"] = {"error": "%s: %s" % (type(e).__name__, e)}

    if rank == 0:
        line = {
            "metric": w.metric, "value": round(m["value"], 3), "unit": w.unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPES.get(args.workload, "f64"),
            "data": "synthetic (seeded SplitMix64, generated on device or by libgeodecomp_gb300.workloads)",
            "config": workload_config(args.workload, args, world),
            "gpu_launches": launches, "roofline": m["roofline"], "e2e": e2e, "cpu_baseline": cpu,
            "clocks": m["clocks"],
        }
        line.update(extra)
        if secondary is not None:
            line["secondary"] = secondary
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def timed_on_stream(torch, stream_ptr, fn):
    """(device ms, host seconds) of fn(): CUDA events recorded around it on
    the stream its kernels launch on.  The host synchronises every exchange
    between two launches, so the events' interval covers the exchanges."""
    st = torch.cuda.ExternalStream(stream_ptr)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    a.record(st)
    fn()
    b.record(st)
    b.synchronize()
    return a.elapsed_time(b), time.perf_counter() - t0


def rank_e2e(torch, one_run, hin, hout, units, run_steps, runs, dist, world, unit="GLUPS"):
    """End to end over ranks: every rank runs one_run() - its upload from
    pinned host memory, run_steps steps with their exchanges, its download -
    runs times after one warm-up; the max over ranks of the host time."""
    one_run()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(max(1, runs)):
        one_run()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    barrier(dist)
    runs = max(1, runs)
    return {"value": round(units * world * run_steps * runs / e2e_s / 1e9, 3), "unit": unit,
            "h2d_bytes_per_step": int(hin.nbytes), "d2h_bytes_per_step": int(hout.nbytes),
            "step": "per rank: upload from pinned host + %d time steps with exchanges + download, through the "
                    "library's API" % run_steps, "ms_per_step": round(e2e_s * 1e3 / runs, 3)}


def slab_e2e(torch, s, run_steps, runs, dist, world, units):
    """rank_e2e of a slab grid: each rank's local planes (ghost planes
    included) in and out."""
    dt = np.dtype(s.grid.members[0])
    nbytes = int(np.prod(s.local_shape)) * dt.itemsize
    hin = pinned(torch, nbytes).view(dt).reshape(s.local_shape)
    hout = pinned(torch, nbytes).view(dt).reshape(s.local_shape)
    s.grid.download(0, out=hin)

    def one_run():
        s.grid.upload(0, hin)
        s.since = s.period             # ghost planes refreshed before the first step
        s.step(run_steps)
        s.grid.download(0, out=hout)
    return rank_e2e(torch, one_run, hin, hout, units, run_steps, runs, dist, world)


def run_slabs(args, world, rank, local, dist, peak, peak_kind):
    """Weak scaling over z-slabs: every rank owns a size^3 slab of the
    size x size x (size * world) grid and exchanges ghost planes with its
    neighbours every pass (libgeodecomp_gb300.slabs)."""
    import torch
    from libgeodecomp_gb300 import lgd, slabs
    cell = {"jacobi7_f64_512": lgd.CELL_JACOBI7_F64_FIX, "jacobi7_f64_ieee_512": lgd.CELL_JACOBI7_F64,
            "jacobi7_f32_512": lgd.CELL_JACOBI7_F32, "varcoef_f32_256": lgd.CELL_VARCOEF_F32,
            "gol_u8_8192": lgd.CELL_GOL_U8}[args.workload]
    n = {"varcoef_f32_256": 256, "gol_u8_8192": 8192}.get(args.workload, args.size)
    comm = slabs.TorchComm(dist, device=True)
    if args.workload == "gol_u8_8192":
        # a torus of world slabs of 8192^2 cells, cut along y; ghost zones of
        # 16 rows (one 16-generation pass between exchanges)
        s = slabs.SlabGrid(cell, (n * world, n), comm, periodic=3, ghost=max(args.slab_ghost, 16),
                           time_block=args.time_block)
    else:
        s = slabs.SlabGrid(cell, (n * world, n, n), comm, periodic=7 if args.workload == "varcoef_f32_256" else 0,
                           ghost=args.slab_ghost, time_block=args.time_block)
    if args.workload == "gol_u8_8192":
        s.fill_bernoulli(0.3, seed=42)
    elif args.workload == "varcoef_f32_256":
        from libgeodecomp_gb300 import workloads
        u0, kappa = workloads.varcoef_fields(n, seed=42, length=16.0)
        s.upload(0, np.concatenate([u0] * world).astype(np.float32))
        s.upload(1, np.concatenate([kappa] * world).astype(np.float32))
    else:
        s.fill_uniform(seed=42)
    s.step(args.warmup)
    s.synchronize()
    barrier(dist)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms, host_s = timed_on_stream(torch, s.grid.stream(), lambda: (s.step(args.steps), s.synchronize()))
    torch.cuda.synchronize()
    barrier(dist)
    dt = max_over_ranks(dist, ms * 1e-3)
    host_s = max_over_ranks(dist, host_s)
    units = n * n if args.workload == "gol_u8_8192" else n * n * n
    value = units * world * args.steps / dt / 1e9
    launches = s.launch_count()
    e2e = None
    if not args.no_e2e:
        run_steps = {"gol_u8_8192": GoLWorkload.run_steps}.get(args.workload, JacobiWorkload.run_steps)
        try:
            e2e = slab_e2e(torch, s, run_steps, args.e2e_runs, dist, world, units)
        except Exception as e:      # the device-timed line stands without it
            e2e = {"error": "%s: %s" % (type(e).__name__, e)}
    if rank == 0:
        line = {"metric": JACOBI_METRIC if args.workload.startswith("jacobi7") else METRICS[args.workload],
                "value": round(value, 3), "unit": "GLUPS", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": DTYPES.get(args.workload, "f64"),
                "data": "synthetic (seeded SplitMix64, generated on device)",
                "config": workload_config(args.workload, args, world), "gpu_launches": launches,
                "timing": "CUDA events on each rank's grid stream around its steps (ghost exchanges included), "
                          "max over ranks", "host_ms_per_step": round(host_s * 1e3 / args.steps, 4),
                "slabs": s.describe(), "e2e": e2e, "cpu_baseline": None, "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    s.close()
    dist.destroy_process_group()


def run_sell_shards(args, world, rank, local, dist):
    """Strong scaling of the 4,194,304-node SELL-C-sigma diffusion over row
    blocks: every rank updates its chunks and the ranks all-gather the new
    node values every step (libgeodecomp_gb300.sell_shards)."""
    import torch
    from libgeodecomp_gb300 import lgd, sell_shards, slabs, workloads
    n = SellWorkload.n
    rp, col, w = workloads.powerlaw_graph(n, seed=42)
    g = lgd.SellGrid.from_csr(n, rp, col, w, 32, 256)
    g.upload(workloads.sell_values(n, seed=42))
    s = sell_shards.ShardedSell(g, slabs.TorchComm(dist, device=True), 32)
    s.step(args.warmup)
    s.synchronize()
    barrier(dist)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms, host_s = timed_on_stream(torch, g.stream(), lambda: (s.step(args.steps), s.synchronize()))
    torch.cuda.synchronize()
    barrier(dist)
    dt = max_over_ranks(dist, ms * 1e-3)
    host_s = max_over_ranks(dist, host_s)
    e2e = None
    if not args.no_e2e:
        try:
            hin = pinned(torch, n * 8).view(np.float64)
            hout = pinned(torch, n * 8).view(np.float64)
            hin[:] = workloads.sell_values(n, seed=42)

            def one_run():
                g.upload(hin)
                s.step(SellWorkload.run_steps)
                g.download(out=hout)
            e2e = rank_e2e(torch, one_run, hin, hout, n, SellWorkload.run_steps, args.e2e_runs, dist, 1)
        except Exception as e:      # the device-timed line stands without it
            e2e = {"error": "%s: %s" % (type(e).__name__, e)}
    if rank == 0:
        line = {"metric": METRICS["sell_f64_4m"], "value": round(n * args.steps / dt / 1e9, 3), "unit": "GLUPS",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(dt * 1e3 / args.steps, 4), "s_per_step": round(dt / args.steps, 7),
                "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded power-law graph and values)",
                "config": workload_config("sell_f64_4m", args, world), "gpu_launches": args.steps,
                "timing": "CUDA events on each rank's grid stream around its steps (all-gathers included), "
                          "max over ranks", "host_ms_per_step": round(host_s * 1e3 / args.steps, 4),
                "row_blocks": s.describe(), "e2e": e2e, "cpu_baseline": None, "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    g.close()
    dist.destroy_process_group()


# ------------------------------------------------------------ CPU baseline
def cpu_stepper(name):
    """(units per step, state, function advancing the state by s steps) of
    the oracle for a workload."""
    import oracle
    from libgeodecomp_gb300 import workloads
    if name.startswith("jacobi7"):
        st = oracle.Jacobi7PingPong(workloads.jacobi_initial(512, 512, 512, seed=42))
        return st.a.size, st, lambda a, s: a.step(s)
    if name == "gol_u8_8192":
        c = workloads.gol_initial(8192, 8192, seed=42)
        return c.size, c, lambda a, s: oracle.gol(a, s)
    if name == "sell_f64_4m":
        n = 4194304
        rp, col, w = workloads.powerlaw_graph(n, seed=42)
        s = oracle.sell_build(n, rp, col, w, 32, 256)
        x = workloads.sell_values(n, seed=42)[s["perm"]]
        return n, x, lambda a, k: oracle.sell_diffusion(s, 32, a, k)
    if name == "varcoef_f32_256":
        u0, kappa = workloads.varcoef_fields(256, seed=42, length=16.0)
        return u0.size, u0, lambda a, k: oracle.varcoef(a, kappa, k)
    if name == "lbm_d3q19_ensemble_512":
        # the ensemble's first instances (same edges and omegas), FP64, until
        # about 2e7 cells; the oracle has no FP32 cell
        edges, omegas = workloads.lbm_ensemble(512, seed=42, edge_max=192)
        take, cells = 0, 0
        while take < len(edges) and cells < 20_000_000:
            cells += int(edges[take]) ** 3
            take += 1
        sample = [oracle.lbm_rest(int(L)) for L in edges[:take]]

        def advance(fs, k):
            return [oracle.lbm(int(L), k, float(om), 0.05, f) for f, L, om in zip(fs, edges[:take], omegas[:take])]
        advance.sample = "the ensemble's first %d cavities (%d cells), FP64" % (take, cells)
        return cells, sample, advance
    raise ValueError(name)


def cpu_baseline(name: str, budget_s: float = 15.0):
    """The oracle on all host cores, on whole time steps of the same input,
    for about budget_s seconds."""
    import oracle
    units, state, fn = cpu_stepper(name)
    state = fn(state, 1)
    t0 = time.perf_counter()
    state = fn(state, 1)
    one = time.perf_counter() - t0
    steps = max(1, int(budget_s / max(one, 1e-6)))
    t0 = time.perf_counter()
    fn(state, steps)
    dt = time.perf_counter() - t0
    what = getattr(fn, "sample", "the %s input" % name)
    return {"value": round(units * steps / dt / 1e9, 4), "unit": "GLUPS", "cores": oracle.max_threads(),
            "kind": "port", "sample": "%d whole time steps of %s (%.1f s)" % (steps, what, dt)}


def run_reference(args, world, rank):
    if rank != 0:
        return
    import oracle
    units, state, fn = cpu_stepper(args.workload)
    for _ in range(args.warmup):
        state = fn(state, 1)
    t0 = time.perf_counter()
    state = fn(state, args.steps)
    dt = time.perf_counter() - t0
    value = units * args.steps / dt / 1e9
    line = {
        "metric": METRICS.get(args.workload, JACOBI_METRIC), "value": round(value, 4), "unit": "GLUPS",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (IEEE, the reference's cell arithmetic)" if args.workload.startswith("jacobi7_f64")
        else DTYPES.get(args.workload, "f64"),
        "data": "synthetic (seeded SplitMix64, generated on device or by libgeodecomp_gb300.workloads)",
        "config": workload_config(args.workload, args, world),
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 4), "unit": "GLUPS", "cores": oracle.max_threads(), "kind": "port",
                         "sample": "%d whole time steps of the %s input%s" % (
                             args.steps, args.workload, " (rank 0 only, one slab's worth of cells)"
                             if world > 1 else "")},
        "e2e": {"value": round(value, 4), "unit": "GLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_surrogate(args):
    """Learned surrogate for variable-coefficient diffusion on 256^3 FP32 to
    t = 4096 steps: train on plain-stencil trajectories (GPU, the library's
    own forward / backward / Adam kernels), then time surrogate plus judge
    against the plain FP32 stencil, both measured against the FP64 stencil."""
    import torch
    from libgeodecomp_gb300 import surrogate as S
    from libgeodecomp_gb300 import workloads
    n = args.surrogate_size
    steps = args.surrogate_steps
    t0 = time.perf_counter()
    states, kappa_tr = S.make_trajectories(count=args.trajectories, n=args.train_size, calls=4, length=16.0, seed=7)
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    params, hist = S.train(states, kappa_tr, channels=24, iters=args.train_iters, batch=8, lr=1e-3, seed=1)
    t_train = time.perf_counter() - t0
    err_net, err_id = S.one_call_errors(params, states[-64:], kappa_tr[-64:], channels=24)
    del states, kappa_tr

    u0_np, k_np = workloads.varcoef_fields(n, seed=42, length=16.0)
    u0 = torch.tensor(u0_np, dtype=torch.float32, device="cuda").contiguous()
    kap = torch.tensor(k_np, dtype=torch.float32, device="cuda").contiguous()
    # FP64 reference with the FP64 stencil (bit-identical to the reference's
    # simulator at small sizes, see tests), timed: the comparator an FP64
    # user would otherwise run
    ref = S.PlainStencil(n, precision=8)
    try:
        u64 = torch.tensor(u0_np, dtype=torch.float64, device="cuda").contiguous()
        ref.set_kappa(torch.tensor(k_np, dtype=torch.float64, device="cuda").contiguous())
        ref.run(u64.clone(), 16)                     # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ref.run(u64, steps)
        torch.cuda.synchronize()
        t_fp64 = time.perf_counter() - t0
    finally:
        ref.close()
    S.run_plain(u0, kap, 16)                         # warm-up
    S.run_surrogate_with_judge(params, u0, kap, S.STEPS_PER_CALL * S.CALLS_PER_JUDGE, tol=args.judge_tol)
    u_plain, t_plain = S.run_plain(u0, kap, steps)
    u_sur, t_sur, stats = S.run_surrogate_with_judge(params, u0, kap, steps, tol=args.judge_tol)
    # the same run with a judge that accepts the network's own error level:
    # what the surrogate path costs and how far it drifts when it is used
    u_rel, t_rel, st_rel = S.run_surrogate_with_judge(params, u0, kap, steps, tol=args.relaxed_tol)
    # and with the judge at the accuracy bar itself (one call within 1e-3)
    u_bar, t_bar, st_bar = S.run_surrogate_with_judge(params, u0, kap, steps, tol=1e-3)
    net_ms = S.time_calls(params, u0, kap, calls=8)
    line = {
        "metric": "surrogate vs plain time at rel-L2<=1e-3", "value": round(t_plain / t_sur, 4),
        "unit": "x (plain FP32 stencil time / surrogate-plus-judge time)", "higher_is_better": True,
        "n_gpus": 1, "steps": steps, "warmup": 1, "dtype": "bf16 net (fp32 accumulate), fp32 plain stencil",
        "data": "synthetic (seeded Gaussian random fields)", "vs_baseline": None, "scaling": "weak",
        "config": {"workload": "surrogate_varcoef_%d" % n, "grid": [n, n, n], "t_final": steps,
                   "kappa": "GRF length 16 mapped to [0.02, 0.15]", "net": "4 x conv3^3, 24 ch, GELU, residual",
                   "steps_per_call": S.STEPS_PER_CALL, "judge_every_calls": S.CALLS_PER_JUDGE,
                   "judge_tol": args.judge_tol, "trajectories": args.trajectories, "train_iters": args.train_iters,
                   "train_size": args.train_size},
        "plain_fp32_s": round(t_plain, 4), "plain_fp64_s": round(t_fp64, 4), "surrogate_judge_s": round(t_sur, 4),
        "comparators": {"fp64_over_surrogate": round(t_fp64 / t_sur, 4),
                        "fp64_over_relaxed_surrogate": round(t_fp64 / t_rel, 4),
                        "fp32_over_surrogate": round(t_plain / t_sur, 4)},
        "rel_l2_vs_fp64": {"plain_fp32": S.rel_l2(u_plain, u64), "surrogate_judge": S.rel_l2(u_sur, u64)},
        "judge": {"segments": stats["segments"], "fallbacks": stats["fallbacks"],
                  "max_error": max(stats["judge_errors"]) if stats["judge_errors"] else None,
                  "min_error": min(stats["judge_errors"]) if stats["judge_errors"] else None,
                  "median_error": float(np.median(stats["judge_errors"])) if stats["judge_errors"] else None},
        "relaxed_judge": {"tol": args.relaxed_tol, "surrogate_judge_s": round(t_rel, 4),
                          "plain_over_surrogate": round(t_plain / t_rel, 4), "fallbacks": st_rel["fallbacks"],
                          "segments": st_rel["segments"], "rel_l2_vs_fp64": S.rel_l2(u_rel, u64)},
        "judge_at_1e-3": {"tol": 1e-3, "surrogate_judge_s": round(t_bar, 4),
                          "plain_over_surrogate": round(t_plain / t_bar, 4), "fallbacks": st_bar["fallbacks"],
                          "segments": st_bar["segments"], "rel_l2_vs_fp64": S.rel_l2(u_bar, u64)},
        "net_call_ms": round(net_ms, 4),
        "net_call_tflops": round(S.FLOP_PER_VOXEL * n ** 3 / (net_ms * 1e-3) / 1e12, 1),
        "plain_16_steps_ms": round(t_plain / steps * S.STEPS_PER_CALL * 1e3, 4),
        "training": {"data_s": round(t_data, 2), "train_s": round(t_train, 2), "loss_first": hist[0],
                     "loss_last": float(np.mean(hist[-20:])),
                     "one_call_rel_l2": {"net": float(err_net), "no_learning_baseline": float(err_id)}},
    }
    print(json.dumps(line), flush=True)


def run_net_calls(args):
    """The surrogate network alone: --net-calls calls (u <- u + net(u, k)) on
    a --surrogate-size^3 grid with randomly initialised parameters, after
    one warm-up call (inference path; for profiling the layers)."""
    import torch
    from libgeodecomp_gb300 import surrogate as S
    from libgeodecomp_gb300 import workloads
    n = args.surrogate_size
    u0_np, k_np = workloads.varcoef_fields(n, seed=42, length=16.0)
    u0 = torch.tensor(u0_np, dtype=torch.float32, device="cuda").contiguous()
    kap = torch.tensor(k_np, dtype=torch.float32, device="cuda").contiguous()
    ms = S.time_calls(S.init_params(24, seed=0), u0, kap, calls=args.net_calls)
    print(json.dumps({"metric": "surrogate network call", "value": round(ms, 4), "unit": "ms per call",
                      "higher_is_better": False, "tflops": round(S.FLOP_PER_VOXEL * n ** 3 / (ms * 1e-3) / 1e12, 1),
                      "config": {"workload": "surrogate_net_%d" % n, "calls": args.net_calls}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=WORKLOAD_NAMES, default="jacobi7_f64_512")
    ap.add_argument("--e2e-runs", type=int, default=5)
    ap.add_argument("--secondary-e2e-runs", type=int, default=3)
    ap.add_argument("--size", type=int, default=512, help="cube edge of the Jacobi workloads (small profiling cases)")
    ap.add_argument("--time-block", type=int, default=0, help="Jacobi steps fused per pass (0 = library default)")
    ap.add_argument("--time-block-shape", type=int, default=0, help="box shape of the fused passes (tuning)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--secondary-cpu-seconds", type=float, default=5.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-ieee", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="headline workload only")
    ap.add_argument("--slab-ghost", type=int, default=8, help="ghost planes per side (steps between exchanges)")
    ap.add_argument("--lbm-instances", type=int, default=512, help="ensemble size (smaller for profiling captures)")
    ap.add_argument("--lbm-edge-max", type=int, default=192)
    ap.add_argument("--lbm-no-tune", action="store_true", help="keep the default launch shape (profiling captures)")
    ap.add_argument("--lbm-time-block", default="", help="depth,shape,ctas: steps per launch of the ensemble, "
                    "overriding the tuner (profiling captures)")
    ap.add_argument("--surrogate", action="store_true", help="run the learned-surrogate time-to-solution benchmark")
    ap.add_argument("--surrogate-size", type=int, default=256)
    ap.add_argument("--surrogate-steps", type=int, default=4096)
    ap.add_argument("--trajectories", type=int, default=2000)
    ap.add_argument("--train-iters", type=int, default=6000)
    ap.add_argument("--train-size", type=int, default=64, help="edge of the training trajectories' tori")
    ap.add_argument("--judge-tol", type=float, default=1e-4)
    ap.add_argument("--relaxed-tol", type=float, default=1e-2)
    ap.add_argument("--net-calls", type=int, default=0, help="time this many surrogate network calls alone")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.net_calls > 0:
        run_net_calls(args)
        return
    if args.surrogate:
        run_surrogate(args)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    # NCCL where the ranks exchange device data (slabs, SELL row blocks)
    exchanges = slab_capable(args.workload) or args.workload == "sell_f64_4m"
    world, rank, local, dist = dist_setup("nccl" if world > 1 and exchanges else "gloo")
    run_gpu(args, world, rank, local, dist)


if __name__ == "__main__":
    main()
