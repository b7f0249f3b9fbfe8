"""Speed of the oracle port against the reference itself, on the host cores.

The timed CPU baseline of the benchmark is the oracle port (the reference's
runner cannot be built where the GPU is: the reference's sources are not
there).  This script times both on the same inputs and thread count here,
where oracle/_ref/lgd_ref is built from the reference's own headers
(oracle/Makefile), so that the port's figure can be read as the reference's:
a ratio port/reference below 1 means the port is slower than the reference.

    python oracle/calibrate_port.py [--threads T] [--only jacobi,gol,sell,lbm,varcoef]

Prints one JSON object per workload.  Test infrastructure: nothing of the
library runs here.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from libgeodecomp_gb300 import workloads  # noqa: E402


def run_ref(args, threads):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="false")
    out = subprocess.run([os.path.join(HERE, "_ref", "lgd_ref"), *map(str, args)], env=env, check=True,
                         capture_output=True, text=True).stdout
    return json.loads(out.strip().splitlines()[-1])


def best_of(fn, repeats=3):
    best = float("inf")
    for _ in range(repeats):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return best


def jacobi(tmp, threads, edge=256, steps=8):
    u0 = workloads.jacobi_initial(edge, edge, edge, seed=42)
    path = os.path.join(tmp, "u.f64")
    u0.tofile(path)
    ref_s = min(run_ref(["jacobi7", "cube", edge, edge, edge, steps, path, os.path.join(tmp, "o.f64"), "omp",
                         "time"], threads)["seconds"] for _ in range(3))
    # whole steps between two preallocated buffers, as the benchmark's CPU
    # baseline times them (no allocation, no copy of the input)
    st = oracle.Jacobi7PingPong(u0, threads=threads)
    st.step(2)
    port_s = best_of(lambda: st.step(steps))
    cells = u0.size * steps
    return {"workload": "jacobi7 %d^3 x %d" % (edge, steps), "ref_glups": cells / ref_s / 1e9,
            "port_glups": cells / port_s / 1e9, "port_over_ref": ref_s / port_s}


def gol(tmp, threads, edge=4096, steps=40):
    c0 = workloads.gol_initial(edge, edge, seed=42)
    path = os.path.join(tmp, "c.u8")
    c0.tofile(path)
    ref_s = min(run_ref(["gol", edge, edge, steps, path, os.path.join(tmp, "o.u8"), "omp", "time"],
                        threads)["seconds"] for _ in range(3))
    port_s = best_of(lambda: oracle.gol(c0, steps, threads=threads))
    cells = c0.size * steps
    return {"workload": "gol %d^2 x %d" % (edge, steps), "ref_glups": cells / ref_s / 1e9,
            "port_glups": cells / port_s / 1e9, "port_over_ref": ref_s / port_s}


def sell(tmp, threads, n=1 << 20, steps=10):
    rp, col, w = workloads.powerlaw_graph(n, seed=42)
    x0 = workloads.sell_values(n, seed=42)
    files = []
    for name, arr in (("rp.i64", rp.astype(np.int64)), ("col.i32", col.astype(np.int32)),
                      ("w.f64", w.astype(np.float64)), ("x.f64", x0.astype(np.float64))):
        files.append(os.path.join(tmp, name))
        arr.tofile(files[-1])
    ref_step = min(run_ref(["sell", 32, 256, n, len(col), steps, *files, os.path.join(tmp, "o.f64"), "omp", "time"],
                           threads)["s_per_step"] for _ in range(3))
    s = oracle.sell_build(n, rp, col, w, 32, 256)
    xp = x0[s["perm"]]
    port_s = best_of(lambda: oracle.sell_diffusion(s, 32, xp, steps, threads=threads))
    return {"workload": "sell-c-sigma %d nodes x %d" % (n, steps), "ref_glups": n / ref_step / 1e9,
            "port_glups": n * steps / port_s / 1e9, "port_over_ref": ref_step * steps / port_s}


def lbm(tmp, threads, edge=96, steps=10, omega=1.7):
    ref_s = min(run_ref(["lbm", edge, steps, omega, 0.05, os.path.join(tmp, "o.f64"), "omp", "time"],
                        threads)["seconds"] for _ in range(3))
    # the rest state is built once, outside the timing, as the reference
    # builds its grid before the timed steps (each call still copies it)
    f0 = oracle.lbm_rest(edge)
    oracle.lbm(edge, 1, omega, 0.05, f0, threads=threads)
    port_s = best_of(lambda: oracle.lbm(edge, steps, omega, 0.05, f0, threads=threads))
    cells = edge ** 3 * steps
    return {"workload": "d3q19 %d^3 x %d" % (edge, steps), "ref_glups": cells / ref_s / 1e9,
            "port_glups": cells / port_s / 1e9, "port_over_ref": ref_s / port_s}


def varcoef(tmp, threads, edge=128, steps=20):
    u0, k = workloads.varcoef_fields(edge, seed=42, length=16.0)
    pu, pk = os.path.join(tmp, "u.f64"), os.path.join(tmp, "k.f64")
    u0.tofile(pu)
    k.tofile(pk)
    ref_s = min(run_ref(["varcoef", edge, edge, edge, steps, pu, pk, os.path.join(tmp, "o.f64"), "omp", "time"],
                        threads)["seconds"] for _ in range(3))
    port_s = best_of(lambda: oracle.varcoef(u0, k, steps, threads=threads))
    cells = u0.size * steps
    return {"workload": "varcoef %d^3 x %d" % (edge, steps), "ref_glups": cells / ref_s / 1e9,
            "port_glups": cells / port_s / 1e9, "port_over_ref": ref_s / port_s}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--only", default="jacobi,gol,sell,lbm,varcoef")
    args = ap.parse_args()
    if not os.path.exists(os.path.join(HERE, "_ref", "lgd_ref")):
        sys.exit("oracle/_ref/lgd_ref is not built (make -C oracle)")
    with tempfile.TemporaryDirectory() as tmp:
        for name in args.only.split(","):
            r = {"jacobi": jacobi, "gol": gol, "sell": sell, "lbm": lbm, "varcoef": varcoef}[name](tmp, args.threads)
            r.update(threads=args.threads)
            print(json.dumps({k: round(v, 4) if isinstance(v, float) else v for k, v in r.items()}), flush=True)


if __name__ == "__main__":
    main()
