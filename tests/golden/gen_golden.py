#!/usr/bin/env python3
"""Write the golden fixtures in tests/golden/ by running the reference.

The reference runner ``oracle/_ref/lgd_ref`` (built by ``oracle/Makefile``
from the reference's own headers) advances each workload cell with the
reference's SerialSimulator / OpenMPSimulator, or dumps the SELL-C-sigma
arrays the reference builds.  Inputs come from
``libgeodecomp_gb300.workloads`` (seeded SplitMix64); each fixture stores
the SHA-256 of its inputs (the inputs themselves where they come from an
FFT, whose last bits may vary by platform), so a drifting generator is
caught instead of silently changing what the fixture means.

Run in the build container (the reference is not present elsewhere):
    python tests/golden/gen_golden.py [--only edge_shapes]
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from libgeodecomp_gb300 import workloads  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def run(args, tmp):
    ref = oracle.build_reference()
    if ref is None:
        raise SystemExit("reference headers not found; fixtures can only be generated in the build container")
    res = subprocess.run([ref] + [str(a) for a in args], cwd=tmp, check=True, capture_output=True, text=True)
    return json.loads(res.stdout.strip().splitlines()[-1]) if res.stdout.strip() else {}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def sample_indices(n: int, count: int = 4096) -> np.ndarray:
    return np.unique(np.linspace(0, n - 1, count).astype(np.int64))


def summary(a: np.ndarray) -> dict:
    flat = a.reshape(-1)
    idx = sample_indices(flat.size)
    return dict(sha256=np.array(hashlib.sha256(np.ascontiguousarray(flat).tobytes()).hexdigest()),
                sample_idx=idx, sample=flat[idx], total=np.array(flat.astype(np.float64).sum()))


def jacobi(tmp, name, topo, nx, ny, nz, steps, full=True):
    u0 = workloads.jacobi_initial(nx, ny, nz, seed=42)
    fin = os.path.join(tmp, "in.f64")
    fout = os.path.join(tmp, "out.f64")
    u0.tofile(fin)
    run(["jacobi7", topo, nx, ny, nz, steps, fin, fout, "serial"], tmp)
    out = np.fromfile(fout, dtype=np.float64).reshape(nz, ny, nx)
    extra = dict(out=out) if full else summary(out)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), shape=np.array([nz, ny, nx]), steps=np.array(steps),
                        torus=np.array(topo == "torus"), seed=np.array(42), u0_sha256=np.array(sha(u0)), **extra)


def bov(tmp, name, nx, ny, nz, steps):
    """Header and data files of the reference's SerialBOVWriter for the
    Jacobi cube cell at step 0 and at step `steps` (prefix "jac", relative
    to the working directory, as DATA_FILE records it)."""
    u0 = workloads.jacobi_initial(nx, ny, nz, seed=42)
    fin = os.path.join(tmp, "in.f64")
    u0.tofile(fin)
    run(["bov", nx, ny, nz, steps, fin, "jac"], tmp)
    files = {}
    for step in (0, steps):
        stem = os.path.join(tmp, "jac.%05d" % step)
        with open(stem + ".bov", "rb") as f:
            files["bov_%d" % step] = np.frombuffer(f.read(), dtype=np.uint8)
        with open(stem + ".data", "rb") as f:
            files["data_%d" % step] = np.frombuffer(f.read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), shape=np.array([nz, ny, nx]), steps=np.array(steps),
                        seed=np.array(42), u0_sha256=np.array(sha(u0)), **files)


def gol(tmp, name, nx, ny, steps, full=True):
    c0 = workloads.gol_initial(nx, ny, seed=42)
    fin = os.path.join(tmp, "in.u8")
    fout = os.path.join(tmp, "out.u8")
    c0.tofile(fin)
    run(["gol", nx, ny, steps, fin, fout, "omp"], tmp)
    out = np.fromfile(fout, dtype=np.uint8).reshape(ny, nx)
    if full:
        extra = dict(out=out, c0_sha256=np.array(sha(c0)))
    else:
        extra = dict(sha256=np.array(hashlib.sha256(out.tobytes()).hexdigest()),
                     row_alive=out.sum(axis=1).astype(np.int32))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), shape=np.array([ny, nx]), steps=np.array(steps),
                        seed=np.array(42), **extra)


def write_csr(tmp, row_ptr, col, w):
    row_ptr.astype(np.int64).tofile(os.path.join(tmp, "rp.i64"))
    col.astype(np.int32).tofile(os.path.join(tmp, "col.i32"))
    w.astype(np.float64).tofile(os.path.join(tmp, "w.f64"))


def read_sell(prefix, n):
    r = {}
    for key, dt in (("perm", np.int32), ("chunk_offset", np.int32), ("chunk_length", np.int32),
                    ("row_length", np.int32), ("values", np.float64), ("column", np.int32)):
        r[key] = np.fromfile(prefix + key + "." + ("f64" if dt == np.float64 else "i32"), dtype=dt)
    return r


def sell_dump(tmp, mode, n, row_ptr, col, w, C, sigma):
    write_csr(tmp, row_ptr, col, w)
    prefix = os.path.join(tmp, "sell_")
    run([mode, C, sigma, n, len(col), "rp.i64", "col.i32", "w.f64", prefix], tmp)
    return read_sell(prefix, n)


def ragged_graph(n):
    """Hand-made ragged CSR: row i has (7 i) mod 9 entries (0..8), targets
    (i + 1 + 3 k) mod n sorted, weights k + 1 + i / 100."""
    rows, cols, ws = [], [], []
    row_ptr = [0]
    for i in range(n):
        d = (7 * i) % 9
        t = sorted({(i + 1 + 3 * k) % n for k in range(d)})
        for k, c in enumerate(t):
            cols.append(c)
            ws.append(k + 1 + i / 100.0)
        row_ptr.append(len(cols))
    return np.array(row_ptr, dtype=np.int64), np.array(cols, dtype=np.int32), np.array(ws, dtype=np.float64)


def kat_matrix(entries, n):
    """CSR from (row, col, value) triples listed row-major."""
    entries = sorted(entries)
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    for r, _, _ in entries:
        row_ptr[r + 1] += 1
    row_ptr = np.cumsum(row_ptr)
    col = np.array([c for _, c, _ in entries], dtype=np.int32)
    w = np.array([v for _, _, v in entries], dtype=np.float64)
    return row_ptr, col, w


def sell_cases(tmp):
    cases = {}
    # the reference's own container known-answer matrices
    # (storage/test/unit/sellcsigmasparsematrixcontainertest.h:602-888)
    m4 = [(0, 1, 1), (0, 3, 2), (1, 3, 1), (2, 1, 2), (2, 3, 3), (3, 0, 1), (3, 1, 1)]
    m5 = [(0, 1, 1), (1, 1, 5), (1, 3, 8), (1, 4, 7), (2, 0, 1), (2, 1, 4), (2, 3, 3), (2, 4, 2),
          (3, 2, 5), (4, 3, 2), (4, 4, 3)]
    for tag, entries, n, C, sigma in (("kat4_c2s1", m4, 4, 2, 1), ("kat5_c2s1", m5, 5, 2, 1),
                                      ("kat5_c2s4", m5, 5, 2, 4), ("kat5_c2s8", m5, 5, 2, 8)):
        rp, col, w = kat_matrix(entries, n)
        d = sell_dump(tmp, "sellcontainer", n, rp, col, w, C, sigma)
        cases[tag] = dict(n=n, C=C, sigma=sigma, mode="container", row_ptr=rp, col=col, w=w, **d)
    # ragged hand-made graph, grid path
    rp, col, w = ragged_graph(37)
    for C, sigma in ((4, 1), (4, 60), (8, 16), (32, 256), (2, 4)):
        d = sell_dump(tmp, "sellbuild", 37, rp, col, w, C, sigma)
        cases["ragged37_c%ds%d" % (C, sigma)] = dict(n=37, C=C, sigma=sigma, mode="grid", row_ptr=rp, col=col, w=w, **d)
    # power-law graph, grid path
    n = 300
    rp, col, w = workloads.powerlaw_graph(n, seed=7)
    for C, sigma in ((32, 256), (8, 16)):
        d = sell_dump(tmp, "sellbuild", n, rp, col, w, C, sigma)
        cases["powerlaw300_c%ds%d" % (C, sigma)] = dict(n=n, C=C, sigma=sigma, mode="grid", row_ptr=rp, col=col, w=w, **d)
    flat = {}
    for tag, d in cases.items():
        for k, v in d.items():
            flat[tag + "__" + k] = np.array(v)
    np.savez_compressed(os.path.join(OUT, "sell_build.npz"), tags=np.array(sorted(cases)), **flat)


def sell_run(tmp, name, n, C, sigma, steps, seed, full=True):
    rp, col, w = workloads.powerlaw_graph(n, seed=seed)
    x0 = workloads.sell_values(n, seed=seed)
    write_csr(tmp, rp, col, w)
    x0.tofile(os.path.join(tmp, "x.f64"))
    run(["sell", C, sigma, n, len(col), steps, "rp.i64", "col.i32", "w.f64", "x.f64", "out.f64", "serial"], tmp)
    out = np.fromfile(os.path.join(tmp, "out.f64"), dtype=np.float64)
    extra = dict(out=out) if full else summary(out)
    extra["x0_sha256"] = np.array(sha(x0))
    extra["w_sha256"] = np.array(sha(w))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), n=np.array(n), C=np.array(C), sigma=np.array(sigma),
                        steps=np.array(steps), seed=np.array(seed), **extra)


def lbm(tmp, name, L, steps, omega, lid, full=True):
    run(["lbm", L, steps, repr(omega), repr(lid), "out.f64", "serial"], tmp)
    out = np.fromfile(os.path.join(tmp, "out.f64"), dtype=np.float64).reshape(19, L, L, L)
    extra = dict(out=out) if full else summary(out)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), L=np.array(L), steps=np.array(steps),
                        omega=np.array(omega), lid=np.array(lid), **extra)


def varcoef(tmp, name, n, steps, length):
    u0, k = workloads.varcoef_fields(n, seed=42, length=length)
    u0.tofile(os.path.join(tmp, "u.f64"))
    k.tofile(os.path.join(tmp, "k.f64"))
    run(["varcoef", n, n, n, steps, "u.f64", "k.f64", "out.f64", "serial"], tmp)
    out = np.fromfile(os.path.join(tmp, "out.f64"), dtype=np.float64).reshape(n, n, n)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), n=np.array(n), steps=np.array(steps),
                        length=np.array(length), u0=u0, k=k, out=out)


# degenerate and odd shapes of every cell, all in edge_shapes.npz
EDGE_JACOBI = [("cube", 1, 1, 9), ("cube", 9, 1, 1), ("cube", 1, 7, 1), ("cube", 2, 3, 5), ("cube", 5, 1, 3),
               ("torus", 1, 3, 4), ("torus", 4, 1, 1), ("torus", 3, 4, 1), ("torus", 1, 2, 2)]
# (the reference refuses a 3D torus with y = 1 and z > 1: "expected 1D grid, but z != 1")
EDGE_GOL = [(7, 5), (1, 9), (9, 1), (33, 17), (2, 2)]
EDGE_LBM = [2, 3]
EDGE_VARCOEF = [(1, 1, 4), (3, 5, 2), (7, 3, 5)]
EDGE_SELL = [(1000, 32, 256), (100, 4, 60), (130, 8, 16), (70, 2, 4)]      # (n, C, sigma)
EDGE_STEPS = 6


def edge_key(kind, *dims):
    return "%s_%s" % (kind, "x".join(str(d) for d in dims))


def edge_shapes(tmp):
    """Degenerate and odd shapes (axes of extent 1 and 2, sizes that are
    not multiples of C or sigma, boxes that are all wall cells) for every
    cell, EDGE_STEPS steps each, from seeded inputs (seed 7)."""
    out = {}
    for topo, nx, ny, nz in EDGE_JACOBI:
        u0 = workloads.jacobi_initial(nx, ny, nz, seed=7)
        u0.tofile(os.path.join(tmp, "in.f64"))
        run(["jacobi7", topo, nx, ny, nz, EDGE_STEPS, "in.f64", "out.f64", "serial"], tmp)
        out[edge_key("jacobi_" + topo, nx, ny, nz)] = np.fromfile(os.path.join(tmp, "out.f64"),
                                                                  dtype=np.float64).reshape(nz, ny, nx)
    for nx, ny in EDGE_GOL:
        c0 = workloads.gol_initial(nx, ny, seed=7)
        c0.tofile(os.path.join(tmp, "in.u8"))
        run(["gol", nx, ny, EDGE_STEPS, "in.u8", "out.u8", "serial"], tmp)
        out[edge_key("gol", nx, ny)] = np.fromfile(os.path.join(tmp, "out.u8"), dtype=np.uint8).reshape(ny, nx)
    for L in EDGE_LBM:
        run(["lbm", L, EDGE_STEPS, repr(1.5), repr(0.05), "out.f64", "serial"], tmp)
        out[edge_key("lbm", L)] = np.fromfile(os.path.join(tmp, "out.f64"), dtype=np.float64).reshape(19, L, L, L)
    for nx, ny, nz in EDGE_VARCOEF:
        n = nx * ny * nz
        u0 = workloads.uniform(7, workloads.STREAM_GRID, n).reshape(nz, ny, nx)
        k = 0.02 + 0.13 * workloads.uniform(7, workloads.STREAM_DEGREE, n).reshape(nz, ny, nx)
        u0.tofile(os.path.join(tmp, "u.f64"))
        k.tofile(os.path.join(tmp, "k.f64"))
        run(["varcoef", nx, ny, nz, EDGE_STEPS, "u.f64", "k.f64", "out.f64", "serial"], tmp)
        out[edge_key("varcoef", nx, ny, nz)] = np.fromfile(os.path.join(tmp, "out.f64"),
                                                           dtype=np.float64).reshape(nz, ny, nx)
    for n, C, sigma in EDGE_SELL:
        rp, col, w = workloads.powerlaw_graph(n, seed=7)
        x0 = workloads.sell_values(n, seed=7)
        write_csr(tmp, rp, col, w)
        x0.tofile(os.path.join(tmp, "x.f64"))
        run(["sell", C, sigma, n, len(col), EDGE_STEPS, "rp.i64", "col.i32", "w.f64", "x.f64", "out.f64", "serial"],
            tmp)
        out[edge_key("sell", n, C, sigma)] = np.fromfile(os.path.join(tmp, "out.f64"), dtype=np.float64)
    np.savez_compressed(os.path.join(OUT, "edge_shapes.npz"), steps=np.array(EDGE_STEPS), seed=np.array(7), **out)


def main():
    if sys.argv[1:] == ["--only", "edge_shapes"]:
        with tempfile.TemporaryDirectory() as tmp:
            edge_shapes(tmp)
        print("edge_shapes.npz written to", OUT)
        return
    with tempfile.TemporaryDirectory() as tmp:
        jacobi(tmp, "jacobi7_cube_24x20x16", "cube", 24, 20, 16, 10)
        jacobi(tmp, "jacobi7_torus_17x13x11", "torus", 17, 13, 11, 7)
        jacobi(tmp, "jacobi7_cube_128", "cube", 128, 128, 128, 100, full=False)
        gol(tmp, "gol_64x48", 64, 48, 50)
        gol(tmp, "gol_1024", 1024, 1024, 1000, full=False)
        sell_cases(tmp)
        sell_run(tmp, "sell_diffusion_2000", 2000, 32, 256, 20, seed=11)
        sell_run(tmp, "sell_diffusion_100k", 100000, 32, 256, 10, seed=12, full=False)
        lbm(tmp, "lbm_L8", 8, 30, 1.7, 0.05)
        lbm(tmp, "lbm_L24", 24, 100, 1.2, 0.05, full=False)
        varcoef(tmp, "varcoef_16", 16, 20, 4.0)
        bov(tmp, "bov_jacobi_24x20x16", 24, 20, 16, 6)
        edge_shapes(tmp)
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()
