"""CPU oracle for the cell-update hot path (test infrastructure only).

``oracle/lgd_oracle.c`` restates the reference's algorithms in plain C;
this module builds it into ``oracle/liblgd_oracle.so`` and exposes numpy
wrappers.  Only the tests, the smoke check and the CPU-baseline leg of the
benchmark may import it - to compare results against, never as the thing
measured or shipped.  ``oracle/_ref/lgd_ref`` (built by ``oracle/Makefile`` from the
reference's own headers, only where they are present) is the reference
itself; ``tests/golden/gen_golden.py`` runs it to pin this oracle.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblgd_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "lgd_ref")
# where the reference's sources lie (only in the build container)
REFERENCE_ROOT = os.environ.get("LGD_REFERENCE_ROOT", "/root/reference")

_lib = None


def build(force: bool = False) -> str:
    """Compile the C restatement (gcc -O3, OpenMP, no FMA contraction: the
    vectorised loops keep every cell's operations and their order)."""
    src = os.path.join(HERE, "lgd_oracle.c")
    hdr = os.path.join(HERE, "lbm_d3q19.h")
    newest = max(os.path.getmtime(src), os.path.getmtime(hdr))
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               src, "-o", LIB_PATH + ".tmp"]
        subprocess.check_call(cmd)
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


def build_reference(force: bool = False) -> str | None:
    """Build oracle/_ref/lgd_ref from the reference headers if they exist."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "src", "libgeodecomp")):
        return None
    if force or not os.path.exists(REF_BIN):
        subprocess.check_call(["make", "-C", HERE, "REF=" + REFERENCE_ROOT])
    return REF_BIN


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int
        D = ctypes.c_double
        L.lgd_oracle_max_threads.restype = I
        L.lgd_oracle_jacobi7.argtypes = [I, I, I, I, D, I, P, I]
        L.lgd_oracle_jacobi7_pp.argtypes = [I, I, I, I, D, I, P, P, I]
        L.lgd_oracle_gol.argtypes = [I, I, I, P, I]
        L.lgd_oracle_sell_plan.argtypes = [I, P, I, I, P, P, P, P]
        L.lgd_oracle_sell_plan.restype = ctypes.c_longlong
        L.lgd_oracle_sell_fill.argtypes = [I, P, P, P, I, P, P, ctypes.c_longlong, P, P, I]
        L.lgd_oracle_sell_diffusion.argtypes = [I, I, P, P, P, P, I, P, I]
        L.lgd_oracle_lbm.argtypes = [I, I, D, D, P, I]
        L.lgd_oracle_varcoef.argtypes = [I, I, I, I, P, P, I]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def max_threads() -> int:
    return lib().lgd_oracle_max_threads()


def jacobi7(u: np.ndarray, steps: int, torus: bool = False, edge: float = 0.0, threads: int = 0) -> np.ndarray:
    """Advance a (nz, ny, nx) FP64 grid; returns a new array."""
    out = np.ascontiguousarray(u, dtype=np.float64).copy()
    nz, ny, nx = out.shape
    rc = lib().lgd_oracle_jacobi7(nx, ny, nz, int(torus), float(edge), int(steps), _ptr(out), threads)
    assert rc == 0
    return out


class Jacobi7PingPong:
    """Jacobi-7 state with two preallocated buffers, for timing whole steps
    without allocation or copies."""

    def __init__(self, u: np.ndarray, torus: bool = False, edge: float = 0.0, threads: int = 0):
        self.a = np.ascontiguousarray(u, dtype=np.float64).copy()
        self.b = np.empty_like(self.a)
        self.torus, self.edge, self.threads = int(torus), float(edge), threads

    def step(self, steps: int) -> "Jacobi7PingPong":
        nz, ny, nx = self.a.shape
        if lib().lgd_oracle_jacobi7_pp(nx, ny, nz, self.torus, self.edge, int(steps), _ptr(self.a), _ptr(self.b),
                                       self.threads):
            self.a, self.b = self.b, self.a
        return self


def gol(cells: np.ndarray, steps: int, threads: int = 0) -> np.ndarray:
    out = np.ascontiguousarray(cells, dtype=np.uint8).copy()
    ny, nx = out.shape
    assert lib().lgd_oracle_gol(nx, ny, int(steps), _ptr(out), threads) == 0
    return out


def sell_build(n: int, row_ptr: np.ndarray, col: np.ndarray, w: np.ndarray, C: int, sigma: int,
               remap_columns: bool = True) -> dict:
    """SELL-C-sigma arrays as the reference builds them (physical order).

    remap_columns=True is the grid path (ReorderingUnstructuredGrid),
    False the bare SellCSigmaSparseMatrixContainer."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    w = np.ascontiguousarray(w, dtype=np.float64)
    n_chunks = (n - 1) // C + 1
    perm = np.zeros(n, dtype=np.int32)
    row_length = np.zeros(n_chunks * C, dtype=np.int32)
    chunk_length = np.zeros(n_chunks, dtype=np.int32)
    chunk_offset = np.zeros(n_chunks + 1, dtype=np.int32)
    total = lib().lgd_oracle_sell_plan(n, _ptr(row_ptr), C, sigma, _ptr(perm), _ptr(row_length),
                                       _ptr(chunk_length), _ptr(chunk_offset))
    assert total >= 0
    values = np.zeros(max(total, 1), dtype=np.float64)
    column = np.zeros(max(total, 1), dtype=np.int32)
    rc = lib().lgd_oracle_sell_fill(n, _ptr(row_ptr), _ptr(col), _ptr(w), C, _ptr(perm),
                                    _ptr(chunk_offset), total, _ptr(values), _ptr(column),
                                    int(remap_columns))
    assert rc == 0
    return dict(perm=perm, row_length=row_length, chunk_length=chunk_length,
                chunk_offset=chunk_offset, values=values[:total], column=column[:total])


def sell_diffusion(sell: dict, C: int, x_phys: np.ndarray, steps: int, threads: int = 0) -> np.ndarray:
    """x' = 0.1 x + W x on the physical-order vector; returns a new array."""
    out = np.ascontiguousarray(x_phys, dtype=np.float64).copy()
    n = out.shape[0]
    values = sell["values"] if sell["values"].size else np.zeros(1)
    column = sell["column"] if sell["column"].size else np.zeros(1, dtype=np.int32)
    rc = lib().lgd_oracle_sell_diffusion(n, C, _ptr(sell["chunk_offset"]), _ptr(sell["row_length"]),
                                         _ptr(values), _ptr(column), int(steps), _ptr(out), threads)
    assert rc == 0
    return out


def lbm(L: int, steps: int, omega: float, lid: float, f: np.ndarray | None = None, threads: int = 0) -> np.ndarray:
    """D3Q19 cavity; f is (19, L, L, L) FP64, default equilibrium at rest."""
    if f is None:
        f = lbm_rest(L)
    out = np.ascontiguousarray(f, dtype=np.float64).copy()
    assert lib().lgd_oracle_lbm(L, int(steps), float(omega), float(lid), _ptr(out), threads) == 0
    return out


def lbm_rest(L: int) -> np.ndarray:
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, dtype=np.float64)
    return np.ascontiguousarray(np.broadcast_to(w[:, None, None, None], (19, L, L, L)))


def varcoef(u: np.ndarray, k: np.ndarray, steps: int, threads: int = 0) -> np.ndarray:
    out = np.ascontiguousarray(u, dtype=np.float64).copy()
    kk = np.ascontiguousarray(k, dtype=np.float64)
    nz, ny, nx = out.shape
    assert lib().lgd_oracle_varcoef(nx, ny, nz, int(steps), _ptr(out), _ptr(kk), threads) == 0
    return out
