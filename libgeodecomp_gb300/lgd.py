"""ctypes binding of the C ABI in include/lgd_gpu.h.

Used by the tests and the benchmark.  Loading fails loudly when the CUDA
library has not been built: there is no CPU fallback anywhere on this path.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblgd_gb300.so")

OK = 0
ERR_INVALID = 1
ERR_RANGE = 2
ERR_CUDA = 3
ERR_NOMEM = 4
ERR_TIMEOUT = 5
ERR_UNSUPPORTED = 6
TB_MAX_DEPTH = 32       # LGD_TB_MAX_DEPTH

CELL_JACOBI7_F64 = 1
CELL_JACOBI7_F64_FIX = 2
CELL_JACOBI7_F32 = 3
CELL_SUM6_F64 = 4
CELL_GOL_U8 = 5
CELL_VARCOEF_F32 = 6
CELL_VARCOEF_F64 = 7
CELL_TEST = 8
CELL_RECORD = 9
RECORD_MAX_BYTES = 4096
TEST_VON_NEUMANN = 1


def TEST_NANO_STEPS(n: int) -> int:
    return n << 8


# lgd_test_record (include/lgd_gpu.h), 64 bytes
TEST_RECORD = np.dtype([("pos", "<i4", 3), ("dim", "<i4", 3), ("cycle", "<u4"), ("edge", "u1"), ("valid", "u1"),
                        ("pad0", "u1"), ("pad1", "u1"), ("test_value", "<f4"), ("pad", "<i4", 7)])
assert TEST_RECORD.itemsize == 64

# host dtype of each member, per cell kind
MEMBERS = {
    CELL_JACOBI7_F64: [np.float64],
    CELL_JACOBI7_F64_FIX: [np.float64],
    CELL_JACOBI7_F32: [np.float32],
    CELL_SUM6_F64: [np.float64, np.float64],
    CELL_GOL_U8: [np.uint8],
    CELL_VARCOEF_F32: [np.float32, np.float32],
    CELL_VARCOEF_F64: [np.float64, np.float64],
    CELL_TEST: [TEST_RECORD],
}


class LGDError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("lgd error %d: %s" % (code, msg))
        self.code = code


class GridDesc(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("periodic", ctypes.c_int), ("cell", ctypes.c_int), ("flags", ctypes.c_int),
                ("edge", ctypes.c_double * 4)]


_lib = None


def lib():
    """The loaded library; raises if it is missing (build it with
    ``python -c "import __graft_entry__ as g; g.build()"``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("CUDA library %s is not built" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int
        S = ctypes.c_size_t
        U64 = ctypes.c_uint64
        for name, args in {
            "lgd_gpu_last_error": [ctypes.c_char_p, S],
            "lgd_gpu_version": [],
            "lgd_gpu_device_count": [P],
            "lgd_gpu_create": [P, P],
            "lgd_gpu_destroy": [P],
            "lgd_gpu_upload": [P, I, I, P, S],
            "lgd_gpu_download": [P, I, I, P, S],
            "lgd_gpu_save_region": [P, I, P, I, P, S],
            "lgd_gpu_load_region": [P, I, P, I, P, S],
            "lgd_gpu_step": [P, ctypes.c_uint, I],
            "lgd_gpu_update_region": [P, P, I, ctypes.c_uint],
            "lgd_gpu_swap": [P],
            "lgd_gpu_fill_uniform": [P, I, I, U64, I],
            "lgd_gpu_fill_bernoulli": [P, I, I, U64, I, ctypes.c_double],
            "lgd_gpu_fixed_point_exponent": [P, P],
            "lgd_gpu_checksum": [P, I, I, P],
            "lgd_gpu_synchronize": [P],
            "lgd_gpu_device_ptr": [P, I, I, P, P],
            "lgd_gpu_launch_count": [P, P],
            "lgd_gpu_set_time_block": [P, I],
            "lgd_gpu_set_time_block_shape": [P, I],
            "lgd_gpu_write_bov": [P, I, ctypes.c_char_p, ctypes.c_uint, ctypes.c_char_p],
            "lgd_gpu_write_snapshot": [P, ctypes.c_char_p, ctypes.c_uint, ctypes.c_uint],
            "lgd_gpu_read_snapshot": [P, ctypes.c_char_p, P, P],
            "lgd_snapshot_info": [ctypes.c_char_p, I, P, P, P],
            "lgd_gpu_set_variant": [P, I],
            "lgd_gpu_stream": [P, P],
            "lgd_gpu_create_records": [P, S, P, P],
            "lgd_gpu_set_edge_record": [P, P, S],
            "lgd_gpu_edge_record_device": [P, P],
            "lgd_gpu_get_desc": [P, P],
            "lgd_gpu_count_launches": [P, U64],
            "lgd_gpu_set_fixed_point_exponent": [P, I, I],
            "lgd_gpu_plane_bytes": [P, I, P],
            "lgd_gpu_copy_planes": [P, I, I, I, I, P, S, I],
            "lgd_gpu_test_bounded_waits": [P, ctypes.c_longlong, I],
            "lgd_sell_plan": [I, P, I, I, P, P, P, P, P],
            "lgd_sell_fill": [I, P, P, P, I, P, P, ctypes.c_int64, I, P, P],
            "lgd_sell_create": [I, I, ctypes.c_int64, P, P, P, P, P, I, I, P],
            "lgd_sell_destroy": [P],
            "lgd_sell_upload_x": [P, I, I, P, S],
            "lgd_sell_download_x": [P, I, I, P, S],
            "lgd_sell_step": [P, I],
            "lgd_sell_update_rows": [P, I, I],
            "lgd_sell_swap": [P],
            "lgd_sell_x_device": [P, I, P, P],
            "lgd_graph_rcm": [I, P, P, P],
            "lgd_sell_synchronize": [P],
            "lgd_sell_stream": [P, P],
            "lgd_sell_launch_count": [P, P],
            "lgd_sell_set_variant": [P, I],
            "lgd_sell_create_from_csr": [I, P, P, P, I, I, I, I, I, P],
            "lgd_sell_get_layout": [P, P, P, P, P, P, P],
            "lgd_lbm_create": [I, P, P, ctypes.c_double, I, P],
            "lgd_lbm_destroy": [P],
            "lgd_lbm_step": [P, I],
            "lgd_lbm_step_looped": [P, I],
            "lgd_lbm_set_config": [P, I, I, I],
            "lgd_lbm_get_config": [P, P, P, P],
            "lgd_lbm_tune": [P, I, P, P, P, P],
            "lgd_lbm_reset": [P],
            "lgd_lbm_download": [P, I, P, S],
            "lgd_lbm_upload": [P, I, P, S],
            "lgd_lbm_info": [P, P, P],
            "lgd_lbm_synchronize": [P],
            "lgd_lbm_stream": [P, P],
            "lgd_lbm_launch_count": [P, P],
            "lgd_lbm_set_variant": [P, I],
            "lgd_lbm_set_time_block": [P, I, I, I],
            "lgd_lbm_get_time_block": [P, P, P, P],
        }.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = I
        _lib = L
    return _lib


def check(rc: int):
    if rc != OK:
        buf = ctypes.create_string_buffer(512)
        lib().lgd_gpu_last_error(buf, 512)
        raise LGDError(rc, buf.value.decode(errors="replace"))


def device_count() -> int:
    n = ctypes.c_int(0)
    check(lib().lgd_gpu_device_count(ctypes.byref(n)))
    return n.value


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


class Grid:
    """One structured device grid (a handle of the C ABI)."""

    def __init__(self, cell: int, shape, periodic: int = 0, edge=(0.0, 0.0, 0.0, 0.0), flags: int = 0):
        shape = tuple(int(s) for s in shape)
        if len(shape) == 1:
            (nx,) = shape
            ny, nz, dim = 1, 1, 1
        elif len(shape) == 2:
            ny, nx = shape
            nz, dim = 1, 2
        else:
            nz, ny, nx = shape
            dim = 3
        d = GridDesc()
        d.dim, d.nx, d.ny, d.nz = dim, nx, ny, nz
        d.periodic, d.cell, d.flags = periodic, cell, flags
        for i, e in enumerate(list(edge)[:4]):
            d.edge[i] = float(e)
        self.cell = cell
        self.shape = shape
        self.cells = nx * ny * nz
        self.members = MEMBERS.get(cell, [])
        self._h = ctypes.c_void_p()
        check(lib().lgd_gpu_create(ctypes.byref(d), ctypes.byref(self._h)))

    def close(self):
        if self._h:
            check(lib().lgd_gpu_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def upload(self, member: int, values: np.ndarray, which: int = 0):
        a = np.ascontiguousarray(values, dtype=self.members[member])
        assert a.size == self.cells
        check(lib().lgd_gpu_upload(self._h, member, which, _ptr(a), a.nbytes))

    def download(self, member: int = 0, which: int = 0, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.shape, dtype=self.members[member])
        check(lib().lgd_gpu_download(self._h, member, which, _ptr(out), out.nbytes))
        return out

    def step(self, count: int = 1, nano_step: int = 0):
        check(lib().lgd_gpu_step(self._h, nano_step, count))

    def update_region(self, streaks, nano_step: int = 0):
        s = np.ascontiguousarray(np.asarray(streaks, dtype=np.int32).reshape(-1, 4))
        check(lib().lgd_gpu_update_region(self._h, _ptr(s), s.shape[0], nano_step))

    def swap(self):
        check(lib().lgd_gpu_swap(self._h))

    def save_region(self, member: int, streaks) -> np.ndarray:
        s = np.ascontiguousarray(np.asarray(streaks, dtype=np.int32).reshape(-1, 4))
        n = int((s[:, 3] - s[:, 0]).sum())
        out = np.empty(n, dtype=self.members[member])
        check(lib().lgd_gpu_save_region(self._h, member, _ptr(s), s.shape[0], _ptr(out), out.nbytes))
        return out

    def load_region(self, member: int, streaks, values: np.ndarray):
        s = np.ascontiguousarray(np.asarray(streaks, dtype=np.int32).reshape(-1, 4))
        v = np.ascontiguousarray(values, dtype=self.members[member])
        check(lib().lgd_gpu_load_region(self._h, member, _ptr(s), s.shape[0], _ptr(v), v.nbytes))

    def fill_uniform(self, member: int = 0, seed: int = 42, stream: int = 1, which: int = 0):
        check(lib().lgd_gpu_fill_uniform(self._h, member, which, seed, stream))

    def fill_bernoulli(self, p: float, member: int = 0, seed: int = 42, stream: int = 1, which: int = 0):
        check(lib().lgd_gpu_fill_bernoulli(self._h, member, which, seed, stream, p))

    def checksum(self, member: int = 0, which: int = 0) -> float:
        s = ctypes.c_double()
        check(lib().lgd_gpu_checksum(self._h, member, which, ctypes.byref(s)))
        return s.value

    def synchronize(self):
        check(lib().lgd_gpu_synchronize(self._h))

    def stream(self) -> int:
        """The handle's CUDA stream (a cudaStream_t) as an integer."""
        p = ctypes.c_void_p()
        check(lib().lgd_gpu_stream(self._h, ctypes.byref(p)))
        return p.value

    def device_ptr(self, member: int = 0, which: int = 0):
        p = ctypes.c_void_p()
        pitch = ctypes.c_size_t()
        check(lib().lgd_gpu_device_ptr(self._h, member, which, ctypes.byref(p), ctypes.byref(pitch)))
        return p.value, pitch.value

    def launch_count(self) -> int:
        n = ctypes.c_uint64()
        check(lib().lgd_gpu_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def set_time_block(self, depth: int):
        check(lib().lgd_gpu_set_time_block(self._h, depth))

    def write_bov(self, prefix: str, step: int, member: int = 0, variable: str = "var"):
        """BOV snapshot of one member straight from the device (prefix.<step>.bov / .data)."""
        check(lib().lgd_gpu_write_bov(self._h, member, prefix.encode(), step, variable.encode()))

    def write_snapshot(self, path: str, step: int, max_steps: int):
        """Checkpoint of the current grid in the reference's MPIIO layout."""
        check(lib().lgd_gpu_write_snapshot(self._h, path.encode(), step, max_steps))

    def read_snapshot(self, path: str):
        """Loads a checkpoint into the current grid; returns (step, max_steps)."""
        step = ctypes.c_uint()
        max_steps = ctypes.c_uint()
        check(lib().lgd_gpu_read_snapshot(self._h, path.encode(), ctypes.byref(step), ctypes.byref(max_steps)))
        return step.value, max_steps.value

    def set_time_block_shape(self, shape: int):
        check(lib().lgd_gpu_set_time_block_shape(self._h, shape))

    def set_variant(self, variant: int):
        """Kernel variant of cells that have several (identical results)."""
        check(lib().lgd_gpu_set_variant(self._h, variant))

    def fixed_point_exponent(self) -> int:
        e = ctypes.c_int()
        check(lib().lgd_gpu_fixed_point_exponent(self._h, ctypes.byref(e)))
        return e.value

    def set_fixed_point_exponent(self, e: int, pin: bool = True):
        check(lib().lgd_gpu_set_fixed_point_exponent(self._h, e, int(pin)))

    def plane_bytes(self, member: int = 0) -> int:
        n = ctypes.c_size_t()
        check(lib().lgd_gpu_plane_bytes(self._h, member, ctypes.byref(n)))
        return n.value

    def save_planes(self, p0: int, n: int, member: int = 0, which: int = 0, out: np.ndarray | None = None):
        """Raw planes p0 .. p0 + n - 1 of the slowest axis (device representation,
        row padding included) into a host byte array."""
        nbytes = n * self.plane_bytes(member)
        if out is None:
            out = np.empty(nbytes, dtype=np.uint8)
        assert out.nbytes == nbytes and out.flags["C_CONTIGUOUS"]
        check(lib().lgd_gpu_copy_planes(self._h, member, which, p0, n, _ptr(out), nbytes, 0))
        return out

    def load_planes(self, p0: int, data: np.ndarray, member: int = 0, which: int = 0):
        a = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
        pb = self.plane_bytes(member)
        assert a.nbytes % pb == 0
        check(lib().lgd_gpu_copy_planes(self._h, member, which, p0, a.nbytes // pb, _ptr(a), a.nbytes, 1))

    def copy_planes_device(self, p0: int, n: int, dev_ptr: int, to_grid: bool, member: int = 0, which: int = 0):
        """Raw planes to or from device memory at dev_ptr (n * plane_bytes)."""
        nbytes = n * self.plane_bytes(member)
        check(lib().lgd_gpu_copy_planes(self._h, member, which, p0, n, ctypes.c_void_p(dev_ptr), nbytes,
                                        int(to_grid)))


# ----------------------------------------------------------- SELL-C-sigma
SELL_EXACT = 1
SELL_RENUMBER = 2


def snapshot_info(path: str, dim: int = 3):
    """(dims (x, y[, z]), step, max_steps) of a checkpoint file."""
    dims = (ctypes.c_int * dim)()
    step = ctypes.c_uint()
    max_steps = ctypes.c_uint()
    check(lib().lgd_snapshot_info(path.encode(), dim, dims, ctypes.byref(step), ctypes.byref(max_steps)))
    return tuple(dims), step.value, max_steps.value


def sell_build(n: int, row_ptr, col, w, C: int, sigma: int, remap_columns: bool = True) -> dict:
    """SELL-C-sigma arrays from a logical CSR matrix (host-side builder of
    the library; the layout is the reference's)."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    w = np.ascontiguousarray(w, dtype=np.float64)
    n_chunks = (n - 1) // C + 1
    perm = np.zeros(n, dtype=np.int32)
    row_length = np.zeros(n_chunks * C, dtype=np.int32)
    chunk_length = np.zeros(n_chunks, dtype=np.int32)
    chunk_offset = np.zeros(n_chunks + 1, dtype=np.int32)
    total = ctypes.c_int64()
    check(lib().lgd_sell_plan(n, _ptr(row_ptr), C, sigma, _ptr(perm), _ptr(row_length), _ptr(chunk_length),
                              _ptr(chunk_offset), ctypes.byref(total)))
    t = total.value
    values = np.zeros(max(t, 1), dtype=np.float64)
    column = np.zeros(max(t, 1), dtype=np.int32)
    check(lib().lgd_sell_fill(n, _ptr(row_ptr), _ptr(col if col.size else np.zeros(1, np.int32)),
                              _ptr(w if w.size else np.zeros(1)), C, _ptr(perm), _ptr(chunk_offset), t,
                              int(remap_columns), _ptr(values), _ptr(column)))
    return dict(perm=perm, row_length=row_length, chunk_length=chunk_length, chunk_offset=chunk_offset,
                values=values[:t], column=column[:t], C=C, sigma=sigma, n=n)


SELL_GPU_MAX_SIGMA = 4096     # LGD_SELL_GPU_MAX_SIGMA
SELL_GPU_MAX_ROW = 1024       # LGD_SELL_GPU_MAX_ROW


def graph_rcm(n: int, row_ptr, col) -> np.ndarray:
    """Reverse Cuthill-McKee order of a CSR graph (lgd_graph_rcm, host
    code): order[k] = the node numbered k."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cc = np.ascontiguousarray(col, dtype=np.int32)
    out = np.empty(n, dtype=np.int32)
    check(lib().lgd_graph_rcm(n, _ptr(rp), _ptr(cc) if cc.size else None, _ptr(out)))
    return out


class SellGrid:
    """Device SELL-C-sigma grid running the diffusion cell."""

    @classmethod
    def from_csr(cls, n: int, row_ptr, col, w, C: int, sigma: int, precision: int = 8, exact: bool = False,
                 device: bool = False, renumber: bool = False):
        """Builds the matrix on the GPU (lgd_sell_create_from_csr).  With
        device=True the CSR arrays are torch CUDA tensors (int64, int32,
        float64), else numpy arrays.  renumber=True numbers the nodes in
        reverse Cuthill-McKee order first (host arrays; logical order
        unchanged; each row's terms are added in another order, so values
        agree with the plain grid's to rounding)."""
        self = cls.__new__(cls)
        self.n = n
        if device:
            self._keep = [row_ptr, col, w]
            ptrs = [ctypes.c_void_p(t.data_ptr()) for t in self._keep]
        else:
            self._keep = [np.ascontiguousarray(row_ptr, dtype=np.int64), np.ascontiguousarray(col, dtype=np.int32),
                          np.ascontiguousarray(w, dtype=np.float64)]
            ptrs = [_ptr(a) if a.size else ctypes.c_void_p() for a in self._keep]
        self._h = ctypes.c_void_p()
        self._C = C
        flags = (SELL_EXACT if exact else 0) | (SELL_RENUMBER if renumber else 0)
        check(lib().lgd_sell_create_from_csr(n, ptrs[0], ptrs[1], ptrs[2], C, sigma, int(device), precision,
                                             flags, ctypes.byref(self._h)))
        return self

    def layout(self) -> dict:
        """The device matrix as host arrays (chunk_offset, row_length,
        values as FP64, column, perm)."""
        total = ctypes.c_int64()
        check(lib().lgd_sell_get_layout(self._h, None, None, None, None, None, ctypes.byref(total)))
        t = total.value
        C = self.C_of()
        n_chunks = (self.n - 1) // C + 1
        co = np.zeros(n_chunks + 1, dtype=np.int32)
        rl = np.zeros(n_chunks * C, dtype=np.int32)
        vals = np.zeros(max(t, 1), dtype=np.float64)
        cols = np.zeros(max(t, 1), dtype=np.int32)
        perm = np.zeros(self.n, dtype=np.int32)
        check(lib().lgd_sell_get_layout(self._h, _ptr(co), _ptr(rl), _ptr(vals), _ptr(cols), _ptr(perm),
                                        ctypes.byref(total)))
        return dict(chunk_offset=co, row_length=rl, values=vals[:t], column=cols[:t], perm=perm)

    def C_of(self) -> int:
        return self._C

    def __init__(self, sell: dict, precision: int = 8, exact: bool = False):
        self.n = sell["n"]
        self._C = sell["C"]
        self._keep = [np.ascontiguousarray(sell[k]) for k in ("chunk_offset", "row_length", "values", "column", "perm")]
        co, rl, vals, cols, perm = self._keep
        if vals.size == 0:
            vals = np.zeros(1)
            cols = np.zeros(1, dtype=np.int32)
        self._h = ctypes.c_void_p()
        check(lib().lgd_sell_create(self.n, sell["C"], int(sell["values"].size), _ptr(co), _ptr(rl), _ptr(vals),
                                    _ptr(cols), _ptr(perm), precision, SELL_EXACT if exact else 0,
                                    ctypes.byref(self._h)))

    def close(self):
        if self._h:
            check(lib().lgd_sell_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def upload(self, x: np.ndarray, logical: bool = True, which: int = 0):
        a = np.ascontiguousarray(x, dtype=np.float64)
        assert a.size == self.n
        check(lib().lgd_sell_upload_x(self._h, which, int(logical), _ptr(a), a.nbytes))

    def download(self, logical: bool = True, which: int = 0, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.n, dtype=np.float64)
        check(lib().lgd_sell_download_x(self._h, which, int(logical), _ptr(out), out.nbytes))
        return out

    def step(self, count: int = 1):
        check(lib().lgd_sell_step(self._h, count))

    def update_rows(self, begin: int, end: int):
        check(lib().lgd_sell_update_rows(self._h, begin, end))

    def swap(self):
        check(lib().lgd_sell_swap(self._h))

    def x_device(self, which: int = 0):
        """(device address, rows_padded) of node-value buffer which (physical
        order, the handle's precision)."""
        p, n = ctypes.c_void_p(), ctypes.c_int64()
        check(lib().lgd_sell_x_device(self._h, which, ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    def synchronize(self):
        check(lib().lgd_sell_synchronize(self._h))

    def stream(self) -> int:
        p = ctypes.c_void_p()
        check(lib().lgd_sell_stream(self._h, ctypes.byref(p)))
        return p.value

    def launch_count(self) -> int:
        n = ctypes.c_uint64()
        check(lib().lgd_sell_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def set_variant(self, variant: int):
        """Kernel variant (identical results): 0 pipelined, 1 unpipelined, 2 pipelined depth 2."""
        check(lib().lgd_sell_set_variant(self._h, variant))


# ------------------------------------------------------------ LBM ensemble
class LbmEnsemble:
    """Ensemble of D3Q19 lid-driven cavities (include/lgd_ensemble.h)."""

    def __init__(self, edges, omegas, lid: float = 0.05, precision: int = 4):
        self.edges = np.ascontiguousarray(edges, dtype=np.int32)
        self.omegas = np.ascontiguousarray(omegas, dtype=np.float64)
        self._h = ctypes.c_void_p()
        check(lib().lgd_lbm_create(len(self.edges), _ptr(self.edges), _ptr(self.omegas), float(lid), precision,
                                   ctypes.byref(self._h)))

    def close(self):
        if self._h:
            check(lib().lgd_lbm_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def step(self, steps: int = 1):
        check(lib().lgd_lbm_step(self._h, steps))

    def step_looped(self, steps: int = 1):
        check(lib().lgd_lbm_step_looped(self._h, steps))

    def set_config(self, tile_rows: int, threads: int, ctas_per_sm: int):
        check(lib().lgd_lbm_set_config(self._h, tile_rows, threads, ctas_per_sm))

    def config(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().lgd_lbm_get_config(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def tune(self, trial_steps: int = 4):
        a, b, c, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        check(lib().lgd_lbm_tune(self._h, trial_steps, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                 ctypes.byref(t)))
        return (a.value, b.value, c.value), t.value

    def reset(self):
        check(lib().lgd_lbm_reset(self._h))

    def download(self, instance: int) -> np.ndarray:
        L = int(self.edges[instance])
        out = np.empty((19, L, L, L), dtype=np.float64)
        check(lib().lgd_lbm_download(self._h, instance, _ptr(out), out.nbytes))
        return out

    def upload(self, instance: int, f: np.ndarray):
        a = np.ascontiguousarray(f, dtype=np.float64)
        check(lib().lgd_lbm_upload(self._h, instance, _ptr(a), a.nbytes))

    def info(self):
        c, n = ctypes.c_longlong(), ctypes.c_int()
        check(lib().lgd_lbm_info(self._h, ctypes.byref(c), ctypes.byref(n)))
        return c.value, n.value

    def synchronize(self):
        check(lib().lgd_lbm_synchronize(self._h))

    def stream(self) -> int:
        p = ctypes.c_void_p()
        check(lib().lgd_lbm_stream(self._h, ctypes.byref(p)))
        return p.value

    def launch_count(self) -> int:
        n = ctypes.c_uint64()
        check(lib().lgd_lbm_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def set_variant(self, variant: int):
        """Memory path (identical results): 0 plain, 1 read-only loads + evict-first stores."""
        check(lib().lgd_lbm_set_variant(self._h, variant))

    def set_time_block(self, depth: int, shape: int = 0, ctas_per_sm: int = 1):
        """Steps per launch (1 or 2), the two-step kernel's tile shape and residency."""
        check(lib().lgd_lbm_set_time_block(self._h, depth, shape, ctas_per_sm))

    def time_block(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().lgd_lbm_get_time_block(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value
