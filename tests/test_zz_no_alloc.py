"""lgd_sum_f64_static: the allocation-free variant of the grid checksum.

It is meant for callers that cannot allocate device memory themselves or
through the library - plugins and solvers running inside another
framework's stream and memory pool, where cudaMalloc would synchronise the
device - so it keeps its partial sums in a fixed device array.  This test
calls it through the C ABI twice in a row, on two different grids (the
second smaller, so stale partials from the first call would show), and
checks each result against lgd_gpu_checksum on the same grid within the
1e-12 relative tolerance the FP64 tests use.  It also checks the size limit.
"""
import ctypes

import numpy as np
import pytest

from libgeodecomp_gb300 import lgd

pytestmark = pytest.mark.gpu


def _bind():
    fn = lgd.lib().lgd_sum_f64_static
    fn.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _stream(grid):
    p = ctypes.c_void_p()
    lgd.check(lgd.lib().lgd_gpu_stream(grid._h, ctypes.byref(p)))
    return p


def _static_sum(fn, grid, out_grid):
    """Sum of grid's current buffer via the allocation-free entry point; the
    result goes to element 0 of out_grid's device buffer."""
    d_in, pitch = grid.device_ptr(0, 0)
    # The library pitches rows to 128 bytes; the grids here have rows of a
    # multiple of 16 FP64 cells (16 * 8 = 128 bytes), so their rows are dense
    # and the buffer is one flat array of the grid's values.
    assert pitch == grid.shape[-1] * 8
    d_out, _ = out_grid.device_ptr(0, 0)
    lgd.check(fn(d_in, grid.cells, d_out, _stream(grid)))
    grid.synchronize()
    return float(out_grid.download(0).reshape(-1)[0])


def test_static_sum_matches_checksum_on_two_calls_in_a_row():
    fn = _bind()
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (40, 64, 48)) as a, \
            lgd.Grid(lgd.CELL_JACOBI7_F64, (3, 5, 16)) as b, \
            lgd.Grid(lgd.CELL_JACOBI7_F64, (1, 1, 16)) as out:
        a.fill_uniform(0, seed=11, stream=1)
        b.fill_uniform(0, seed=12, stream=1)
        for grid in (a, b):
            expected = grid.checksum(0)
            got = _static_sum(fn, grid, out)
            assert abs(got - expected) <= 1e-12 * abs(expected), (got, expected)


def test_static_sum_limits():
    fn = _bind()
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (1, 1, 16)) as out:
        d_out, _ = out.device_ptr(0, 0)
        out.upload(0, np.full((1, 1, 16), 5.0))
        # too many values for the fixed scratch: rejected before any launch
        rc = fn(d_out, (1 << 30) + 1, d_out, None)
        assert rc == lgd.ERR_RANGE
        # no values: the sum is 0
        lgd.check(fn(None, 0, d_out, _stream(out)))
        out.synchronize()
        assert out.download(0).reshape(-1)[0] == 0.0
