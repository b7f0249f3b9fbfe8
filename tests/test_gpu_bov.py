"""BOV snapshots written straight from the device (lgd_gpu_write_bov) are
byte-identical to the reference's SerialBOVWriter on the same cell and
input: header and data at the initial step and after 6 Jacobi steps
(fixture written by the reference through tests/golden/gen_golden.py)."""
import os

import numpy as np
import pytest

from libgeodecomp_gb300 import lgd, workloads

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def read(path):
    with open(path, "rb") as f:
        return f.read()


def test_bov_snapshots_byte_identical_to_reference(tmp_path, monkeypatch):
    g = np.load(os.path.join(GOLD, "bov_jacobi_24x20x16.npz"))
    nz, ny, nx = (int(v) for v in g["shape"])
    steps = int(g["steps"])
    u0 = workloads.jacobi_initial(nx, ny, nz, seed=42)
    monkeypatch.chdir(tmp_path)           # the header records DATA_FILE relative to the prefix
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (nz, ny, nx)) as grid:
        grid.upload(0, u0)
        grid.write_bov("jac", 0, variable="temp")
        grid.step(steps)
        grid.write_bov("jac", steps, variable="temp")
    for step in (0, steps):
        stem = "jac.%05d" % step
        assert read(stem + ".bov") == bytes(g["bov_%d" % step]), stem
        assert read(stem + ".data") == bytes(g["data_%d" % step]), stem


@pytest.mark.parametrize("cell,fmt,size", [(lgd.CELL_JACOBI7_F32, b"FLOAT", 4), (lgd.CELL_GOL_U8, b"BYTE", 1),
                                           (lgd.CELL_JACOBI7_F64_FIX, b"DOUBLE", 8)])
def test_bov_formats_and_2d_grids(tmp_path, cell, fmt, size):
    shape = (33, 70) if cell == lgd.CELL_GOL_U8 else (5, 9, 17)
    with lgd.Grid(cell, shape, periodic=3 if cell == lgd.CELL_GOL_U8 else 0) as grid:
        if cell == lgd.CELL_GOL_U8:
            grid.fill_bernoulli(0.3, seed=2)
        else:
            grid.fill_uniform(0, seed=2)
        grid.step(3)
        expect = grid.download(0)
        prefix = str(tmp_path / "snap")
        grid.write_bov(prefix, 3, variable="v")
    header = read(prefix + ".00003.bov")
    dims = (b"%d %d 1" % (shape[1], shape[0])) if len(shape) == 2 else (b"%d %d %d" % (shape[2], shape[1], shape[0]))
    assert b"DATA_FORMAT: " + fmt + b"\n" in header
    assert b"DATA_SIZE: " + dims + b"\n" in header
    assert read(prefix + ".00003.data") == np.ascontiguousarray(expect).tobytes()
    assert len(read(prefix + ".00003.data")) == expect.size * size


def test_bov_reports_unwritable_path():
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (4, 4, 4)) as grid:
        with pytest.raises(lgd.LGDError) as e:
            grid.write_bov("/nonexistent-directory/x", 0)
        assert e.value.code == lgd.ERR_INVALID
