"""Checkpoint snapshots (lgd_gpu_write_snapshot / lgd_gpu_read_snapshot) in
the file layout of the reference's MPIIOWriter / MPIIOInitializer
(io/mpiio.h:85-125 writeRegion, :180-200 offset and getLengths): the
dimensions as DIM int32, the step and maximum as uint32, the edge cell,
then the cells x fastest, each a record of the grid's members.  The
reference's MPI-IO path needs MPI, which this image lacks, so the layout is
restated here (`parse`) and the files are checked against it and against a
restart: a grid loaded from the snapshot of step k and advanced to step n
equals the grid advanced without interruption."""
import struct

import numpy as np
import pytest

from libgeodecomp_gb300 import lgd, workloads

pytestmark = pytest.mark.gpu


def parse(path, dim, member_types):
    """The reference's MPIIO layout (io/mpiio.h): header, edge cell, cells."""
    raw = open(path, "rb").read()
    dims = struct.unpack_from("<%di" % dim, raw, 0)
    step, max_steps = struct.unpack_from("<2I", raw, 4 * dim)
    rec = np.dtype([("m%d" % i, t) for i, t in enumerate(member_types)])
    edge = np.frombuffer(raw, dtype=rec, count=1, offset=4 * dim + 8)[0]
    n = int(np.prod(dims))
    cells = np.frombuffer(raw, dtype=rec, count=n, offset=4 * dim + 8 + rec.itemsize)
    assert len(raw) == 4 * dim + 8 + rec.itemsize * (n + 1)
    return dims, step, max_steps, edge, cells


CASES = [
    # cell, shape (z, y, x) or (y, x), member dtypes, periodic, edge
    (lgd.CELL_JACOBI7_F64, (7, 9, 12), ["<f8"], 0, 0.25),
    (lgd.CELL_JACOBI7_F32, (6, 10, 33), ["<f4"], 0, 0.0),
    (lgd.CELL_GOL_U8, (40, 64), ["u1"], 3, 0.0),
    (lgd.CELL_VARCOEF_F64, (5, 8, 16), ["<f8", "<f8"], 7, 0.0),
]


def make_grid(cell, shape, periodic, edge, seed):
    g = lgd.Grid(cell, shape, periodic=periodic, edge=(edge,))
    rng = np.random.default_rng(seed)
    if cell == lgd.CELL_GOL_U8:
        g.upload(0, (rng.random(shape) < 0.3).astype(np.uint8))
    elif cell == lgd.CELL_VARCOEF_F64:
        g.upload(0, rng.random(shape))
        g.upload(1, 0.02 + 0.13 * rng.random(shape))
    elif cell == lgd.CELL_JACOBI7_F32:
        g.upload(0, rng.random(shape).astype(np.float32))
    else:
        g.upload(0, rng.random(shape))
    return g


@pytest.mark.parametrize("cell,shape,types,periodic,edge", CASES)
def test_snapshot_layout_matches_the_reference_format(tmp_path, cell, shape, types, periodic, edge):
    path = str(tmp_path / "snap00005.mpiio")
    with make_grid(cell, shape, periodic, edge, 5) as g:
        g.step(5)
        g.write_snapshot(path, 5, 21)
        want = [g.download(m) for m in range(len(types))]
    dims, step, max_steps, e, cells = parse(path, len(shape), types)
    assert dims == tuple(reversed(shape))
    assert (step, max_steps) == (5, 21)
    for m in range(len(types)):
        assert e["m%d" % m] == np.array(edge if m == 0 else 0.0).astype(types[m])
        np.testing.assert_array_equal(cells["m%d" % m].reshape(shape), want[m])
    assert lgd.snapshot_info(path, len(shape)) == (tuple(reversed(shape)), 5, 21)


@pytest.mark.parametrize("cell,shape,types,periodic,edge", CASES)
def test_restart_from_snapshot_equals_uninterrupted_run(tmp_path, cell, shape, types, periodic, edge):
    path = str(tmp_path / "snap00004.mpiio")
    with make_grid(cell, shape, periodic, edge, 7) as a:
        a.step(4)
        a.write_snapshot(path, 4, 10)
        a.step(6)
        want = [a.download(m) for m in range(len(types))]
    with lgd.Grid(cell, shape, periodic=periodic, edge=(edge,)) as b:
        assert b.read_snapshot(path) == (4, 10)
        b.step(6)
        for m in range(len(types)):
            np.testing.assert_array_equal(b.download(m), want[m])


def test_fixed_point_grid_restarts_within_tolerance(tmp_path):
    """The fixed-point grid writes FP64 values (56-bit integers rounded to
    53 bits), so its restart agrees within the cell's 1e-12 bound."""
    path = str(tmp_path / "fix00010.mpiio")
    u0 = workloads.jacobi_initial(40, 24, 20, seed=3)
    with lgd.Grid(lgd.CELL_JACOBI7_F64_FIX, u0.shape) as a:
        a.upload(0, u0)
        a.step(10)
        a.write_snapshot(path, 10, 30)
        mid = a.download(0)
        a.step(20)
        want = a.download(0)
    _, step, max_steps, _, cells = parse(path, 3, ["<f8"])
    np.testing.assert_array_equal(cells["m0"].reshape(u0.shape), mid)
    with lgd.Grid(lgd.CELL_JACOBI7_F64_FIX, u0.shape) as b:
        assert b.read_snapshot(path) == (10, 30)
        b.step(20)
        got = b.download(0)
    assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-300)) <= 1e-12


def test_snapshot_mismatches_are_rejected(tmp_path):
    path = str(tmp_path / "s00000.mpiio")
    with make_grid(lgd.CELL_JACOBI7_F64, (7, 9, 12), 0, 0.25, 1) as g:
        g.write_snapshot(path, 0, 3)
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (7, 9, 11), edge=(0.25,)) as g:        # other dimensions
        with pytest.raises(lgd.LGDError) as e:
            g.read_snapshot(path)
        assert e.value.code == lgd.ERR_INVALID
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (7, 9, 12), edge=(0.5,)) as g:         # other edge cell
        with pytest.raises(lgd.LGDError) as e:
            g.read_snapshot(path)
        assert e.value.code == lgd.ERR_INVALID
    short = str(tmp_path / "short.mpiio")
    with open(path, "rb") as f, open(short, "wb") as o:
        o.write(f.read()[:-8])
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (7, 9, 12), edge=(0.25,)) as g:        # one cell missing
        with pytest.raises(lgd.LGDError) as e:
            g.read_snapshot(short)
        assert e.value.code == lgd.ERR_INVALID
    with pytest.raises(lgd.LGDError):
        lgd.snapshot_info(str(tmp_path / "missing.mpiio"))
