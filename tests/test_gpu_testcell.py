"""The self-validating test cell (LGD_CELL_TEST, the reference's TestCell,
misc/testcell.h:205-372) through the C ABI: grids initialised as the
reference's TestInitializer does (io/testinitializer.h:27-41) stay valid
and count one cycle per nano step in 1D, 2D and 3D, cube and torus, Moore
and von Neumann; a wrong nano step, a cell that claims a wrong position and
a bad edge cell are caught by the cells themselves.  The C++ drop-in runs
the reference's CUDASimulator conformance cases on the same cell
(tests/cpp/gb300simulator_test.cpp, testTestCellConformance)."""
import numpy as np
import pytest

from libgeodecomp_gb300 import lgd

pytestmark = pytest.mark.gpu


def initial(shape, nano_steps, start_step=0):
    """TestInitializer: every cell at its own position, cycle = start *
    nano steps, test value 1 + index; shape is (z, y, x) / (y, x) / (x,)."""
    dims = tuple(reversed(shape))                      # x first
    rec = np.zeros(shape, dtype=lgd.TEST_RECORD)
    idx = np.indices(shape)                            # z, y, x order
    for a in range(len(dims)):
        rec["pos"][..., a] = idx[len(shape) - 1 - a]
        rec["dim"][..., a] = dims[a]
    for a in range(len(dims), 3):
        rec["dim"][..., a] = 1
    rec["cycle"] = start_step * nano_steps
    rec["valid"] = 1
    rec["test_value"] = 1 + np.arange(rec.size).reshape(shape)
    return rec


EDGE = 1 + 2        # the edge cell: valid and marked as edge


@pytest.mark.parametrize("shape,periodic,von_neumann,nano", [
    ((777,), 0, True, 27), ((666,), 1, False, 27),
    ((151, 121), 0, True, 27), ((131, 141), 3, False, 27),
    ((10, 20, 50), 0, True, 3), ((13, 20, 54), 7, False, 3), ((5, 7, 9), 5, False, 3), ((4, 6, 8), 2, True, 3)])
def test_test_cell_grids_stay_valid(shape, periodic, von_neumann, nano):
    flags = lgd.TEST_NANO_STEPS(nano) | (lgd.TEST_VON_NEUMANN if von_neumann else 0)
    start = 4
    with lgd.Grid(lgd.CELL_TEST, shape, periodic=periodic, edge=(EDGE,), flags=flags) as g:
        g.upload(0, initial(shape, nano, start))
        for step in range(3):
            for k in range(nano):
                g.step(1, nano_step=k)
        out = g.download(0)
        assert out["valid"].all()
        assert (out["edge"] == 0).all()
        assert (out["cycle"] == (start + 3) * nano).all()
        np.testing.assert_array_equal(out["pos"], initial(shape, nano)["pos"])
        # one call with a count runs consecutive nano steps
        g.step(nano, nano_step=0)
        out = g.download(0)
        assert out["valid"].all() and (out["cycle"] == (start + 4) * nano).all()


def test_test_cell_catches_wrong_nano_step_position_and_edge():
    shape = (6, 8, 10)
    flags = lgd.TEST_NANO_STEPS(3)
    with lgd.Grid(lgd.CELL_TEST, shape, edge=(EDGE,), flags=flags) as g:     # nano step out of sync
        g.upload(0, initial(shape, 3))
        g.step(1, nano_step=1)
        out = g.download(0)
        assert not out["valid"].any()
        assert (out["cycle"] == 0).all()
    with lgd.Grid(lgd.CELL_TEST, shape, edge=(EDGE,), flags=flags) as g:     # one cell with a wrong position
        rec = initial(shape, 3)
        rec["pos"][3, 4, 5, 0] = 6
        g.upload(0, rec)
        g.step(1, nano_step=0)
        out = g.download(0)
        bad = ~out["valid"].astype(bool)
        want = np.zeros(shape, dtype=bool)
        want[2:5, 3:6, 4:7] = True                     # its Moore neighbours (they see it) and itself
        np.testing.assert_array_equal(bad, want)
    with lgd.Grid(lgd.CELL_TEST, shape, edge=(1,), flags=flags) as g:        # edge cell not marked as edge
        g.upload(0, initial(shape, 3))
        g.step(1, nano_step=0)
        out = g.download(0)
        inner = np.zeros(shape, dtype=bool)
        inner[1:-1, 1:-1, 1:-1] = True
        assert out["valid"][inner].all() and not out["valid"][~inner].any()


def test_test_cell_flags_are_checked():
    with pytest.raises(lgd.LGDError):
        lgd.Grid(lgd.CELL_TEST, (4, 4, 4), flags=1 << 20)
    with pytest.raises(lgd.LGDError):
        lgd.Grid(lgd.CELL_JACOBI7_F64, (4, 4, 4), flags=lgd.TEST_NANO_STEPS(3))
