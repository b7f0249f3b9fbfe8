"""The timeout path of the bounded device waits, made to run out on purpose
without a fault: the TMA Jacobi kernel's first CTA leaves one plane's copy
unissued (lgd_gpu_test_bounded_waits), its wait for that plane returns after
a short bound, the CTA drains the copies it did issue and returns, and the
host sees LGD_ERR_TIMEOUT at the next synchronising call.  The same handle
then runs normal steps, bit-identical to the oracle."""
import numpy as np
import pytest

import oracle
from libgeodecomp_gb300 import lgd, workloads

pytestmark = pytest.mark.gpu


def bounded_waits(g, cycles, skip_plane):
    lgd.check(lgd.lib().lgd_gpu_test_bounded_waits(g._h, cycles, skip_plane))


@pytest.mark.parametrize("skip_plane", [0, 1, 2])
def test_wait_runs_out_reports_timeout_and_the_grid_recovers(skip_plane):
    u0 = workloads.jacobi_initial(64, 32, 24, seed=3)
    with lgd.Grid(lgd.CELL_JACOBI7_F64, u0.shape) as g:
        g.upload(0, u0)
        bounded_waits(g, 2_000_000, skip_plane)        # about a millisecond
        before = g.launch_count()
        g.step(1)
        assert g.launch_count() - before == 1          # the TMA kernel ran
        with pytest.raises(lgd.LGDError) as e:
            g.synchronize()
        assert e.value.code == lgd.ERR_TIMEOUT
        g.synchronize()                                # the error word was cleared
        bounded_waits(g, 0, -1)
        g.upload(0, u0)
        g.step(5)
        out = g.download(0)
    np.testing.assert_array_equal(out, oracle.jacobi7(u0, 5))


def test_short_bound_alone_does_not_fire():
    """A bound of a millisecond is far above a plane copy's latency: normal
    steps under it are unaffected."""
    u0 = workloads.jacobi_initial(64, 32, 24, seed=4)
    with lgd.Grid(lgd.CELL_JACOBI7_F64, u0.shape) as g:
        g.upload(0, u0)
        bounded_waits(g, 2_000_000, -1)
        g.step(6)
        out = g.download(0)
    np.testing.assert_array_equal(out, oracle.jacobi7(u0, 6))


def test_bad_arguments():
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (8, 8, 8)) as g:
        with pytest.raises(lgd.LGDError):
            bounded_waits(g, -1, -1)
        with pytest.raises(lgd.LGDError):
            bounded_waits(g, 0, -2)
