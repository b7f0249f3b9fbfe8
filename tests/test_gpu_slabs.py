"""The slab decomposition on the GPU: two and three ranks, as threads of one
process on one GPU (each rank its own library grid and stream; the ghost
planes travel through host memory between steps, no kernel waits for
another), give the single grid's result bit for bit - for the IEEE and the
fixed-point Jacobi cells, the FP32 cell with three steps per pass, Game of
Life on a torus cut along y and variable-coefficient diffusion on a torus
cut along z."""
import threading

import numpy as np
import pytest

from libgeodecomp_gb300 import lgd, slabs, workloads

pytestmark = pytest.mark.gpu


def run_ranks(cell, arrays, periodic, steps, world, ghost, time_block=0, edge=(0.0, 0.0, 0.0, 0.0), pin=None,
              device=False):
    hub = slabs.InProcessComm.Hub(world)
    parts = [None] * world
    errors = []
    shape = arrays[0].shape

    def rank_main(r):
        try:
            comm = slabs.InProcessComm(hub, r, device=device)
            s = slabs.SlabGrid(cell, shape, comm, periodic=periodic, ghost=ghost, time_block=time_block,
                               make_grid=lambda sh, m: lgd.Grid(cell, sh, periodic=m, edge=edge),
                               fixed_point=cell == lgd.CELL_JACOBI7_F64_FIX)
            for m, a in enumerate(arrays):
                s.upload(m, a)
            s.step(steps // 3)
            s.step(steps - steps // 3)
            parts[r] = s.download_owned()
            s.close()
        except Exception as e:
            errors.append(e)
            hub.barrier.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    return np.concatenate(parts, axis=0)


def run_single(cell, arrays, periodic, steps, time_block=0, edge=(0.0, 0.0, 0.0, 0.0), pin=None):
    with lgd.Grid(cell, arrays[0].shape, periodic=periodic, edge=edge) as g:
        if time_block:
            g.set_time_block(time_block)
        if pin is not None:
            g.set_fixed_point_exponent(pin, True)
        for m, a in enumerate(arrays):
            g.upload(m, a)
        g.step(steps)
        return g.download(0)


@pytest.mark.parametrize("world,ghost,device", [(2, 4, False), (3, 6, False), (3, 5, True)])
def test_ieee_jacobi_slabs_bit_identical(world, ghost, device):
    """device=True exchanges through CUDA buffers with device-to-device
    plane copies, as NCCL ranks do."""
    u0 = workloads.jacobi_initial(70, 33, 61, seed=4)
    ref = run_single(lgd.CELL_JACOBI7_F64, [u0], 0, 25)
    out = run_ranks(lgd.CELL_JACOBI7_F64, [u0], 0, 25, world, ghost, device=device)
    np.testing.assert_array_equal(out, ref)


@pytest.mark.parametrize("world,ghost", [(2, 4), (3, 8)])
def test_fixed_point_jacobi_slabs_bit_identical(world, ghost):
    """Two steps per pass on every rank, one pinned exponent everywhere."""
    u0 = workloads.jacobi_initial(64, 40, 72, seed=5)
    e = int(np.frexp(np.max(u0))[1])
    ref = run_single(lgd.CELL_JACOBI7_F64_FIX, [u0], 0, 30, pin=e)
    out = run_ranks(lgd.CELL_JACOBI7_F64_FIX, [u0], 0, 30, world, ghost)
    np.testing.assert_array_equal(out, ref)


def test_f32_jacobi_slabs_three_steps_per_pass():
    u0 = workloads.jacobi_initial(64, 32, 90, seed=6).astype(np.float32)
    ref = run_single(lgd.CELL_JACOBI7_F32, [u0], 0, 24, time_block=3)
    out = run_ranks(lgd.CELL_JACOBI7_F32, [u0], 0, 24, 3, 6, time_block=3)
    np.testing.assert_array_equal(out, ref)


def test_life_slabs_torus_cut_along_y():
    c0 = workloads.gol_initial(96, 90, seed=8)
    ref = run_single(lgd.CELL_GOL_U8, [c0], 3, 60)
    out = run_ranks(lgd.CELL_GOL_U8, [c0], 3, 60, 3, 10)
    np.testing.assert_array_equal(out, ref)


def test_varcoef_slabs_torus_cut_along_z():
    u0, k = workloads.varcoef_fields(32, seed=9, length=6.0)
    arrays = [u0.astype(np.float32), k.astype(np.float32)]
    ref = run_single(lgd.CELL_VARCOEF_F32, arrays, 7, 20)
    out = run_ranks(lgd.CELL_VARCOEF_F32, arrays, 7, 20, 2, 5)
    np.testing.assert_array_equal(out, ref)


def test_copy_planes_round_trip_and_bounds():
    u0 = workloads.jacobi_initial(20, 6, 9, seed=1)
    with lgd.Grid(lgd.CELL_JACOBI7_F64, u0.shape) as g:
        g.upload(0, u0)
        pb = g.plane_bytes()
        assert pb % 128 == 0 and pb >= 6 * 20 * 8
        raw = g.save_planes(2, 3)
        assert raw.nbytes == 3 * pb
        g.load_planes(5, raw)
        out = g.download(0)
        np.testing.assert_array_equal(out[5:8], u0[2:5])
        with pytest.raises(lgd.LGDError) as e:
            g.save_planes(8, 2)
        assert e.value.code == lgd.ERR_RANGE
