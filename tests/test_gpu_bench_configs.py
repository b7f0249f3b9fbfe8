"""Parity at the benchmarked configurations, on the benchmark's own inputs.

The benchmark times Jacobi-7 on 512^3 (fixed-point cell, device fill of
U[0,1) with seed 42, two steps per pass), Game of Life on 8192^2 for 1000
generations, SELL-C-sigma diffusion on 4,194,304 nodes for 200 steps and the
512-cavity D3Q19 ensemble in FP32 for 500 steps.  These tests run exactly
those inputs through the C ABI and compare with the oracle: Game of Life bit
for bit, the FP64 cells within 1e-12 relative per cell, the FP32 ensemble
with its error against FP64 stated.  The long runs show what the fixed-point cell guarantees over
thousands of steps: it multiplies by the same fl(1/7) as the reference's
cell (no drift against it), its exponent follows a decaying grid down, and
its error stays within its stated absolute bound.
"""
import numpy as np
import pytest

import oracle
from libgeodecomp_gb300 import lgd, workloads

pytestmark = pytest.mark.gpu


def rel_per_cell(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def rel_normwise(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def jacobi_512_initial():
    return workloads.jacobi_initial(512, 512, 512, seed=42)


@pytest.mark.parametrize("steps", [20, 100])
def test_jacobi7_fixed_point_512_bench_grid(jacobi_512_initial, steps):
    """The headline workload: device-filled 512^3 grid, default depth (passes
    of two steps), 20 and 100 steps, per-cell relative error <= 1e-12."""
    with lgd.Grid(lgd.CELL_JACOBI7_F64_FIX, (512, 512, 512)) as g:
        g.fill_uniform(0, seed=42, stream=workloads.STREAM_GRID)
        before = g.launch_count()
        g.step(steps)
        assert g.launch_count() - before == steps // 2      # two steps per pass
        out = g.download(0)
    ref = oracle.jacobi7(jacobi_512_initial, steps)
    assert rel_per_cell(out, ref) <= 1e-12


def test_jacobi7_ieee_512_bench_grid_bit_exact(jacobi_512_initial):
    """The IEEE FP64 cell on the same grid: bit-identical to the oracle."""
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (512, 512, 512)) as g:
        g.fill_uniform(0, seed=42, stream=workloads.STREAM_GRID)
        g.step(10)
        out = g.download(0)
    np.testing.assert_array_equal(out, oracle.jacobi7(jacobi_512_initial, 10))


@pytest.mark.parametrize("edge,steps", [(128, 5000), (64, 20000)])
def test_jacobi7_fixed_point_long_runs(edge, steps):
    """Thousands of steps with the constant-zero boundary: the field decays
    (64^3 x 20000 by nine orders of magnitude) and its values span five
    orders between the centre and the corners.

    The bound the fixed-point cell guarantees per cell is absolute: each
    step rounds once, by at most half a unit 2^(e - 58), and the averaging
    never amplifies an error, so |fix - exact| <= steps * 2^(e0 - 58) with
    e0 the exponent at upload (it only falls afterwards).  Against the
    reference (which rounds seven times per step) every cell stays within
    1e-12 relative plus that absolute bound, the grid within 1e-12 of its
    maximum, and every cell above a thousandth of the maximum within 1e-12
    relative; cells far below the maximum carry the grid's absolute
    resolution (the corners of 128^3 after 5000 steps: about 1e-12)."""
    u0 = workloads.jacobi_initial(edge, edge, edge, seed=42)
    with lgd.Grid(lgd.CELL_JACOBI7_F64_FIX, u0.shape) as g:
        g.upload(0, u0)
        e0 = g.fixed_point_exponent()
        g.step(steps)
        out = g.download(0)
        e1 = g.fixed_point_exponent()
    ref = oracle.jacobi7(u0, steps)
    assert e1 <= e0              # the exponent followed the decay down
    absolute = steps * 2.0 ** (e0 - 58)
    assert np.all(np.abs(out - ref) <= 1e-12 * np.abs(ref) + absolute)
    assert rel_normwise(out, ref) <= 1e-12
    big = np.abs(ref) >= 1e-3 * np.max(np.abs(ref))
    assert rel_per_cell(out[big], ref[big]) <= 1e-12


def test_jacobi7_fixed_point_exponent_follows_uploads_and_decay():
    """A grid of small values gets a small exponent at upload (all 57
    fraction bits used), and the exponent falls as a grid decays."""
    u0 = workloads.jacobi_initial(24, 20, 16, seed=3) * 1e-3
    with lgd.Grid(lgd.CELL_JACOBI7_F64_FIX, u0.shape) as g:
        g.upload(0, u0)
        assert g.fixed_point_exponent() == int(np.frexp(np.max(u0))[1])
        e0 = g.fixed_point_exponent()
        g.step(512)
        out = g.download(0)
        assert g.fixed_point_exponent() < e0
    ref = oracle.jacobi7(u0, 512)
    assert rel_per_cell(out, ref) <= 1e-12


def test_gol_8192_full_run_bit_exact():
    """Game of Life 8192^2 torus, Bernoulli(0.3) seed 42 (device fill), the
    configuration's 1000 generations: bit-identical to the oracle."""
    with lgd.Grid(lgd.CELL_GOL_U8, (8192, 8192), periodic=3) as g:
        g.fill_bernoulli(0.3, seed=42, stream=workloads.STREAM_GRID)
        c0 = g.download(0)
        g.step(1000)
        out = g.download(0)
    np.testing.assert_array_equal(c0, workloads.gol_initial(8192, 8192, seed=42))
    np.testing.assert_array_equal(out, oracle.gol(c0, 1000))


@pytest.fixture(scope="module")
def sell_4m():
    n = 4194304
    rp, col, w = workloads.powerlaw_graph(n, seed=42)
    return n, rp, col, w, workloads.sell_values(n, seed=42)


def test_sell_4m_full_run_gpu_built(sell_4m):
    """The benchmark's grid: SELL-C-sigma built on the GPU from CSR, the
    configuration's 200 steps of the fused kernel, within 1e-12 per node of
    the oracle; the exact-mode kernel bit-identical to it."""
    n, rp, col, w, x0 = sell_4m
    s = oracle.sell_build(n, rp, col, w, 32, 256)
    ref_phys = oracle.sell_diffusion(s, 32, x0[s["perm"]], 200)
    ref = np.empty(n)
    ref[s["perm"]] = ref_phys
    with lgd.SellGrid.from_csr(n, rp, col, w, 32, 256) as g:
        g.upload(x0)
        g.step(200)
        out = g.download()
    assert rel_per_cell(out, ref) <= 1e-12
    with lgd.SellGrid.from_csr(n, rp, col, w, 32, 256, exact=True) as g:
        g.upload(x0)
        g.step(200)
        out = g.download()
    np.testing.assert_array_equal(out, ref)


def test_lbm_512_ensemble_fp32_error_at_500_steps():
    """The benchmark's ensemble: 512 cavities (1.09e9 cells, 83 GB per
    buffer), FP32, the configuration's 500 steps in the launch form the
    tuner picks on it (two steps per launch, 32 x 4 columns); four of its
    cavities against the FP64 oracle.  The FP32 error is stated, not
    bit-exact: measured on GB300 rel-L2 1.9e-5 - 2.5e-5 and max-abs 6.4e-6 -
    8.5e-6 per cavity."""
    edges, omegas = workloads.lbm_ensemble(512, seed=42)
    picks = [287, 156, 504, 72]           # three of the 32^3 cavities and a 64^3 one, omegas 1.01 - 1.74
    with lgd.LbmEnsemble(edges, omegas, lid=0.05, precision=4) as e:
        e.set_time_block(2, 1, 4)
        e.step(500)
        got = {j: e.download(j) for j in picks}
    for j in picks:
        ref = oracle.lbm(int(edges[j]), 500, float(omegas[j]), 0.05)
        rel_l2 = float(np.linalg.norm(got[j] - ref) / np.linalg.norm(ref))
        max_abs = float(np.max(np.abs(got[j] - ref)))
        print("cavity %d (L = %d, omega %.3f): rel-L2 %.3g, max-abs %.3g" % (j, edges[j], omegas[j], rel_l2, max_abs))
        assert rel_l2 < 2e-4 and max_abs < 2e-4, (j, rel_l2, max_abs)


def test_varcoef_256_full_run():
    """The variable-coefficient configuration: 256^3 torus, GRF fields
    (length 16), to t = 4096.  The FP64 cell is bit-identical to the oracle
    over the whole run; the FP32 cell (the benchmarked one, packed FP32
    arithmetic) stays within rel-L2 1e-5 of it (measured on GB300: 5.6e-6)."""
    u0, k = workloads.varcoef_fields(256, seed=42, length=16.0)
    ref = oracle.varcoef(u0, k, 4096)
    with lgd.Grid(lgd.CELL_VARCOEF_F64, u0.shape, periodic=7) as g:
        g.upload(0, u0)
        g.upload(1, k)
        g.step(4096)
        np.testing.assert_array_equal(g.download(0), ref)
    with lgd.Grid(lgd.CELL_VARCOEF_F32, u0.shape, periodic=7) as g:
        g.upload(0, u0.astype(np.float32))
        g.upload(1, k.astype(np.float32))
        g.step(4096)
        out = g.download(0).astype(np.float64)
    rel_l2 = float(np.linalg.norm(out - ref) / np.linalg.norm(ref))
    assert rel_l2 < 1e-5, rel_l2
