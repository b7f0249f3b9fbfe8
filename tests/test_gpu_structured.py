"""Structured-grid parity on the GPU, through the C ABI.

Integer and IEEE-FP64 cells must match the reference bit for bit; the
fixed-point FP64 Jacobi must stay within 1e-12 relative of the FP64
reference; FP32 cells state their error against the FP64 oracle.  The
boundary-handling cases restate the reference's own known-answer test
(storage/test/unit/fixedneighborhoodupdatefunctortest.h:109-379).
"""
import hashlib
import os

import numpy as np
import pytest

import oracle
from libgeodecomp_gb300 import lgd, workloads

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name + ".npz"), allow_pickle=False)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_grid(cell, arrays, steps, periodic=0, edge=(0.0, 0.0, 0.0, 0.0), member=0):
    shape = arrays[0].shape
    with lgd.Grid(cell, shape, periodic=periodic, edge=edge) as g:
        for m, a in enumerate(arrays):
            g.upload(m, a)
        g.step(steps)
        return g.download(member)


# ------------------------------------------------------------------ Jacobi-7
@pytest.mark.parametrize("name", ["jacobi7_cube_24x20x16", "jacobi7_torus_17x13x11"])
def test_jacobi7_f64_bit_exact_small(name):
    g = load(name)
    nz, ny, nx = g["shape"]
    u0 = workloads.jacobi_initial(nx, ny, nz, seed=42)
    out = run_grid(lgd.CELL_JACOBI7_F64, [u0], int(g["steps"]), periodic=7 if bool(g["torus"]) else 0)
    np.testing.assert_array_equal(out, g["out"])


def test_jacobi7_f64_bit_exact_128_config():
    g = load("jacobi7_cube_128")
    u0 = workloads.jacobi_initial(128, 128, 128, seed=42)
    out = run_grid(lgd.CELL_JACOBI7_F64, [u0], 100)
    np.testing.assert_array_equal(out.reshape(-1)[g["sample_idx"]], g["sample"])
    assert sha(out) == str(g["sha256"])


@pytest.mark.parametrize("shape,periodic", [((13, 11, 7), 0), ((5, 9, 33), 7), ((1, 10, 20), 7), ((40, 3, 65), 0),
                                            ((1, 1, 1), 0), ((2, 1, 37), 7)])
def test_jacobi7_f64_odd_shapes_match_oracle(shape, periodic):
    u0 = workloads.jacobi_initial(shape[2], shape[1], shape[0], seed=5)
    out = run_grid(lgd.CELL_JACOBI7_F64, [u0], 9, periodic=periodic)
    np.testing.assert_array_equal(out, oracle.jacobi7(u0, 9, torus=periodic == 7))


@pytest.mark.parametrize("shape", [(9, 12, 20), (17, 23, 45), (5, 70, 130)])
def test_jacobi7_f64_nonzero_edge(shape):
    u0 = workloads.jacobi_initial(shape[2], shape[1], shape[0], seed=8)
    out = run_grid(lgd.CELL_JACOBI7_F64, [u0], 6, edge=(0.75, 0, 0, 0))
    np.testing.assert_array_equal(out, oracle.jacobi7(u0, 6, edge=0.75))


def rel_err(a, b):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def test_jacobi7_fixed_point_within_1e12_of_reference_128_config():
    g = load("jacobi7_cube_128")
    u0 = workloads.jacobi_initial(128, 128, 128, seed=42)
    out = run_grid(lgd.CELL_JACOBI7_F64_FIX, [u0], 100)
    ref = oracle.jacobi7(u0, 100)
    assert sha(ref) == str(g["sha256"])
    assert rel_err(out, ref) <= 1e-12
    np.testing.assert_allclose(out.reshape(-1)[g["sample_idx"]], g["sample"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", ["jacobi7_cube_24x20x16", "jacobi7_torus_17x13x11"])
def test_jacobi7_fixed_point_small(name):
    g = load(name)
    nz, ny, nx = g["shape"]
    u0 = workloads.jacobi_initial(nx, ny, nz, seed=42)
    out = run_grid(lgd.CELL_JACOBI7_F64_FIX, [u0], int(g["steps"]), periodic=7 if bool(g["torus"]) else 0)
    assert rel_err(out, g["out"]) <= 1e-12


def test_jacobi7_fixed_point_signed_values_and_edge():
    u0 = workloads.jacobi_initial(31, 17, 12, seed=9) * 6.0 - 3.0
    out = run_grid(lgd.CELL_JACOBI7_F64_FIX, [u0], 20, edge=(-2.5, 0, 0, 0))
    ref = oracle.jacobi7(u0, 20, edge=-2.5)
    # the fixed-point grid adds at most 20 * 2^(2 - 60) ~ 6.9e-17; the FP64
    # reference itself rounds each of its 7 operations per step (ulp(2.4) =
    # 4.4e-16), so the difference is dominated by the reference's own rounding
    assert np.max(np.abs(out - ref)) <= 20 * 7 * 4.5e-16
    # relative error is meaningful away from the values that cross zero
    mask = np.abs(ref) > 1e-3
    assert rel_err(out[mask], ref[mask]) <= 1e-12


def test_jacobi7_fixed_point_device_fill_matches_host_generator():
    with lgd.Grid(lgd.CELL_JACOBI7_F64_FIX, (16, 16, 16)) as g:
        g.fill_uniform(0, seed=42, stream=workloads.STREAM_GRID)
        got = g.download(0)
    np.testing.assert_array_equal(got, workloads.jacobi_initial(16, 16, 16, seed=42))


def test_jacobi7_f32_error_against_fp64():
    u0 = workloads.jacobi_initial(64, 64, 64, seed=42)
    out = run_grid(lgd.CELL_JACOBI7_F32, [u0.astype(np.float32)], 50).astype(np.float64)
    ref = oracle.jacobi7(u0, 50)
    rel_l2 = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    max_abs = np.max(np.abs(out - ref))
    # measured on GB300: rel-L2 2.4e-6, max-abs 1.5e-6 (64^3, 50 steps)
    assert rel_l2 < 1e-5 and max_abs < 1e-5, (rel_l2, max_abs)


# ---------------------------------------- boundary handling (reference KAT)
def coord_values(nz, ny, nx, origin):
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return (x + origin[0]) + (y + origin[1]) * 1000.0 + (z + origin[2]) * 1000.0 * 1000.0


def expected_sum6(nz, ny, nx, origin, streaks, torus):
    """The reference test's expectation: the coordinate-encoded sum over the
    six face neighbours, normalised on the torus, (-1,-1,-1) off the cube."""
    exp = {}
    for (x0, y, z, end) in streaks:
        for x in range(x0, end):
            sx = sy = sz = 0
            for d in ((0, 0, -1), (0, -1, 0), (-1, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)):
                cx, cy, cz = x + d[0], y + d[1], z + d[2]
                if torus:
                    cx, cy, cz = cx % nx, cy % ny, cz % nz
                    sx += cx + origin[0]
                    sy += cy + origin[1]
                    sz += cz + origin[2]
                elif 0 <= cx < nx and 0 <= cy < ny and 0 <= cz < nz:
                    sx += cx + origin[0]
                    sy += cy + origin[1]
                    sz += cz + origin[2]
                else:
                    sx -= 1
                    sy -= 1
                    sz -= 1
            exp[(x, y, z)] = sx + sy * 1000.0 + sz * 1000 * 1000.0
    return exp


# the reference test's region, shifted to the box origin (10, 20, 30)
REF_STREAKS = [(10, 20, 30, 209), (10, 21, 30, 210), (10, 30, 30, 210), (10, 30, 40, 210),
               (25, 31, 40, 200), (25, 119, 40, 200), (10, 30, 49, 210)]


@pytest.mark.parametrize("torus", [True, False])
def test_sum6_reference_region_kat(torus):
    origin = (10, 20, 30)
    nx, ny, nz = 200, 100, 50
    streaks = [(x - origin[0], y - origin[1], z - origin[2], e - origin[0]) for (x, y, z, e) in REF_STREAKS]
    a = coord_values(nz, ny, nx, origin)
    edge = (-1001001.0, -1.0, 0, 0)
    with lgd.Grid(lgd.CELL_SUM6_F64, (nz, ny, nx), periodic=7 if torus else 0, edge=edge) as g:
        g.upload(0, a)
        g.upload(1, np.full(a.shape, 777.0))
        g.upload(1, np.full(a.shape, 999.0), which=1)
        g.update_region(streaks)
        g.swap()
        b = g.download(1)
    exp = expected_sum6(nz, ny, nx, origin, streaks, torus)
    for (x, y, z), v in exp.items():
        assert b[z, y, x] == v, (x, y, z)
    # cells outside the region keep the new grid's previous contents
    mask = np.ones(b.shape, dtype=bool)
    for (x, y, z) in exp:
        mask[z, y, x] = False
    assert np.all(b[mask] == 999.0)


def test_sum6_degenerated_torus_kat():
    nx, ny, nz = 1, 10, 20
    a = coord_values(nz, ny, nx, (0, 0, 0))
    streaks = [(0, y, z, 1) for z in range(nz) for y in range(ny)]
    with lgd.Grid(lgd.CELL_SUM6_F64, (nz, ny, nx), periodic=7) as g:
        g.upload(0, a)
        g.update_region(streaks)
        g.swap()
        b = g.download(1)
    exp = expected_sum6(nz, ny, nx, (0, 0, 0), streaks, True)
    for (x, y, z), v in exp.items():
        assert b[z, y, x] == v


def test_region_rejects_streaks_outside_the_grid():
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (4, 4, 4)) as g:
        with pytest.raises(lgd.LGDError) as e:
            g.update_region([(0, 0, 0, 5)])
        assert e.value.code == lgd.ERR_RANGE
        with pytest.raises(lgd.LGDError) as e:
            g.update_region([(0, 4, 0, 1)])
        assert e.value.code == lgd.ERR_RANGE


def test_upload_rejects_wrong_size():
    with lgd.Grid(lgd.CELL_JACOBI7_F64, (4, 4, 4)) as g:
        with pytest.raises(lgd.LGDError) as e:
            lgd.check(lgd.lib().lgd_gpu_upload(g._h, 0, 0, lgd._ptr(np.zeros(10)), 80))
        assert e.value.code == lgd.ERR_INVALID


@pytest.mark.parametrize("cell", [lgd.CELL_JACOBI7_F64, lgd.CELL_JACOBI7_F64_FIX])
def test_region_save_load_roundtrip(cell):
    """Streak copies (the drop-in's writers read planes this way); the
    fixed-point grid converts at the boundary, exactly for values whose
    53-bit mantissa fits its 57 fraction bits.  Loading negative values
    into the fixed-point grid ends its sign-free fast path and the next
    steps stay right."""
    u0 = workloads.jacobi_initial(30, 20, 10, seed=4)
    streaks = [(3, 2, 1, 17), (0, 19, 9, 30), (5, 5, 5, 6)]
    with lgd.Grid(cell, u0.shape) as g:
        g.upload(0, u0)
        got = g.save_region(0, streaks)
        exp = np.concatenate([u0[z, y, x:e] for (x, y, z, e) in streaks])
        np.testing.assert_array_equal(got, exp)
        g.load_region(0, streaks, -got)
        u1 = g.download(0)
    ref = u0.copy()
    for (x, y, z, e) in streaks:
        ref[z, y, x:e] = -ref[z, y, x:e]
    np.testing.assert_array_equal(u1, ref)
    if cell == lgd.CELL_JACOBI7_F64_FIX:
        with lgd.Grid(cell, u0.shape) as g:
            g.upload(0, u0)
            g.load_region(0, streaks, -got)
            g.step(4)
            out = g.download(0)
        # four steps of values in (-1, 1): the fixed-point rounding (4 x
        # 2^-58) and the reference's own (seven roundings per step)
        assert np.max(np.abs(out - oracle.jacobi7(ref, 4))) < 1e-14


def test_checksum_matches_host_sum():
    u0 = workloads.jacobi_initial(50, 40, 30, seed=2)
    with lgd.Grid(lgd.CELL_JACOBI7_F64, u0.shape) as g:
        g.upload(0, u0)
        assert abs(g.checksum(0) - u0.sum()) <= 1e-9 * u0.sum()


# ------------------------------------------------------------- Game of Life
def test_gol_small_bit_exact():
    g = load("gol_64x48")
    c0 = workloads.gol_initial(64, 48, seed=42)
    np.testing.assert_array_equal(run_grid(lgd.CELL_GOL_U8, [c0], 50, periodic=3), g["out"])


def test_gol_1024_1000_steps_golden():
    g = load("gol_1024")
    c0 = workloads.gol_initial(1024, 1024, seed=42)
    out = run_grid(lgd.CELL_GOL_U8, [c0], 1000, periodic=3)
    np.testing.assert_array_equal(out.sum(axis=1), g["row_alive"])
    assert sha(out) == str(g["sha256"])


@pytest.mark.parametrize("shape", [(37, 50), (1, 16), (3, 3), (17, 48)])
def test_gol_odd_shapes_match_oracle(shape):
    c0 = workloads.gol_initial(shape[1], shape[0], seed=6)
    np.testing.assert_array_equal(run_grid(lgd.CELL_GOL_U8, [c0], 23, periodic=3), oracle.gol(c0, 23))


def gol_cube_numpy(c, steps):
    c = c.astype(np.int32)
    for _ in range(steps):
        p = np.pad(c, 1)
        n = sum(p[1 + dy:1 + dy + c.shape[0], 1 + dx:1 + dx + c.shape[1]]
                for dy in (-1, 0, 1) for dx in (-1, 0, 1) if (dy, dx) != (0, 0))
        c = np.where(c == 1, ((n == 2) | (n == 3)), n == 3).astype(np.int32)
    return c.astype(np.uint8)


def test_gol_cube_dead_edge():
    c0 = workloads.gol_initial(45, 31, seed=3)
    np.testing.assert_array_equal(run_grid(lgd.CELL_GOL_U8, [c0], 15, periodic=0), gol_cube_numpy(c0, 15))


def test_gol_8192_config_against_oracle_100_steps():
    with lgd.Grid(lgd.CELL_GOL_U8, (8192, 8192), periodic=3) as g:
        g.fill_bernoulli(0.3, seed=42, stream=workloads.STREAM_GRID)
        c0 = g.download(0)
        np.testing.assert_array_equal(c0[:4], workloads.gol_initial(8192, 8192, seed=42)[:4])
        g.step(100)
        out = g.download(0)
    np.testing.assert_array_equal(out, oracle.gol(c0, 100))


# ------------------------------------------------------------- var-coef
def test_varcoef_f64_bit_exact():
    g = load("varcoef_16")
    out = run_grid(lgd.CELL_VARCOEF_F64, [g["u0"], g["k"]], int(g["steps"]), periodic=7)
    np.testing.assert_array_equal(out, g["out"])


def test_varcoef_f32_error_against_fp64():
    u0, k = workloads.varcoef_fields(32, seed=42, length=8.0)
    out = run_grid(lgd.CELL_VARCOEF_F32, [u0.astype(np.float32), k.astype(np.float32)], 64, periodic=7)
    ref = oracle.varcoef(u0, k, 64)
    rel_l2 = np.linalg.norm(out.astype(np.float64) - ref) / np.linalg.norm(ref)
    assert rel_l2 < 1e-6, rel_l2


@pytest.mark.parametrize("shape", [(8, 12, 64), (20, 10, 128), (5, 7, 130), (3, 2, 64), (66, 4, 192)])
def test_varcoef_f64_wide_grids_bit_exact(shape):
    """Grids whose x extent fills 64-wide warps run the register kernel's
    vector path (wrap decisions per row and plane)."""
    nz, ny, nx = shape
    rng = np.random.default_rng(nx * ny + nz)
    u0 = rng.random(shape)
    k = 0.02 + 0.13 * rng.random(shape)
    out = run_grid(lgd.CELL_VARCOEF_F64, [u0, k], 9, periodic=7)
    np.testing.assert_array_equal(out, oracle.varcoef(u0, k, 9))


def test_varcoef_f32_register_kernel_equals_shared_memory_kernel():
    u0, k = workloads.varcoef_fields(64, seed=3, length=8.0)
    res = []
    for variant in (0, 1):
        with lgd.Grid(lgd.CELL_VARCOEF_F32, u0.shape, periodic=7) as g:
            _set_variant(g, variant)
            g.upload(0, u0.astype(np.float32))
            g.upload(1, k.astype(np.float32))
            g.step(12)
            res.append(g.download(0).astype(np.float64))
    ref = oracle.varcoef(u0, k, 12)
    for r in res:
        assert np.linalg.norm(r - ref) / np.linalg.norm(ref) < 1e-6


@pytest.mark.parametrize("shape,periodic", [((16, 32, 64), 7), ((9, 19, 70), 7), ((20, 17, 130), 0),
                                            ((7, 33, 66), 1), ((12, 16, 64), 2), ((18, 5, 128), 4),
                                            ((6, 40, 100), 3), ((3, 2, 2), 7), ((33, 18, 200), 6)])
def test_varcoef_f64_tma_kernel_equals_register_and_shared_memory_kernels(shape, periodic):
    """The TMA kernel (variant 6: applies on these grids - zero edges, even
    rows) against the thread-loaded kernels, bit for bit in FP64, on every
    mix of wrapping axes and on tiles cut by the grid's edge."""
    rng = np.random.default_rng(sum(shape) + periodic)
    u0 = rng.random(shape)
    k = 0.02 + 0.13 * rng.random(shape)
    res = []
    for variant in (6, 1, 2):
        with lgd.Grid(lgd.CELL_VARCOEF_F64, shape, periodic=periodic) as g:
            _set_variant(g, variant)
            g.upload(0, u0)
            g.upload(1, k)
            g.step(7)
            res.append(g.download(0))
    np.testing.assert_array_equal(res[0], res[1])
    np.testing.assert_array_equal(res[0], res[2])
    if periodic == 7:
        np.testing.assert_array_equal(res[0], oracle.varcoef(u0, k, 7))


def test_varcoef_f32_tma_kernel_against_fp64():
    u0, k = workloads.varcoef_fields(96, seed=11, length=8.0)
    with lgd.Grid(lgd.CELL_VARCOEF_F32, u0.shape, periodic=7) as g:
        g.upload(0, u0.astype(np.float32))
        g.upload(1, k.astype(np.float32))
        g.step(40)
        out = g.download(0).astype(np.float64)
    ref = oracle.varcoef(u0, k, 40)
    rel_l2 = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert rel_l2 < 1e-6, rel_l2
    assert np.max(np.abs(out - ref)) < 1e-5


# ------------------------------------------ kernel variants and fast paths
def _set_variant(g, v):
    fn = lgd.lib().lgd_gpu_set_variant
    fn.argtypes = [lgd.ctypes.c_void_p, lgd.ctypes.c_int]
    lgd.check(fn(g._h, v))


@pytest.mark.parametrize("shape,periodic", [((9, 20, 128), 0), ((9, 20, 128), 7), ((70, 16, 64), 0),
                                            ((70, 16, 64), 7), ((3, 4, 64), 7), ((1, 8, 192), 0),
                                            ((33, 13, 130), 7), ((17, 7, 96), 0)])
@pytest.mark.parametrize("variant", [0, 1, 2])
def test_jacobi7_variants_bit_exact_on_wide_grids(shape, periodic, variant):
    """Shapes whose x extent fills whole 64-wide warps take the vector path
    of the default kernel; all variants must equal the oracle bit for bit."""
    u0 = workloads.jacobi_initial(shape[2], shape[1], shape[0], seed=13)
    with lgd.Grid(lgd.CELL_JACOBI7_F64, shape, periodic=periodic, edge=(0.5, 0, 0, 0)) as g:
        _set_variant(g, variant)
        g.upload(0, u0)
        g.step(5)
        out = g.download(0)
    np.testing.assert_array_equal(out, oracle.jacobi7(u0, 5, torus=periodic == 7, edge=0.5))


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_jacobi7_fixed_point_variants_identical(variant):
    """Single-step kernels of the fixed-point cell (one step per pass: the
    fused two-step pass rounds once and is checked separately)."""
    u0 = workloads.jacobi_initial(128, 24, 40, seed=14)
    with lgd.Grid(lgd.CELL_JACOBI7_F64_FIX, u0.shape) as g:
        _set_variant(g, variant)
        g.set_time_block(1)
        g.upload(0, u0)
        g.step(6)
        out = g.download(0)
    with lgd.Grid(lgd.CELL_JACOBI7_F64_FIX, u0.shape) as g:
        _set_variant(g, 1)
        g.upload(0, u0)
        g.step(6)
        ref = g.download(0)
    np.testing.assert_array_equal(out, ref)


TMA_SHAPES = [(9, 20, 128), (70, 16, 64), (1, 8, 192), (33, 13, 130), (17, 7, 96), (2, 1, 37), (5, 40, 70),
              (3, 17, 1), (40, 33, 65)]


@pytest.mark.parametrize("shape", TMA_SHAPES)
def test_jacobi7_tma_kernel_bit_exact_fp64(shape):
    """Cube grids with a zero edge cell run the TMA-staged kernel (variant 0):
    ragged tiles in x and y, z chunks of one or a few planes."""
    u0 = workloads.jacobi_initial(shape[2], shape[1], shape[0], seed=17)
    out = run_grid(lgd.CELL_JACOBI7_F64, [u0], 7)
    np.testing.assert_array_equal(out, oracle.jacobi7(u0, 7))


@pytest.mark.parametrize("shape", TMA_SHAPES)
@pytest.mark.parametrize("cell", [lgd.CELL_JACOBI7_F64_FIX, lgd.CELL_JACOBI7_F32])
def test_jacobi7_tma_kernel_equals_register_kernel(shape, cell):
    u0 = workloads.jacobi_initial(shape[2], shape[1], shape[0], seed=18)
    if cell == lgd.CELL_JACOBI7_F32:
        u0 = u0.astype(np.float32)
    res = []
    for variant in (0, 5):
        with lgd.Grid(cell, shape) as g:
            _set_variant(g, variant)
            g.set_time_block(1)           # the single-step TMA kernel against the register kernel
            g.upload(0, u0)
            g.step(7)
            res.append(g.download(0))
    np.testing.assert_array_equal(res[0], res[1])


# ------------------------------------------------------ temporal blocking
TB_SHAPES = [(9, 20, 128), (70, 16, 64), (33, 61, 130), (5, 40, 70), (2, 1, 37), (1, 8, 192), (40, 33, 65),
             (3, 17, 1), (12, 70, 250)]


def _run_blocked(cell, u0, steps, depth, shape=0):
    with lgd.Grid(cell, u0.shape) as g:
        g.set_time_block(depth)
        g.set_time_block_shape(shape)
        g.upload(0, u0)
        before = g.launch_count()
        g.step(steps)
        passes = g.launch_count() - before
        return g.download(0), passes


FIX_UNIT = 2.0 ** -57          # one unit of the fixed-point grid for values in [0, 1)


def _depth(cell, depth):
    """Depth a request runs at: the fixed-point cell fuses at most two."""
    return min(depth, 2) if cell == lgd.CELL_JACOBI7_F64_FIX else depth


def _passes(steps, depth):
    """Launches of `steps` steps at blocking depth `depth`: full passes, one
    shorter pass for a remainder of two or more, a single step otherwise."""
    if depth <= 1:
        return steps
    full, rem = divmod(steps, depth)
    return full + (1 if rem >= 2 else rem)


def _assert_blocked_matches(cell, out, ref, passes):
    """FP32: fused passes are bit-identical to single steps.  Fixed point: a
    two-step pass rounds once (round of the exact two-step average) where
    two single steps round twice; the two differ by at most one unit per
    pass (plus one when a later single step rounds the difference up), and
    the averaging never amplifies a difference.  The grids are compared as
    downloaded FP64 values, which round the 57-bit grid to 53 bits: one more
    ulp of the value."""
    if cell == lgd.CELL_JACOBI7_F32:
        np.testing.assert_array_equal(out, ref)
    else:
        bound = (passes + 1) * FIX_UNIT + np.spacing(np.maximum(np.abs(out), np.abs(ref)))
        excess = np.abs(out - ref) - bound
        assert np.all(excess <= 0), np.max(np.abs(out - ref)) / FIX_UNIT


@pytest.mark.parametrize("grid_shape", TB_SHAPES)
@pytest.mark.parametrize("cell", [lgd.CELL_JACOBI7_F64_FIX, lgd.CELL_JACOBI7_F32])
@pytest.mark.parametrize("depth", [2, 3, 4])
def test_temporal_blocking_matches_single_steps(grid_shape, cell, depth):
    """depth steps per pass over memory (intermediate levels on chip) give
    the single-step results (FP32 bit for bit, fixed point within one unit
    per pass): ragged tiles in x and y, z chunks, degenerate axes, a step
    count that leaves a remainder pass."""
    u0 = workloads.jacobi_initial(grid_shape[2], grid_shape[1], grid_shape[0], seed=23)
    if cell == lgd.CELL_JACOBI7_F32:
        u0 = u0.astype(np.float32)
    steps = 2 * depth + 1 + (depth > 2)
    ref, n_ref = _run_blocked(cell, u0, steps, 1)
    assert n_ref == steps
    out, n = _run_blocked(cell, u0, steps, depth)
    assert n == _passes(steps, _depth(cell, depth))
    _assert_blocked_matches(cell, out, ref, n)


@pytest.mark.parametrize("cell,depth,shape", [(lgd.CELL_JACOBI7_F64_FIX, 2, 0), (lgd.CELL_JACOBI7_F64_FIX, 2, 1),
                                              (lgd.CELL_JACOBI7_F64_FIX, 2, 2), (lgd.CELL_JACOBI7_F32, 4, 1),
                                              (lgd.CELL_JACOBI7_F32, 4, 2), (lgd.CELL_JACOBI7_F32, 3, 1),
                                              (lgd.CELL_JACOBI7_F32, 3, 2), (lgd.CELL_JACOBI7_F32, 2, 1),
                                              (lgd.CELL_JACOBI7_F32, 2, 2)])
@pytest.mark.parametrize("grid_shape", [(33, 61, 130), (70, 16, 64), (2, 1, 37), (12, 70, 250)])
def test_temporal_blocking_box_shapes(cell, depth, shape, grid_shape):
    u0 = workloads.jacobi_initial(grid_shape[2], grid_shape[1], grid_shape[0], seed=29)
    if cell == lgd.CELL_JACOBI7_F32:
        u0 = u0.astype(np.float32)
    steps = 3 * depth
    ref, _ = _run_blocked(cell, u0, steps, 1)
    out, n = _run_blocked(cell, u0, steps, depth, shape)
    assert n == 3
    _assert_blocked_matches(cell, out, ref, n)


def test_temporal_blocking_fixed_point_shapes_identical():
    """The box shape does not change a fixed-point result."""
    u0 = workloads.jacobi_initial(130, 61, 33, seed=31)
    outs = [_run_blocked(lgd.CELL_JACOBI7_F64_FIX, u0, 8, 2, shape)[0] for shape in (0, 1, 2)]
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])


def test_temporal_blocking_fixed_point_128_config_within_1e12():
    """The Jacobi configuration (128^3, 100 steps) at every blocking depth:
    within 1e-12 of the reference's FP64 result."""
    g = load("jacobi7_cube_128")
    u0 = workloads.jacobi_initial(128, 128, 128, seed=42)
    ref = oracle.jacobi7(u0, 100)
    assert sha(ref) == str(g["sha256"])
    outs = [_run_blocked(lgd.CELL_JACOBI7_F64_FIX, u0, 100, d)[0] for d in (1, 2, 3, 4)]
    for o in outs:
        assert rel_err(o, ref) <= 1e-12
    for o in outs[2:]:                       # depths 3 and 4 run as passes of two
        np.testing.assert_array_equal(o, outs[1])


def test_temporal_blocking_default_depth_and_limits():
    u0 = workloads.jacobi_initial(64, 32, 16, seed=3)
    with lgd.Grid(lgd.CELL_JACOBI7_F32, u0.shape) as g:
        g.upload(0, u0.astype(np.float32))
        before = g.launch_count()
        g.step(10)
        assert g.launch_count() - before == 4          # FP32 default depth 3: 3 + 3 + 3 + 1
    with lgd.Grid(lgd.CELL_JACOBI7_F64_FIX, u0.shape) as g:
        g.upload(0, u0)
        before = g.launch_count()
        g.step(10)
        assert g.launch_count() - before == 5          # fixed point default: passes of two
        with pytest.raises(lgd.LGDError):
            g.set_time_block(lgd.TB_MAX_DEPTH + 1)
        with pytest.raises(lgd.LGDError):
            g.set_time_block_shape(3)
    with lgd.Grid(lgd.CELL_JACOBI7_F64, u0.shape) as g:     # IEEE FP64: one step per pass
        g.set_time_block(4)
        g.upload(0, u0)
        before = g.launch_count()
        g.step(8)
        assert g.launch_count() - before == 8
        np.testing.assert_array_equal(g.download(0), oracle.jacobi7(u0, 8))


# ------------------------------------- Game of Life, generations per pass
GOL_TB_GRIDS = [(16, 16), (32, 48), (40, 8192), (7, 64), (33, 480), (100, 496), (257, 1024), (3, 32)]


GOL_BIT_DEPTHS = (2, 4, 6, 8, 12, 16, 24, 32)
GOL_BYTE_DEPTHS = (2, 4, 6, 8, 12)


def _gol_passes(steps, depth, nx, variant=0):
    """Launches of the Game of Life path: passes of the largest compiled
    depth not above min(depth, steps left) - bit-sliced passes for rows of a
    multiple of 32 cells, byte passes otherwise or under variant 1 - and
    single generations for a remainder of one."""
    depths = GOL_BIT_DEPTHS if (nx % 32 == 0 and variant == 0) else GOL_BYTE_DEPTHS
    n = 0
    while steps >= 2:
        d = max(k for k in depths if k <= min(depth, steps))
        steps -= d
        n += 1
    return n + steps


@pytest.mark.parametrize("grid", GOL_TB_GRIDS)
@pytest.mark.parametrize("depth,variant", [(2, 0), (4, 0), (6, 0), (8, 0), (12, 0), (16, 0), (24, 0), (32, 0),
                                           (4, 1), (12, 1)])
def test_gol_generations_per_pass_bit_identical(grid, depth, variant):
    """Several generations per pass over memory (each warp marches down a
    strip, generations skewed in registers, halo lanes or words wrapped
    around the torus) give exactly the single-generation results: grids
    narrower than a warp, shorter than the depth, wide ragged rows, in the
    bit-sliced passes (rows of a multiple of 32 cells) and the byte passes
    (variant 1, or rows of a multiple of 16)."""
    c0 = workloads.gol_initial(grid[1], grid[0], seed=41)
    steps = 2 * depth + 3
    res = []
    for d in (1, depth):
        with lgd.Grid(lgd.CELL_GOL_U8, c0.shape, periodic=3) as g:
            g.set_time_block(d)
            g.set_variant(variant)
            g.upload(0, c0)
            before = g.launch_count()
            g.step(steps)
            launches = g.launch_count() - before
            res.append(g.download(0))
        assert launches == (steps if d == 1 else _gol_passes(steps, d, grid[1], variant))
    np.testing.assert_array_equal(res[1], res[0])
    np.testing.assert_array_equal(res[0], oracle.gol(c0, steps))


@pytest.mark.parametrize("shape", [1, 2])
def test_gol_strip_shapes_identical(shape):
    c0 = workloads.gol_initial(2048, 300, seed=43)
    out = []
    for s in (0, shape):
        with lgd.Grid(lgd.CELL_GOL_U8, c0.shape, periodic=3) as g:
            g.set_time_block(8)
            g.set_time_block_shape(s)
            g.upload(0, c0)
            g.step(40)
            out.append(g.download(0))
    np.testing.assert_array_equal(out[0], out[1])
