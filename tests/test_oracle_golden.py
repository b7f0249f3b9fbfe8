"""Pin the CPU oracle to the reference.

The fixtures in tests/golden/ were written by running the reference's own
SerialSimulator / SELL-C-sigma container (tests/golden/gen_golden.py); the
oracle must reproduce them bit for bit.  The SELL known-answer values are
the ones the reference's container test asserts
(storage/test/unit/sellcsigmasparsematrixcontainertest.h:602-888).
"""
import hashlib
import os

import numpy as np
import pytest

import oracle
from libgeodecomp_gb300 import workloads

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name + ".npz"), allow_pickle=False)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["jacobi7_cube_24x20x16", "jacobi7_torus_17x13x11"])
def test_jacobi7_small_bit_exact(name):
    g = load(name)
    nz, ny, nx = g["shape"]
    u0 = workloads.jacobi_initial(nx, ny, nz, seed=int(g["seed"]))
    assert sha(u0) == str(g["u0_sha256"])
    out = oracle.jacobi7(u0, int(g["steps"]), torus=bool(g["torus"]))
    np.testing.assert_array_equal(out, g["out"])


def test_jacobi7_128_config_bit_exact():
    g = load("jacobi7_cube_128")
    u0 = workloads.jacobi_initial(128, 128, 128, seed=42)
    assert sha(u0) == str(g["u0_sha256"])
    out = oracle.jacobi7(u0, 100)
    assert sha(out) == str(g["sha256"])
    np.testing.assert_array_equal(out.reshape(-1)[g["sample_idx"]], g["sample"])


def test_gol_small_bit_exact():
    g = load("gol_64x48")
    ny, nx = g["shape"]
    c0 = workloads.gol_initial(nx, ny, seed=42)
    assert sha(c0) == str(g["c0_sha256"])
    np.testing.assert_array_equal(oracle.gol(c0, int(g["steps"])), g["out"])


def test_gol_1024_1000_steps():
    g = load("gol_1024")
    c0 = workloads.gol_initial(1024, 1024, seed=42)
    out = oracle.gol(c0, 1000)
    np.testing.assert_array_equal(out.sum(axis=1), g["row_alive"])
    assert sha(out) == str(g["sha256"])


def _sell_cases():
    g = load("sell_build")
    return g, [str(t) for t in g["tags"]]


@pytest.mark.parametrize("tag", _sell_cases()[1])
def test_sell_build_matches_reference(tag):
    g, _ = _sell_cases()
    n = int(g[tag + "__n"])
    C = int(g[tag + "__C"])
    sigma = int(g[tag + "__sigma"])
    mode = str(g[tag + "__mode"])
    s = oracle.sell_build(n, g[tag + "__row_ptr"], g[tag + "__col"], g[tag + "__w"], C, sigma,
                          remap_columns=(mode == "grid"))
    for key in ("perm", "chunk_offset", "chunk_length", "row_length", "values", "column"):
        np.testing.assert_array_equal(s[key], g[tag + "__" + key], err_msg=key)


def test_sell_container_known_answers():
    """Literal expectations of the reference's container test."""
    g, _ = _sell_cases()

    def build(tag):
        return oracle.sell_build(int(g[tag + "__n"]), g[tag + "__row_ptr"], g[tag + "__col"], g[tag + "__w"],
                                 int(g[tag + "__C"]), int(g[tag + "__sigma"]), remap_columns=False)

    s = build("kat4_c2s1")  # testInitFromMatrix
    assert list(s["chunk_offset"]) == [0, 4, 8]
    assert list(s["chunk_length"]) == [2, 2]
    assert list(s["values"]) == [1, 1, 2, 0, 2, 1, 3, 1]
    assert list(s["column"]) == [1, 3, 3, 0, 1, 0, 3, 1]
    s = build("kat5_c2s1")  # testInitFromMatrixWithoutSIGMA
    assert list(s["chunk_offset"]) == [0, 6, 14, 18]
    assert list(s["chunk_length"]) == [3, 4, 2]
    s = build("kat5_c2s4")  # testInitFromMatrixWithSIGMA1
    assert list(s["chunk_offset"]) == [0, 8, 10, 14]
    assert list(s["chunk_length"]) == [4, 1, 2]
    s = build("kat5_c2s8")  # testInitFromMatrixWithSIGMA2
    assert list(s["chunk_offset"]) == [0, 8, 12, 14]
    assert list(s["chunk_length"]) == [4, 2, 1]


def _sell_run(n, C, sigma, steps, seed):
    rp, col, w = workloads.powerlaw_graph(n, seed=seed)
    x0 = workloads.sell_values(n, seed=seed)
    s = oracle.sell_build(n, rp, col, w, C, sigma)
    x = oracle.sell_diffusion(s, C, x0[s["perm"]], steps)
    out = np.empty_like(x)
    out[s["perm"]] = x
    return x0, w, out


def test_sell_diffusion_2000_bit_exact():
    g = load("sell_diffusion_2000")
    x0, w, out = _sell_run(2000, 32, 256, int(g["steps"]), int(g["seed"]))
    assert sha(x0) == str(g["x0_sha256"]) and sha(w) == str(g["w_sha256"])
    np.testing.assert_array_equal(out, g["out"])


def test_sell_diffusion_100k():
    g = load("sell_diffusion_100k")
    x0, w, out = _sell_run(100000, 32, 256, int(g["steps"]), int(g["seed"]))
    assert sha(x0) == str(g["x0_sha256"]) and sha(w) == str(g["w_sha256"])
    np.testing.assert_array_equal(out[g["sample_idx"]], g["sample"])
    assert sha(out) == str(g["sha256"])


def test_lbm_small_bit_exact():
    g = load("lbm_L8")
    out = oracle.lbm(int(g["L"]), int(g["steps"]), float(g["omega"]), float(g["lid"]))
    np.testing.assert_array_equal(out, g["out"])


def test_lbm_24():
    g = load("lbm_L24")
    out = oracle.lbm(int(g["L"]), int(g["steps"]), float(g["omega"]), float(g["lid"]))
    np.testing.assert_array_equal(out.reshape(-1)[g["sample_idx"]], g["sample"])
    assert sha(out) == str(g["sha256"])


def test_varcoef_small_bit_exact():
    g = load("varcoef_16")
    out = oracle.varcoef(g["u0"], g["k"], int(g["steps"]))
    np.testing.assert_array_equal(out, g["out"])


def test_oracle_thread_count_does_not_change_results():
    u0 = workloads.jacobi_initial(33, 17, 9, seed=3)
    a = oracle.jacobi7(u0, 5, threads=1)
    b = oracle.jacobi7(u0, 5, threads=4)
    np.testing.assert_array_equal(a, b)


def test_bov_fixture_matches_oracle_and_format():
    """The reference's SerialBOVWriter files: data = the oracle's Jacobi
    grid at steps 0 and 6, header in the documented BOV layout."""
    g = np.load(os.path.join(GOLD, "bov_jacobi_24x20x16.npz"))
    nz, ny, nx = (int(v) for v in g["shape"])
    u0 = workloads.jacobi_initial(nx, ny, nz, seed=42)
    for step in (0, int(g["steps"])):
        data = np.frombuffer(bytes(g["data_%d" % step]), dtype=np.float64).reshape(nz, ny, nx)
        np.testing.assert_array_equal(data, oracle.jacobi7(u0, step))
        header = bytes(g["bov_%d" % step]).decode()
        assert header.startswith("TIME: %d\nDATA_FILE: jac.%05d.data\nDATA_SIZE: %d %d %d\n" % (step, step, nx, ny, nz))
        assert "DATA_FORMAT: DOUBLE\nVARIABLE: temp\n" in header


def _edge_cases():
    g = load("edge_shapes")
    return sorted(k for k in g.files if k not in ("steps", "seed"))


@pytest.mark.parametrize("key", _edge_cases())
def test_edge_shapes_bit_exact(key):
    """Degenerate and odd shapes - axes of extent 1 and 2, boxes that are
    all wall cells, node counts that are not multiples of C or sigma - as
    the reference computes them (tests/golden/gen_golden.py edge_shapes)."""
    g = load("edge_shapes")
    steps, seed = int(g["steps"]), int(g["seed"])
    kind, dims = key.rsplit("_", 1)
    dims = [int(d) for d in dims.split("x")]
    want = g[key]
    if kind in ("jacobi_cube", "jacobi_torus"):
        nx, ny, nz = dims
        got = oracle.jacobi7(workloads.jacobi_initial(nx, ny, nz, seed=seed), steps, torus=kind == "jacobi_torus")
    elif kind == "gol":
        nx, ny = dims
        got = oracle.gol(workloads.gol_initial(nx, ny, seed=seed), steps)
    elif kind == "lbm":
        got = oracle.lbm(dims[0], steps, 1.5, 0.05)
    elif kind == "varcoef":
        nx, ny, nz = dims
        n = nx * ny * nz
        u0 = workloads.uniform(seed, workloads.STREAM_GRID, n).reshape(nz, ny, nx)
        k = 0.02 + 0.13 * workloads.uniform(seed, workloads.STREAM_DEGREE, n).reshape(nz, ny, nx)
        got = oracle.varcoef(u0, k, steps)
    elif kind == "sell":
        n, C, sigma = dims
        got = _sell_run(n, C, sigma, steps, seed)[2]
    else:
        raise AssertionError("unknown fixture " + key)
    assert got.shape == want.shape
    np.testing.assert_array_equal(got, want)
