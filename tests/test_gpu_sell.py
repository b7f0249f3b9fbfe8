"""SELL-C-sigma diffusion x' = 0.1 x + W x on the GPU, through the C ABI.

LGD_SELL_EXACT (separate multiply and add) must match the reference's
SerialSimulator bit for bit; the default fused kernel must stay within 1e-12
relative; FP32 states its error against FP64.  Partial-chunk row ranges
restate the reference's loop-peeling cases
(storage/test/unit/unstructuredupdatefunctortest.h:416-422).
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


def gpu_run(n, seed, steps, C=32, sigma=256, precision=8, exact=False, variant=0):
    rp, col, w = workloads.powerlaw_graph(n, seed=seed)
    x0 = workloads.sell_values(n, seed=seed)
    s = lgd.sell_build(n, rp, col, w, C, sigma)
    with lgd.SellGrid(s, precision=precision, exact=exact) as g:
        g.set_variant(variant)
        g.upload(x0)
        g.step(steps)
        return g.download(), s, x0


def rel_err(a, b):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def test_sell_exact_bit_identical_to_reference():
    g = load("sell_diffusion_2000")
    out, _, x0 = gpu_run(2000, int(g["seed"]), int(g["steps"]), exact=True)
    assert sha(x0) == str(g["x0_sha256"])
    np.testing.assert_array_equal(out, g["out"])


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5])
def test_sell_exact_every_kernel_variant_bit_identical(variant):
    g = load("sell_diffusion_2000")
    out, _, _ = gpu_run(2000, int(g["seed"]), int(g["steps"]), exact=True, variant=variant)
    np.testing.assert_array_equal(out, g["out"])


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5])
def test_sell_fused_within_1e12_of_reference(variant):
    g = load("sell_diffusion_2000")
    out, _, _ = gpu_run(2000, int(g["seed"]), int(g["steps"]), variant=variant)
    assert rel_err(out, g["out"]) <= 1e-12


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5])
def test_sell_ragged_rows_every_variant(variant):
    # rows of length 0 .. 9 (every residue of the pipeline depth), C = 8
    rng = np.random.default_rng(5)
    n = 300
    deg = rng.integers(0, 10, size=n)
    rp = np.zeros(n + 1, dtype=np.int64)
    rp[1:] = np.cumsum(deg)
    col = rng.integers(0, n, size=int(rp[-1])).astype(np.int32)
    w = rng.random(int(rp[-1]))
    x0 = rng.random(n)
    s = lgd.sell_build(n, rp, col, w, 8, 32)
    with lgd.SellGrid(s, exact=True) as g:
        g.set_variant(variant)
        g.upload(x0)
        g.step(3)
        out = g.download()
    s_ref = oracle.sell_build(n, rp, col, w, 8, 32)
    ref = oracle.sell_diffusion(s_ref, 8, x0[s_ref["perm"]], 3)
    np.testing.assert_array_equal(out[s_ref["perm"]], ref)


def test_sell_100k_golden():
    g = load("sell_diffusion_100k")
    out, _, _ = gpu_run(100000, int(g["seed"]), int(g["steps"]), exact=True)
    np.testing.assert_array_equal(out[g["sample_idx"]], g["sample"])
    assert sha(out) == str(g["sha256"])


@pytest.mark.parametrize("C,sigma", [(32, 1), (8, 16), (4, 60), (1, 1)])
def test_sell_other_chunk_shapes_match_oracle(C, sigma):
    n = 3001
    out, s, x0 = gpu_run(n, 3, 7, C=C, sigma=sigma, exact=True)
    so = oracle.sell_build(n, *workloads.powerlaw_graph(n, seed=3), C, sigma)
    ref = oracle.sell_diffusion(so, C, x0[so["perm"]], 7)
    exp = np.empty(n)
    exp[so["perm"]] = ref
    np.testing.assert_array_equal(out, exp)


@pytest.mark.parametrize("begin,end", [(0, 32), (5, 77), (31, 33), (100, 2000), (1999, 2000), (7, 7)])
def test_sell_row_range_updates_peel_partial_chunks(begin, end):
    n = 2000
    rp, col, w = workloads.powerlaw_graph(n, seed=21)
    x0 = workloads.sell_values(n, seed=21)
    s = lgd.sell_build(n, rp, col, w, 32, 256)
    xp = x0[s["perm"]]
    full = oracle.sell_diffusion(s, 32, xp, 1)
    with lgd.SellGrid(s, exact=True) as g:
        g.upload(xp, logical=False)
        g.upload(np.full(n, -7.0), logical=False, which=1)
        g.update_rows(begin, end)
        g.swap()
        got = g.download(logical=False)
    exp = np.full(n, -7.0)
    exp[begin:end] = full[begin:end]
    np.testing.assert_array_equal(got, exp)


def test_sell_reference_kat_weights():
    """w(row, col) = row + 10 col and value = 2000 + i, as in the reference's
    unstructured update functor test (storage/test/unit/
    unstructuredupdatefunctortest.h:166-300), on a banded matrix whose sums
    are exact in FP64."""
    n = 150
    rows, cols, ws = [], [], []
    rp = [0]
    for r in range(n):
        for c in range(r, min(n, r + 1 + (r % 5))):
            cols.append(c)
            ws.append(float(r + 10 * c))
        rp.append(len(cols))
    rp = np.array(rp, dtype=np.int64)
    col = np.array(cols, dtype=np.int32)
    w = np.array(ws)
    x0 = 2000.0 + np.arange(n)
    s = lgd.sell_build(n, rp, col, w, 4, 1)
    with lgd.SellGrid(s, exact=True) as g:
        g.upload(x0)
        g.step(1)
        got = g.download()
    exp = np.array([0.1 * x0[r] + sum(x0[col[k]] * w[k] for k in range(rp[r], rp[r + 1])) for r in range(n)])
    np.testing.assert_array_equal(got, exp)


def test_sell_fp32_error_against_fp64():
    n = 50000
    out32, _, _ = gpu_run(n, 4, 50, precision=4)
    out64, _, _ = gpu_run(n, 4, 50, exact=True)
    rel_l2 = np.linalg.norm(out32 - out64) / np.linalg.norm(out64)
    # measured on GB300 and stated in the design notes
    assert rel_l2 < 1e-5, rel_l2


def test_sell_config_size_against_oracle():
    """N = 4,194,304 nodes, C = 32, sigma = 256, power-law degrees on
    [4, 64]: 50 steps of the fused kernel within 1e-12 of the oracle."""
    n = 4194304
    rp, col, w = workloads.powerlaw_graph(n, seed=42)
    x0 = workloads.sell_values(n, seed=42)
    s = lgd.sell_build(n, rp, col, w, 32, 256)
    with lgd.SellGrid(s) as g:
        g.upload(x0)
        g.step(50)
        out = g.download()
    ref_phys = oracle.sell_diffusion(s, 32, x0[s["perm"]], 50)
    ref = np.empty(n)
    ref[s["perm"]] = ref_phys
    assert rel_err(out, ref) <= 1e-12


def test_sell_rejects_bad_arguments():
    n = 64
    rp, col, w = workloads.powerlaw_graph(n, seed=1, dmax=16)
    s = lgd.sell_build(n, rp, col, w, 32, 1)
    with lgd.SellGrid(s) as g:
        with pytest.raises(lgd.LGDError) as e:
            g.update_rows(10, 65)
        assert e.value.code == lgd.ERR_RANGE
        a = np.zeros(n + 1)
        with pytest.raises(lgd.LGDError) as e:
            lgd.check(lgd.lib().lgd_sell_upload_x(g._h, 0, 1, lgd._ptr(a), a.nbytes))
        assert e.value.code == lgd.ERR_INVALID


# ------------------------------------------------ reverse Cuthill-McKee
@pytest.mark.parametrize("exact,precision", [(True, 8), (False, 8), (False, 4)])
def test_renumbered_grid_agrees_to_rounding(exact, precision):
    """LGD_SELL_RENUMBER builds the matrix on RCM node numbers.  The
    container orders a row's entries by physical column (the reference's
    layout), so the renumbered grid adds each row's terms in another order:
    every node's value (in the caller's logical order) agrees with the plain
    grid's to a few units in the last place - on the power-law graph and on
    a randomly numbered periodic 3D mesh."""
    from test_graph_rcm import permuted_mesh
    n1 = 36
    n_mesh, rp_mesh, col_mesh = permuted_mesh(n1, seed=8)
    w_mesh = np.random.default_rng(9).random(col_mesh.size) * (0.9 / 6.0)
    n_pl = 60013
    rp_pl, col_pl, w_pl = workloads.powerlaw_graph(n_pl, seed=13)
    for n, rp, col, w in ((n_pl, rp_pl, col_pl, w_pl), (n_mesh, rp_mesh, col_mesh, w_mesh)):
        x0 = workloads.sell_values(n, seed=5)
        out = []
        for renumber in (False, True):
            with lgd.SellGrid.from_csr(n, rp, col, w, 32, 256, precision=precision, exact=exact,
                                       renumber=renumber) as g:
                g.upload(x0)
                g.step(7)
                out.append(g.download())
        tol = 1e-12 if precision == 8 else 1e-5
        assert np.max(np.abs(out[1] - out[0]) / np.abs(out[0])) <= tol


def test_renumbering_needs_host_arrays():
    torch = pytest.importorskip("torch")
    rp, col, w = workloads.powerlaw_graph(1000, seed=1)
    t = [torch.as_tensor(a, device="cuda") for a in (rp, col.astype(np.int32), w)]
    with pytest.raises(lgd.LGDError):
        lgd.SellGrid.from_csr(1000, t[0], t[1], t[2], 32, 256, device=True, renumber=True)
