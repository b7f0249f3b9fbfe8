"""The SELL-C-sigma matrix built on the GPU (lgd_sell_create_from_csr) is
byte-identical to the reference's arrays (fixtures written by the
reference's ReorderingUnstructuredGrid, tests/golden/gen_golden.py) and to
the host builder, from host or device CSR input, and a grid built either
way steps identically.  Bad input is rejected with the host builder's
status codes; sizes beyond the device path's limits say so."""
import os

import numpy as np
import pytest

from libgeodecomp_gb300 import lgd, workloads

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KEYS = ("perm", "chunk_offset", "row_length", "values", "column")


def golden():
    g = np.load(os.path.join(GOLD, "sell_build.npz"))
    return g, [str(t) for t in g["tags"] if str(g[str(t) + "__mode"]) == "grid"]


def assert_same_layout(a, b):
    for key in KEYS:
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)


@pytest.mark.parametrize("tag", golden()[1])
def test_device_builder_matches_reference_arrays(tag):
    g, _ = golden()
    n, C, sigma = int(g[tag + "__n"]), int(g[tag + "__C"]), int(g[tag + "__sigma"])
    with lgd.SellGrid.from_csr(n, g[tag + "__row_ptr"], g[tag + "__col"], g[tag + "__w"], C, sigma) as s:
        got = s.layout()
    ref = {k: g[tag + "__" + k] for k in KEYS}
    assert_same_layout(got, ref)


@pytest.mark.parametrize("n,C,sigma", [(5000, 32, 256), (4097, 32, 1), (1000, 8, 16), (333, 4, 60), (777, 1, 5),
                                       (3000, 64, 4096), (200000, 32, 256), (65, 32, 4096)])
def test_device_builder_matches_host_builder(n, C, sigma):
    rp, col, w = workloads.powerlaw_graph(n, seed=n + 1)
    host = lgd.sell_build(n, rp, col, w, C, sigma)
    with lgd.SellGrid.from_csr(n, rp, col, w, C, sigma) as s:
        assert_same_layout(s.layout(), host)


def test_device_builder_ragged_rows_duplicates_and_empty_rows():
    rng = np.random.default_rng(3)
    n = 4099
    deg = rng.integers(0, 40, n)
    deg[::7] = 0
    rp = np.concatenate([[0], np.cumsum(deg)]).astype(np.int64)
    col = rng.integers(0, 50, int(rp[-1])).astype(np.int32)      # many repeated columns per row
    w = rng.random(int(rp[-1]))
    for C, sigma in ((32, 256), (4, 60), (8, 1)):
        host = lgd.sell_build(n, rp, col, w, C, sigma)
        with lgd.SellGrid.from_csr(n, rp, col, w, C, sigma) as s:
            assert_same_layout(s.layout(), host)


def test_device_input_matches_host_input():
    torch = pytest.importorskip("torch")
    n = 20000
    rp, col, w = workloads.powerlaw_graph(n, seed=9)
    with lgd.SellGrid.from_csr(n, rp, col, w, 32, 256) as a:
        la = a.layout()
    trp = torch.tensor(rp, dtype=torch.int64, device="cuda")
    tcol = torch.tensor(col, dtype=torch.int32, device="cuda")
    tw = torch.tensor(w, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    with lgd.SellGrid.from_csr(n, trp, tcol, tw, 32, 256, device=True) as b:
        assert_same_layout(b.layout(), la)


@pytest.mark.parametrize("precision,exact", [(8, True), (8, False), (4, False)])
def test_grids_built_either_way_step_identically(precision, exact):
    n = 30000
    rp, col, w = workloads.powerlaw_graph(n, seed=4)
    x0 = workloads.sell_values(n, seed=4)
    host = lgd.sell_build(n, rp, col, w, 32, 256)
    out = []
    for g in (lgd.SellGrid(host, precision=precision, exact=exact),
              lgd.SellGrid.from_csr(n, rp, col, w, 32, 256, precision=precision, exact=exact)):
        with g:
            g.upload(x0)
            g.step(7)
            out.append(g.download())
    np.testing.assert_array_equal(out[0], out[1])


def test_device_builder_rejects_bad_input_and_states_its_limits():
    rp = np.array([0, 1, 2], dtype=np.int64)
    with pytest.raises(lgd.LGDError) as e:
        lgd.SellGrid.from_csr(2, rp, np.array([0, 5], dtype=np.int32), np.ones(2), 2, 1)
    assert e.value.code == lgd.ERR_RANGE
    with pytest.raises(lgd.LGDError) as e:
        lgd.SellGrid.from_csr(2, np.array([0, 2, 1], dtype=np.int64), np.array([0, 1], dtype=np.int32), np.ones(2), 2, 1)
    assert e.value.code == lgd.ERR_INVALID
    with pytest.raises(lgd.LGDError) as e:
        lgd.SellGrid.from_csr(10, np.arange(11, dtype=np.int64), np.zeros(10, dtype=np.int32), np.ones(10), 2,
                              lgd.SELL_GPU_MAX_SIGMA + 1)
    assert e.value.code == lgd.ERR_UNSUPPORTED
    d = lgd.SELL_GPU_MAX_ROW + 1
    with pytest.raises(lgd.LGDError) as e:
        lgd.SellGrid.from_csr(2, np.array([0, d, d], dtype=np.int64), np.zeros(d, dtype=np.int32), np.ones(d), 2, 1)
    assert e.value.code == lgd.ERR_UNSUPPORTED
