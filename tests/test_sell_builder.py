"""The library's host-side SELL-C-sigma builder reproduces the arrays the
reference builds (fixtures from the reference's own
ReorderingUnstructuredGrid / SellCSigmaSparseMatrixContainer, written by
tests/golden/gen_golden.py), including the reference container test's
known answers (storage/test/unit/sellcsigmasparsematrixcontainertest.h:
602-888).  Host code only: no GPU needed."""
import os

import numpy as np
import pytest

import oracle
from libgeodecomp_gb300 import lgd, workloads

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


def cases():
    g = np.load(os.path.join(GOLD, "sell_build.npz"))
    return g, [str(t) for t in g["tags"]]


@pytest.mark.parametrize("tag", cases()[1])
def test_builder_matches_reference_arrays(tag):
    g, _ = cases()
    s = lgd.sell_build(int(g[tag + "__n"]), g[tag + "__row_ptr"], g[tag + "__col"], g[tag + "__w"],
                       int(g[tag + "__C"]), int(g[tag + "__sigma"]), remap_columns=str(g[tag + "__mode"]) == "grid")
    for key in ("perm", "chunk_offset", "chunk_length", "row_length", "values", "column"):
        np.testing.assert_array_equal(s[key], g[tag + "__" + key], err_msg=key)


def test_builder_known_answers():
    g, _ = cases()
    s = lgd.sell_build(4, g["kat4_c2s1__row_ptr"], g["kat4_c2s1__col"], g["kat4_c2s1__w"], 2, 1, remap_columns=False)
    assert list(s["chunk_offset"]) == [0, 4, 8]
    assert list(s["chunk_length"]) == [2, 2]
    assert list(s["values"]) == [1, 1, 2, 0, 2, 1, 3, 1]
    assert list(s["column"]) == [1, 3, 3, 0, 1, 0, 3, 1]
    s = lgd.sell_build(5, g["kat5_c2s4__row_ptr"], g["kat5_c2s4__col"], g["kat5_c2s4__w"], 2, 4, remap_columns=False)
    assert list(s["chunk_offset"]) == [0, 8, 10, 14]
    s = lgd.sell_build(5, g["kat5_c2s8__row_ptr"], g["kat5_c2s8__col"], g["kat5_c2s8__w"], 2, 8, remap_columns=False)
    assert list(s["chunk_offset"]) == [0, 8, 12, 14]


@pytest.mark.parametrize("n,C,sigma", [(5000, 32, 256), (4097, 32, 1), (1000, 8, 16), (333, 4, 60)])
def test_builder_matches_oracle_on_powerlaw_graphs(n, C, sigma):
    rp, col, w = workloads.powerlaw_graph(n, seed=n)
    a = lgd.sell_build(n, rp, col, w, C, sigma)
    b = oracle.sell_build(n, rp, col, w, C, sigma)
    for key in ("perm", "chunk_offset", "chunk_length", "row_length", "values", "column"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)


def test_builder_rejects_bad_input():
    rp = np.array([0, 1, 2], dtype=np.int64)
    with pytest.raises(lgd.LGDError) as e:
        lgd.sell_build(2, rp, np.array([0, 5], dtype=np.int32), np.ones(2), 2, 1)
    assert e.value.code == lgd.ERR_RANGE
    with pytest.raises(lgd.LGDError):
        lgd.sell_build(2, np.array([0, 2, 1], dtype=np.int64), np.array([0, 1], dtype=np.int32), np.ones(2), 2, 1)
