"""The reverse Cuthill-McKee numbering behind LGD_SELL_RENUMBER (host code of
the library, lgd_graph_rcm): a permutation of the nodes for any graph
(power-law, empty rows, several components), and on a randomly numbered
3D mesh it brings the bandwidth (the largest |row - column| of an edge)
back near the mesh's own."""
import numpy as np
import pytest

from libgeodecomp_gb300 import lgd, workloads


def csr_from_edges(n, r, c):
    o = np.argsort(r, kind="stable")
    r, c = r[o], c[o]
    rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rp, r + 1, 1)
    return np.cumsum(rp), c.astype(np.int32)


def permuted_mesh(n1, seed):
    n = n1 ** 3
    idx = np.arange(n).reshape(n1, n1, n1)
    rows, cols = [], []
    for d in ((0, 0, 1), (0, 0, -1), (0, 1, 0), (0, -1, 0), (1, 0, 0), (-1, 0, 0)):
        rows.append(idx.ravel())
        cols.append(np.roll(idx, shift=d, axis=(0, 1, 2)).ravel())
    p = np.random.default_rng(seed).permutation(n)
    return (n,) + csr_from_edges(n, p[np.concatenate(rows)], p[np.concatenate(cols)])


def bandwidth(rp, col):
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    return int(np.max(np.abs(rows - col))) if col.size else 0


def renumber(order, rp, col):
    n = len(rp) - 1
    inv = np.empty(n, dtype=np.int64)
    inv[order] = np.arange(n)
    lens = np.diff(rp)[order]
    rp2 = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    col2 = np.concatenate([inv[col[rp[r]:rp[r + 1]]] for r in order]) if col.size else col
    return rp2, col2


def test_mesh_bandwidth_shrinks():
    n, rp, col = permuted_mesh(24, seed=3)
    order = lgd.graph_rcm(n, rp, col)
    assert np.array_equal(np.sort(order), np.arange(n))
    rp2, col2 = renumber(order, rp, col)
    assert bandwidth(rp, col) > 10000
    assert bandwidth(rp2, col2) < 3 * 24 * 24      # a torus mesh's own is about 2 planes
    # every row keeps its entries (as renumbered ids)
    for k in (0, 17, n - 1):
        r = order[k]
        assert np.array_equal(order[col2[rp2[k]:rp2[k + 1]]], col[rp[r]:rp[r + 1]])


def test_any_graph_gets_a_permutation():
    rp, col, _ = workloads.powerlaw_graph(5000, seed=4)
    order = lgd.graph_rcm(5000, rp, col)
    assert np.array_equal(np.sort(order), np.arange(5000))
    # empty rows and several components (a chain, isolated nodes, a cycle)
    n = 40
    r = np.array([0, 1, 2, 10, 11, 12, 13], dtype=np.int64)
    c = np.array([1, 2, 3, 11, 12, 13, 10], dtype=np.int64)
    rp2, col2 = csr_from_edges(n, r, c)
    order = lgd.graph_rcm(n, rp2, col2)
    assert np.array_equal(np.sort(order), np.arange(n))


def test_bad_graphs_are_refused():
    rp = np.array([0, 1, 2], dtype=np.int64)
    with pytest.raises(lgd.LGDError):
        lgd.graph_rcm(2, rp, np.array([0, 5], dtype=np.int32))       # column outside the node set
    with pytest.raises(lgd.LGDError):
        lgd.graph_rcm(0, np.zeros(1, dtype=np.int64), np.zeros(0, dtype=np.int32))
