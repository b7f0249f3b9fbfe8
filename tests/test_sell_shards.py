"""The row-block decomposition of SELL-C-sigma diffusion on CPU ranks (no
GPU): the chunk-aligned blocks, and whole runs of two to four ranks - threads
of one process and two gloo processes - whose result equals a single grid's
bit for bit.  The local grid is a numpy stand-in with the SellGrid
interface (physical order = logical order, each row summed in its entry
order); the GPU runs of the same code are in test_gpu_sell_shards.py."""
import json
import os
import socket
import subprocess
import sys
import threading

import numpy as np
import pytest

from libgeodecomp_gb300 import sell_shards, slabs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def random_csr(n, seed, max_deg=9):
    rng = np.random.default_rng(seed)
    deg = rng.integers(0, max_deg + 1, n)
    row_ptr = np.concatenate([[0], np.cumsum(deg)]).astype(np.int64)
    col = rng.integers(0, n, int(row_ptr[-1])).astype(np.int32)
    w = rng.random(int(row_ptr[-1]))
    return row_ptr, col, w


class NumpySell:
    """x' = 0.1 x + W x on a CSR matrix, rows updated in their entry order
    (each product rounded, then added), with SellGrid's buffer interface."""

    def __init__(self, row_ptr, col, w):
        self.n = len(row_ptr) - 1
        self.rp, self.col, self.w = row_ptr, col, w
        self.x = [np.zeros(self.n), np.zeros(self.n)]
        self.cur = 0

    def upload(self, x, logical=True, which=0):
        self.x[self.cur if which == 0 else 1 - self.cur][...] = x

    def download(self, logical=True, which=0):
        return self.x[self.cur if which == 0 else 1 - self.cur].copy()

    def update_rows(self, r0, r1):
        x, xn = self.x[self.cur], self.x[1 - self.cur]
        rows = np.arange(r0, r1)
        lens = self.rp[r0 + 1:r1 + 1] - self.rp[r0:r1]
        acc = np.zeros(r1 - r0)
        for k in range(int(lens.max()) if len(lens) else 0):
            m = lens > k
            e = self.rp[rows[m]] + k
            acc[m] = acc[m] + self.w[e] * x[self.col[e]]
        xn[r0:r1] = 0.1 * x[r0:r1] + acc

    def swap(self):
        self.cur = 1 - self.cur

    def step(self, n):
        for _ in range(n):
            self.update_rows(0, self.n)
            self.swap()


def threaded_run(rp, col, w, x0, steps, world, C):
    hub = slabs.InProcessComm.Hub(world)
    out = [None] * world
    errors = []

    def rank_main(r):
        try:
            g = NumpySell(rp, col, w)
            g.upload(x0)
            s = sell_shards.ShardedSell(g, slabs.InProcessComm(hub, r), C)
            s.step(steps // 2)
            s.step(steps - steps // 2)
            out[r] = g.download()
        except Exception as e:      # pragma: no cover - reported below
            errors.append(e)
            hub.barrier.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    return out


def test_blocks_are_chunk_aligned_and_cover_the_rows():
    for n, C, world in ((1000, 32, 3), (4194304, 32, 8), (70, 32, 4), (5, 32, 2)):
        b = sell_shards.RowBlocks(n, C, world)
        assert b.ranges[0][0] == 0 and b.ranges[-1][1] == n
        assert all(p[1] == q[0] for p, q in zip(b.ranges, b.ranges[1:]))
        assert all(r0 % C == 0 for r0, r1 in b.ranges if r1 > r0)
        assert b.block % C == 0


@pytest.mark.parametrize("world", [2, 3, 4])
def test_row_blocks_equal_single_grid(world):
    n = 1000
    rp, col, w = random_csr(n, seed=world)
    x0 = np.random.default_rng(9).random(n)
    ref = NumpySell(rp, col, w)
    ref.upload(x0)
    ref.step(7)
    outs = threaded_run(rp, col, w, x0, 7, world, C=32)
    for o in outs:                       # every rank holds the whole vector
        np.testing.assert_array_equal(o, ref.download())


def test_more_ranks_than_chunks():
    """Ranks without rows still take part in every gather."""
    n = 40
    rp, col, w = random_csr(n, seed=5)
    x0 = np.random.default_rng(1).random(n)
    ref = NumpySell(rp, col, w)
    ref.upload(x0)
    ref.step(5)
    for o in threaded_run(rp, col, w, x0, 5, 4, C=32):
        np.testing.assert_array_equal(o, ref.download())


WORKER = r"""
import os, sys, json
sys.path.insert(0, {root!r})
sys.path.insert(0, {tests!r})
import numpy as np
import torch.distributed as dist
from libgeodecomp_gb300 import sell_shards, slabs
from test_sell_shards import NumpySell, random_csr
dist.init_process_group("gloo")
comm = slabs.TorchComm(dist, device=False)
rp, col, w = random_csr(777, seed=3)
x0 = np.random.default_rng(4).random(777)
g = NumpySell(rp, col, w)
g.upload(x0)
s = sell_shards.ShardedSell(g, comm, 32)
s.step(6)
if comm.rank == 0:
    ref = NumpySell(rp, col, w)
    ref.upload(x0)
    ref.step(6)
    print(json.dumps({{"equal": bool(np.array_equal(g.download(), ref.download())), "gathers": s.gathers}}))
dist.destroy_process_group()
"""


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_gather_through_host_buffers():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        code = WORKER.format(root=ROOT, tests=os.path.join(ROOT, "tests"))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=300) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err[-3000:]
    line = json.loads(outs[0][0].strip().splitlines()[-1])
    assert line["equal"] and line["gathers"] == 6
