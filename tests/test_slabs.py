"""The slab decomposition's host logic on CPU ranks (no GPU): the partition,
the ghost widths and the exchange plan, and whole runs of two and three
ranks - threads of one process and gloo processes - whose gathered result
equals a single grid's bit for bit.  The local grids are a numpy stand-in
for the library's grids with the same plane interface; the GPU runs of the
same code are in test_gpu_slabs.py."""
import json
import os
import socket
import subprocess
import sys
import threading

import numpy as np
import pytest

from libgeodecomp_gb300 import slabs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# ------------------------------------------------------------ stand-in grid
def _pad(a, mask, edge):
    """a padded by one cell on every axis: wrapped on the axes of the mask
    (bit 0 = the fastest axis), the edge value on the others."""
    out = a
    nd = a.ndim
    for ax in range(nd):
        bit = 1 << (nd - 1 - ax)          # array axis 0 is the slowest
        if mask & bit:
            out = np.concatenate([out.take([-1], axis=ax), out, out.take([0], axis=ax)], axis=ax)
        else:
            shape = list(out.shape)
            shape[ax] = 1
            e = np.full(shape, edge, dtype=out.dtype)
            out = np.concatenate([e, out, e], axis=ax)
    return out


class NumpyGrid:
    """Jacobi-7 (3D) or Game of Life (2D) on numpy, with lgd.Grid's plane
    interface (raw planes of the slowest axis as bytes)."""

    def __init__(self, shape, mask, edge=0.0, rule="jacobi"):
        self.a = np.zeros(shape, dtype=np.uint8 if rule == "life" else np.float64)
        self.mask, self.edge, self.rule = mask, edge, rule
        self.steps = 0

    def upload(self, member, values):
        self.a[...] = values

    def download(self, member=0):
        return self.a.copy()

    def step(self, n):
        for _ in range(n):
            p = _pad(self.a, self.mask, self.edge)
            if self.rule == "jacobi":
                c = p[1:-1, 1:-1, 1:-1]
                acc = c + p[1:-1, :-2, 1:-1]
                acc = acc + p[1:-1, 2:, 1:-1]
                acc = acc + p[1:-1, 1:-1, 2:]
                acc = acc + p[1:-1, 1:-1, :-2]
                acc = acc + p[2:, 1:-1, 1:-1]
                acc = acc + p[:-2, 1:-1, 1:-1]
                self.a = acc * (1.0 / 7.0)
            else:
                n8 = sum(p[1 + dy:p.shape[0] - 1 + dy, 1 + dx:p.shape[1] - 1 + dx].astype(np.int32)
                         for dy in (-1, 0, 1) for dx in (-1, 0, 1) if (dx, dy) != (0, 0))
                self.a = ((n8 == 3) | ((self.a == 1) & (n8 == 2))).astype(np.uint8)
            self.steps += 1

    def plane_bytes(self, member=0):
        return self.a[0].nbytes

    def save_planes(self, p0, n, member=0, which=0, out=None):
        b = np.frombuffer(np.ascontiguousarray(self.a[p0:p0 + n]).tobytes(), dtype=np.uint8)
        if out is None:
            return b.copy()
        out[...] = b
        return out

    def load_planes(self, p0, data, member=0, which=0):
        raw = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
        n = raw.nbytes // self.plane_bytes()
        self.a[p0:p0 + n] = np.frombuffer(raw.tobytes(), dtype=self.a.dtype).reshape((n,) + self.a.shape[1:])


def single_run(rule, u0, mask, steps, edge=0.0):
    g = NumpyGrid(u0.shape, mask, edge, rule)
    g.upload(0, u0)
    g.step(steps)
    return g.download()


def threaded_run(rule, u0, mask, steps, world, ghost, edge=0.0, chunks=(3, 5, 100)):
    """world ranks as threads, stepping in uneven chunks; returns the
    gathered grid and the slabs."""
    hub = slabs.InProcessComm.Hub(world)
    parts = [None] * world
    grids = [None] * world
    errors = []

    def rank_main(r):
        try:
            comm = slabs.InProcessComm(hub, r)
            s = slabs.SlabGrid(None, u0.shape, comm, periodic=mask, ghost=ghost,
                               make_grid=lambda shape, m: NumpyGrid(shape, m, edge, rule), fixed_point=False)
            s.upload(0, u0)
            left = steps
            for c in chunks:
                k = min(c, left)
                s.step(k)
                left -= k
            s.step(left)
            parts[r] = s.download_owned()
            grids[r] = s
        except Exception as e:      # pragma: no cover - reported below
            errors.append(e)
            hub.barrier.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    return np.concatenate(parts, axis=0), grids


# ------------------------------------------------------------------ layout
def test_partition_covers_the_axis_once():
    for n, world in ((10, 3), (512, 8), (7, 7), (100, 1)):
        spans = [slabs.partition(n, world, r) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
        sizes = [p1 - p0 for p0, p1 in spans]
        assert max(sizes) - min(sizes) <= 1


def test_layout_ghosts_and_exchanges():
    # non-periodic: the outer ranks have no ghost zone on the outer side
    lay = [slabs.SlabLayout(40, 3, r, 4, periodic=False) for r in range(3)]
    assert (lay[0].ghost_lo, lay[0].ghost_hi) == (0, 4)
    assert (lay[1].ghost_lo, lay[1].ghost_hi) == (4, 4)
    assert (lay[2].ghost_lo, lay[2].ghost_hi) == (4, 0)
    assert lay[1].exchanges() == [(0, 4, 0), (2, 4 + lay[1].owned - 4, 4 + lay[1].owned)]
    assert lay[0].exchanges() == [(1, lay[0].owned - 4, lay[0].owned)]
    # periodic: every rank has both neighbours, the ends wrap
    per = [slabs.SlabLayout(40, 3, r, 4, periodic=True) for r in range(3)]
    assert per[0].lower == 2 and per[2].upper == 0
    assert per[0].global_range() == (-4, per[0].p1 + 4)
    # one rank: the whole axis, wrapping locally when periodic
    one = slabs.SlabLayout(40, 1, 0, 4, periodic=True)
    assert one.exchanges() == [] and one.local_periodic and one.local_planes == 40
    with pytest.raises(ValueError):
        slabs.SlabLayout(10, 4, 0, 4, periodic=False)       # 2 or 3 planes per rank < ghost 4


# ----------------------------------------------------------- whole runs
@pytest.mark.parametrize("world,ghost", [(2, 2), (3, 4), (4, 3)])
def test_jacobi_slabs_equal_single_grid(world, ghost):
    u0 = np.random.default_rng(world).random((29, 11, 13))
    ref = single_run("jacobi", u0, 0, 23, edge=0.25)
    out, grids = threaded_run("jacobi", u0, 0, 23, world, ghost, edge=0.25)
    np.testing.assert_array_equal(out, ref)
    assert all(g.exchange_count >= 23 // ghost for g in grids)


@pytest.mark.parametrize("world", [2, 3])
def test_jacobi_slabs_periodic_cut_axis(world):
    """A torus in every axis: the first and last ranks exchange through the
    wrap (with two ranks each is the other's lower and upper neighbour)."""
    u0 = np.random.default_rng(7).random((18, 9, 10))
    ref = single_run("jacobi", u0, 7, 17)
    out, _ = threaded_run("jacobi", u0, 7, 17, world, 3)
    np.testing.assert_array_equal(out, ref)


def test_life_slabs_on_a_torus():
    rng = np.random.default_rng(3)
    c0 = (rng.random((48, 37)) < 0.3).astype(np.uint8)
    ref = single_run("life", c0, 3, 40)
    out, _ = threaded_run("life", c0, 3, 40, 3, 5)
    np.testing.assert_array_equal(out, ref)


# ------------------------------------------------------ gloo processes
WORKER = r"""
import os, sys, json
sys.path.insert(0, {root!r})
sys.path.insert(0, {tests!r})
import numpy as np
import torch.distributed as dist
from libgeodecomp_gb300 import slabs
from test_slabs import NumpyGrid, single_run
dist.init_process_group("gloo")
comm = slabs.TorchComm(dist, device=False)
u0 = np.random.default_rng(11).random((30, 7, 9))
s = slabs.SlabGrid(None, u0.shape, comm, periodic={mask}, ghost=3,
                   make_grid=lambda shape, m: NumpyGrid(shape, m, 0.5, "jacobi"), fixed_point=False)
s.upload(0, u0)
s.step(4)
s.step(15)
full = s.gather()
if comm.rank == 0:
    ref = single_run("jacobi", u0, {mask}, 19, edge=0.5)
    print(json.dumps({{"equal": bool(np.array_equal(full, ref)), "exchanges": s.exchange_count}}))
dist.destroy_process_group()
"""


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("mask", [0, 7])
def test_two_gloo_ranks_exchange_through_host_buffers(mask):
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        code = WORKER.format(root=ROOT, tests=os.path.join(ROOT, "tests"), mask=mask)
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=300) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err[-3000:]
    line = json.loads(outs[0][0].strip().splitlines()[-1])
    assert line["equal"] and line["exchanges"] >= 6


def test_in_process_allreduce_mean_is_identical_on_every_rank():
    world = 3
    hub = slabs.InProcessComm.Hub(world)
    out = [None] * world

    def rank_main(r):
        comm = slabs.InProcessComm(hub, r)
        out[r] = comm.allreduce_mean(np.arange(5, dtype=np.float32) * (r + 1))

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for o in out:
        np.testing.assert_array_equal(o, out[0])
    np.testing.assert_allclose(out[0], np.arange(5) * 2.0)
    assert out[0].dtype == np.float32


REDUCE_WORKER = r"""
import sys, json
sys.path.insert(0, {root!r})
import numpy as np
import torch.distributed as dist
from libgeodecomp_gb300 import slabs
dist.init_process_group("gloo")
comm = slabs.TorchComm(dist, device=False)
m = comm.allreduce_mean(np.arange(4, dtype=np.float32) + 10 * comm.rank)
print(json.dumps({{"rank": comm.rank, "mean": m.tolist(), "dtype": str(m.dtype)}}))
dist.destroy_process_group()
"""


def test_two_gloo_ranks_average_an_array():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", REDUCE_WORKER.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=300) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err[-3000:]
        line = json.loads(out.strip().splitlines()[-1])
        assert line["mean"] == [5.0, 6.0, 7.0, 8.0] and line["dtype"] == "float32"
