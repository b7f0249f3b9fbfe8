"""The surrogate's slab decomposition without a GPU: ranks as threads and as
gloo processes, with stand-ins for the network (four 3^3 layers per call,
each reaching one plane further along z) and the plain stencil (one plane
per step), give the single torus' result bit for bit, with the judge's
fallback taken and not taken; the ghost zone must hold one judge run."""
import os
import socket
import subprocess
import sys
import tempfile
import threading

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from libgeodecomp_gb300 import slabs  # noqa: E402
from libgeodecomp_gb300.surrogate_slabs import SlabSurrogate  # noqa: E402

SHAPE = (48, 6, 8)
STEPS = 2 * 16 * 8


def _mix(h):
    """One plane of reach along z (torch.roll wraps the local torus like the
    library's kernels), strong enough that a wrong value still shows after
    crossing a ghost zone of 16 planes (a weakly coupled stencil would damp
    it below float32 resolution and hide a wrong exchange schedule)."""
    return 0.5 * (h.roll(1, 0) + h.roll(-1, 0)) + 0.05 * (h.roll(1, 1) + h.roll(-1, 2) - 2.0 * h)


class FakeNet:
    """Four layers of one plane's reach with a nonlinearity, then a
    residual update of u."""

    def __init__(self, shape):
        self.shape = shape

    def advance(self, u, kappa, calls):
        for _ in range(calls):
            h = u
            for layer in range(4):
                h = _mix(h) + 0.1 * torch.sin(h + 0.1 * layer)
            u.copy_(0.9 * h + kappa * u)

    def synchronize(self):
        pass

    def close(self):
        pass


class FakePlain:
    """One plane of reach per step, on the local torus."""

    def __init__(self, shape):
        self.shape = shape
        self.k = None

    def set_kappa(self, k):
        self.k = k.clone()

    def run(self, u, steps):
        for _ in range(steps):
            u.copy_(_mix(u) + self.k * u)

    def close(self):
        pass


def fields(seed=5):
    rng = np.random.default_rng(seed)
    u0 = rng.random(SHAPE).astype(np.float32)
    kappa = (0.02 + 0.1 * rng.random(SHAPE)).astype(np.float32)
    return u0, kappa


def make(comm, ghost=16):
    return SlabSurrogate(None, SHAPE, comm=comm, ghost=ghost, make_net=FakeNet, make_plain=FakePlain)


def single_run(u0, kappa, tol, steps=STEPS):
    s = make(None)
    s.set_kappa(torch.from_numpy(kappa))
    u, _, stats = s.run(torch.from_numpy(u0), steps, tol=tol)
    return u, stats


def thread_run(world, u0, kappa, tol, steps=STEPS):
    hub = slabs.InProcessComm.Hub(world)
    parts, stats, errors, ex = [None] * world, [None] * world, [], [0] * world

    def rank_main(r):
        try:
            s = make(slabs.InProcessComm(hub, r))
            s.set_kappa(torch.from_numpy(kappa))
            parts[r], _, stats[r] = s.run(torch.from_numpy(u0), steps, tol=tol)
            ex[r] = s.exchange_count
        except Exception as e:
            errors.append(e)
            hub.barrier.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    return torch.cat(parts, 0), stats, ex


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("tol", [1.0, 0.0])
def test_threads_equal_the_single_torus(world, tol):
    u0, kappa = fields()
    ref, ref_stats = single_run(u0, kappa, tol)
    out, stats, exchanges = thread_run(world, u0, kappa, tol)
    assert torch.equal(out, ref)
    expect_fallbacks = 0 if tol == 1.0 else 2
    assert ref_stats["fallbacks"] == expect_fallbacks and ref_stats["segments"] == 2
    for st in stats:
        assert st["fallbacks"] == expect_fallbacks and st["segments"] == 2
        np.testing.assert_allclose(st["judge_errors"], ref_stats["judge_errors"], rtol=1e-12)
    # per segment: before the fifth call and before the kept state; with the
    # fallback one more before each of its eight plain blocks but the first
    assert all(e == exchanges[0] for e in exchanges)
    assert exchanges[0] >= (4 if tol == 1.0 else 18)


def test_mixed_judge_decisions_agree_on_every_rank():
    """A tolerance between the judge's errors: the first segment accepted,
    the later ones redone; every rank takes the single torus' decision
    (the error is summed over all ranks' owned planes) and the results
    stay bit-identical."""
    u0, kappa = fields()
    steps = 4 * 16 * 8
    ref, ref_stats = single_run(u0, kappa, 0.71, steps)
    assert ref_stats["judge_errors"][0] < 0.705 and ref_stats["judge_errors"][1] > 0.715
    assert 0 < ref_stats["fallbacks"] < ref_stats["segments"] == 4
    out, stats, _ = thread_run(3, u0, kappa, 0.71, steps)
    assert torch.equal(out, ref)
    assert all(st["fallbacks"] == ref_stats["fallbacks"] for st in stats)


def test_the_ghost_zone_must_hold_a_judge_run():
    with pytest.raises(ValueError):
        make(None, ghost=8)
    hub = slabs.InProcessComm.Hub(4)
    with pytest.raises(ValueError):                  # 12 planes per rank < 16 ghost planes
        make(slabs.InProcessComm(hub, 0))


def test_a_field_of_another_shape_is_refused():
    s = make(None)
    with pytest.raises(ValueError):
        s.set_kappa(torch.zeros((SHAPE[0] + 1,) + SHAPE[1:]))


WORKER = r"""
import os, sys
sys.path.insert(0, {root!r})
sys.path.insert(0, {tests!r})
import numpy as np
import torch
import torch.distributed as dist
from libgeodecomp_gb300 import slabs
from test_surrogate_slabs import make, fields, STEPS
dist.init_process_group("gloo")
comm = slabs.TorchComm(dist, device=False)
u0, kappa = fields()
s = make(comm)
s.set_kappa(torch.from_numpy(kappa))
u, _, stats = s.run(torch.from_numpy(u0), STEPS, tol={tol})
np.save(os.path.join({out!r}, "rank%d.npy" % comm.rank), u.numpy())
dist.destroy_process_group()
"""


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_equal_the_single_torus():
    port = free_port()
    with tempfile.TemporaryDirectory() as out:
        procs = []
        for rank in range(2):
            env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                       MASTER_PORT=str(port))
            code = WORKER.format(root=ROOT, tests=os.path.join(ROOT, "tests"), out=out, tol=0.0)
            procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                          stderr=subprocess.PIPE, text=True))
        outs = [p.communicate(timeout=300) for p in procs]
        for p, (_, err) in zip(procs, outs):
            assert p.returncode == 0, err[-3000:]
        got = np.concatenate([np.load(os.path.join(out, "rank%d.npy" % r)) for r in range(2)], axis=0)
    u0, kappa = fields()
    ref, _ = single_run(u0, kappa, 0.0)
    np.testing.assert_array_equal(got, ref.numpy())
