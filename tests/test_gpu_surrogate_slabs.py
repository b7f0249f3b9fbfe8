"""The surrogate's inference on z-slabs of the torus, on the GPU: two and
three ranks as threads of one process on one GPU (each rank its own
network, plain stencil and streams; ghost planes through device buffers or
host memory between calls, no kernel waits for another) give the single
torus' result bit for bit - the tensor-core layers included (nx = 128) -
with every segment accepted by the judge and with every segment redone by
the plain stencil."""
import threading

import numpy as np
import pytest
import torch

from libgeodecomp_gb300 import slabs
from libgeodecomp_gb300 import surrogate as S
from libgeodecomp_gb300.surrogate_slabs import SlabSurrogate

pytestmark = pytest.mark.gpu

N = 128
STEPS = 2 * S.STEPS_PER_CALL * S.CALLS_PER_JUDGE


@pytest.fixture(scope="module")
def case():
    u0 = S.grf_batch_torch(1, N, 12.0, 0.0, 1.0, seed=21)[0].contiguous()
    kappa = S.grf_batch_torch(1, N, 12.0, 0.02, 0.15, seed=22)[0].contiguous()
    params = S.init_params(24, seed=5)
    return u0, kappa, params


def slab_run(params, u0, kappa, world, tol, device):
    hub = slabs.InProcessComm.Hub(world)
    parts, stats, errors, info = [None] * world, [None] * world, [], [None] * world

    def rank_main(r):
        torch.cuda.set_device(0)
        s = None
        try:
            s = SlabSurrogate(params, N, comm=slabs.InProcessComm(hub, r, device=device))
            s.set_kappa(kappa)
            u, _, stats[r] = s.run(u0, STEPS, tol=tol)
            parts[r] = u
            info[r] = s.describe()
        except Exception as e:
            errors.append(e)
            hub.barrier.abort()
        finally:
            if s is not None:
                s.close()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    return torch.cat(parts, 0), stats, info


@pytest.mark.parametrize("tol", [float("inf"), 0.0])
@pytest.mark.parametrize("world,device", [(2, True), (3, False)])
def test_slabs_equal_the_single_torus(case, tol, world, device):
    u0, kappa, params = case
    ref, _, ref_stats = S.run_surrogate_with_judge(params, u0, kappa, STEPS, tol=tol)
    assert ref_stats["fallbacks"] == (0 if tol > 0 else 2)
    out, stats, info = slab_run(params, u0, kappa, world, tol, device)
    assert torch.equal(out, ref)
    for st in stats:
        assert st["fallbacks"] == ref_stats["fallbacks"] and st["segments"] == ref_stats["segments"]
        np.testing.assert_allclose(st["judge_errors"], ref_stats["judge_errors"], rtol=1e-9)
    assert all(i["exchanges"] >= 4 for i in info)


def test_one_slab_is_the_single_torus(case):
    u0, kappa, params = case
    ref, _, _ = S.run_surrogate_with_judge(params, u0, kappa, STEPS, tol=float("inf"))
    s = SlabSurrogate(params, N)
    try:
        s.set_kappa(kappa)
        out, _, stats = s.run(u0, STEPS, tol=float("inf"))
    finally:
        s.close()
    assert torch.equal(out, ref) and stats["fallbacks"] == 0 and s.exchange_count == 0
