"""The row-block decomposition of SELL-C-sigma diffusion on the GPU: two and
three ranks as threads of one process on one GPU (each rank its own
library grid built from the same CSR and its own stream; the next buffer's
blocks travel through host memory or device to device between steps, no
kernel waits for another) give the single grid's result bit for bit, in the
exact mode and the fused-multiply-add mode, FP64 and FP32."""
import threading

import numpy as np
import pytest

from libgeodecomp_gb300 import lgd, sell_shards, slabs, workloads

pytestmark = pytest.mark.gpu


def run_ranks(n, rp, col, w, x0, steps, world, device, exact, precision):
    hub = slabs.InProcessComm.Hub(world)
    out = [None] * world
    errors = []

    def rank_main(r):
        try:
            with lgd.SellGrid.from_csr(n, rp, col, w, 32, 256, precision=precision, exact=exact) as g:
                g.upload(x0)
                s = sell_shards.ShardedSell(g, slabs.InProcessComm(hub, r, device=device), 32, precision=precision)
                s.step(steps // 2)
                s.step(steps - steps // 2)
                s.synchronize()
                out[r] = g.download()
        except Exception as e:
            errors.append(e)
            hub.barrier.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    return out


@pytest.mark.parametrize("world,device,exact,precision",
                         [(2, False, True, 8), (3, True, True, 8), (2, True, False, 8), (3, False, False, 4)])
def test_row_blocks_equal_single_grid(world, device, exact, precision):
    n = 50021
    rp, col, w = workloads.powerlaw_graph(n, seed=7)
    x0 = workloads.sell_values(n, seed=7)
    with lgd.SellGrid.from_csr(n, rp, col, w, 32, 256, precision=precision, exact=exact) as g:
        g.upload(x0)
        g.step(9)
        ref = g.download()
    for o in run_ranks(n, rp, col, w, x0, 9, world, device, exact, precision):
        np.testing.assert_array_equal(o, ref)


def test_x_device_is_the_physical_buffer():
    n = 1000
    rp, col, w = workloads.powerlaw_graph(n, seed=2)
    x0 = workloads.sell_values(n, seed=2)
    import torch
    with lgd.SellGrid.from_csr(n, rp, col, w, 32, 256) as g:
        g.upload(x0)
        g.synchronize()
        ptr, rows_padded = g.x_device(0)
        assert rows_padded == ((n + 31) // 32) * 32
        view = sell_shards._device_view(ptr, rows_padded, torch.float64)
        np.testing.assert_array_equal(view[:n].cpu().numpy(), g.download(logical=False))
        assert float(view[n:].abs().sum()) == 0.0
        with pytest.raises(lgd.LGDError):
            g.x_device(2)
