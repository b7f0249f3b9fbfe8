"""The learned surrogate's GPU kernels against the FP64 numpy reference
(oracle/surrogate_ref.py): forward pass and parameter gradients agree within
BF16 tolerance; training lowers the loss and the trained network beats the
method without it (the no-learning baseline u' = u); the judge falls back to
the plain stencil when the network is wrong."""
import numpy as np
import pytest

from libgeodecomp_gb300 import lgd

from oracle import surrogate_ref as sr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _fields(n, seed):
    rng = np.random.default_rng(seed)
    from libgeodecomp_gb300 import workloads
    u, k = workloads.varcoef_fields(n, seed=seed, length=4.0)
    return u, k, rng


def _net(shape, channels, training=False, batch=1):
    from libgeodecomp_gb300.surrogate import SurrogateNet
    return SurrogateNet(shape, batch=batch, channels=channels, training=training)


@pytest.mark.parametrize("channels,n", [(8, 32), (24, 32), (24, 64)])
def test_forward_matches_fp64_reference(channels, n):
    u, k, _ = _fields(n, 3)
    p = sr.init_params(channels, seed=5)
    p[-1] = 0.01
    ref, _ = sr.forward(p, u, k, channels)
    with _net((n, n, n), channels) as net:
        net.set_params(p.astype(np.float32))
        ut = torch.tensor(u, dtype=torch.float32, device="cuda").reshape(1, n, n, n)
        kt = torch.tensor(k, dtype=torch.float32, device="cuda").reshape(1, n, n, n)
        du = torch.empty_like(ut)
        net.forward(ut, kt, du)
        net.synchronize()
        got = du.cpu().numpy().reshape(n, n, n).astype(np.float64)
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel < 3e-2, rel   # BF16 activations and weights, FP32 accumulation


def _forward_gpu(p, u, k, variant):
    nz, ny, nx = u.shape
    with _net((nz, ny, nx), 24) as net:
        net.set_params(p.astype(np.float32))
        net.set_variant(variant)
        used_tc = net.uses_tensor_core_path()
        ut = torch.tensor(u, dtype=torch.float32, device="cuda").reshape(1, nz, ny, nx)
        kt = torch.tensor(k, dtype=torch.float32, device="cuda").reshape(1, nz, ny, nx)
        du = torch.empty_like(ut)
        net.forward(ut, kt, du)
        net.synchronize()
        return du.cpu().numpy().reshape(nz, ny, nx).astype(np.float64), used_tc


@pytest.mark.parametrize("shape", [(6, 4, 128), (5, 12, 256), (1, 4, 128)])
def test_tensor_core_layers_match_fp64_reference_and_mma_sync_path(shape):
    """Layers 2 and 3 on tcgen05 (ghosted activations, TMA-fed planes, TMEM
    accumulators): against the FP64 reference within the BF16 tolerance of
    the mma.sync path, and against the mma.sync path itself; shapes with
    one plane, two rows and several 128-voxel row tiles exercise the ghost
    copies on every face."""
    rng = np.random.default_rng(sum(shape))
    u = rng.random(shape)
    k = 0.02 + 0.13 * rng.random(shape)
    p = sr.init_params(24, seed=8)
    p[-1] = 0.01
    ref, _ = sr.forward(p, u, k, 24)
    tc, used = _forward_gpu(p, u, k, 0)
    assert used
    ms, used_ms = _forward_gpu(p, u, k, 1)
    assert not used_ms
    scale = np.linalg.norm(ref)
    assert np.linalg.norm(tc - ref) / scale < 3e-2
    assert np.linalg.norm(ms - ref) / scale < 3e-2
    # the two GPU paths round the same FP32 sums to BF16; they differ only
    # where the summation order flips a rounding
    assert np.linalg.norm(tc - ms) / scale < 1e-2, np.linalg.norm(tc - ms) / scale


def test_gradients_match_fp64_reference():
    channels, n = 8, 32
    u, k, rng = _fields(n, 4)
    target = 0.05 * rng.standard_normal((n, n, n))
    p = sr.init_params(channels, seed=6)
    p[-1] = 0.02
    loss_ref, g_ref = sr.loss_and_grad(p, u, k, target, channels)
    with _net((n, n, n), channels, training=True) as net:
        net.set_params(p.astype(np.float32))
        ut = torch.tensor(u, dtype=torch.float32, device="cuda").reshape(1, n, n, n)
        kt = torch.tensor(k, dtype=torch.float32, device="cuda").reshape(1, n, n, n)
        tt = torch.tensor(target, dtype=torch.float32, device="cuda").reshape(1, n, n, n)
        du = torch.empty_like(ut)
        net.forward(ut, kt, du)
        loss = net.backward(tt)
        g = net.get_grads().astype(np.float64)
    assert abs(loss - loss_ref) / loss_ref < 2e-2
    # per layer: direction and size of the gradient
    o = 0
    for ci, co in sr.layer_shapes(channels):
        for size in (27 * ci * co, co):
            a = g[o:o + size]
            b = g_ref[o:o + size]
            o += size
            cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30)
            rel = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30)
            assert cos > 0.995 and rel < 0.08, (ci, co, size, cos, rel)


def test_training_lowers_loss_and_beats_the_no_learning_baseline():
    from libgeodecomp_gb300 import surrogate as S
    states, kappa = S.make_trajectories(count=48, n=32, calls=3, length=8.0, seed=11)
    params, hist = S.train(states[:40], kappa[:40], channels=24, iters=400, batch=4, lr=2e-3, seed=1)
    assert np.mean(hist[-20:]) < 0.3 * np.mean(hist[:5])
    err_net, err_id = S.one_call_errors(params, states[40:], kappa[40:], channels=24)
    # what the trained network gains over the method without it
    assert err_net < 0.5 * err_id, (err_net, err_id)


def test_data_parallel_training_follows_the_global_batch():
    """Two ranks (threads of one process, each its own network on the GPU)
    train on halves of the same global batch and average their gradients
    before every Adam step: both replicas end bit-identical, and equal to
    one network trained on the whole batch up to the order of the FP32
    gradient sums."""
    import threading
    from libgeodecomp_gb300 import slabs
    from libgeodecomp_gb300 import surrogate as S
    states, kappa = S.make_trajectories(count=16, n=32, calls=3, length=8.0, seed=5)
    p0 = S.init_params(24, seed=2)
    single, hist1 = S.train(states, kappa, channels=24, iters=6, batch=4, lr=1e-3, seed=4, params=p0)
    hub = slabs.InProcessComm.Hub(2)
    out = [None, None]
    errors = []

    def rank_main(r):
        try:
            out[r] = S.train(states, kappa, channels=24, iters=6, batch=2, lr=1e-3, seed=4, params=p0,
                             comm=slabs.InProcessComm(hub, r))
        except Exception as e:
            errors.append(e)
            hub.barrier.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    (pa, ha), (pb, hb) = out
    np.testing.assert_array_equal(pa, pb)
    assert ha == hb
    np.testing.assert_allclose(pa, single, rtol=1e-3, atol=1e-5)
    np.testing.assert_allclose(ha, hist1, rtol=1e-3)
    assert not np.array_equal(pa, p0)
    with S.SurrogateNet((32, 32, 32), batch=1, channels=24) as net:      # no training buffers
        with pytest.raises(lgd.LGDError):
            net.set_grads(np.zeros(net.P, dtype=np.float32))


def test_judge_falls_back_to_the_plain_stencil():
    from libgeodecomp_gb300 import surrogate as S
    n = 32
    u0 = S.grf_batch_torch(1, n, 8.0, 0.0, 1.0, seed=3)[0].contiguous()
    kappa = S.grf_batch_torch(1, n, 8.0, 0.02, 0.15, seed=4)[0].contiguous()
    bad = S.init_params(24, seed=9) * 50.0          # a network that is badly wrong
    steps = S.STEPS_PER_CALL * S.CALLS_PER_JUDGE * 2
    u_sur, _, stats = S.run_surrogate_with_judge(bad, u0, kappa, steps, tol=1e-4)
    u_plain, _ = S.run_plain(u0, kappa, steps)
    assert stats["fallbacks"] == stats["segments"] == 2
    assert S.rel_l2(u_sur, u_plain) < 1e-6


@pytest.mark.parametrize("shape", [(6, 4, 128), (5, 12, 256)])
def test_advance_equals_forward_plus_residual(shape):
    """advance() lets the last layer add du into u itself on the fast path;
    the result is the same as forward() followed by u + du."""
    rng = np.random.default_rng(7)
    u = rng.random(shape)
    k = 0.02 + 0.13 * rng.random(shape)
    p = sr.init_params(24, seed=12)
    p[-1] = 0.01
    nz, ny, nx = shape
    with _net(shape, 24) as net:
        net.set_params(p.astype(np.float32))
        ut = torch.tensor(u, dtype=torch.float32, device="cuda").reshape(1, nz, ny, nx)
        kt = torch.tensor(k, dtype=torch.float32, device="cuda").reshape(1, nz, ny, nx)
        du = torch.empty_like(ut)
        net.forward(ut, kt, du)
        net.synchronize()                  # the net works on its own stream
        expect = ut + du
        torch.cuda.synchronize()
        net.advance(ut, kt, 1)
        net.synchronize()
        assert torch.equal(ut, expect)
