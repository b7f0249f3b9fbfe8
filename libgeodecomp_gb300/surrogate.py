"""Learned surrogate for variable-coefficient diffusion (host side).

Drives the C ABI of include/lgd_surrogate.h (network forward / backward /
Adam kernels) and include/lgd_gpu.h (the plain var-coef stencil, which
makes the training trajectories and judges the surrogate at run time).
Device buffers are torch CUDA tensors used as plain memory.

Run time scheme (surrogate plus judge):
  - one surrogate call advances u by 16 plain steps: u <- u + net(u, kappa);
  - after every 8 calls the judge re-runs the last call's 16 steps with the
    plain stencil from the state before that call and compares;
  - if the relative L2 difference exceeds the tolerance, the whole segment
    of 8 calls is redone with the plain stencil (fallback), so the answer
    never drifts further than one segment past the judge.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import lgd

STEPS_PER_CALL = 16
CALLS_PER_JUDGE = 8
# multiply-adds x 2 per voxel and call: 27 taps x (2x24 + 24x24 + 24x24 + 24x1)
FLOP_PER_VOXEL = 2 * 27 * (2 * 24 + 24 * 24 + 24 * 24 + 24 * 1)


def _bind():
    L = lgd.lib()
    P = ctypes.c_void_p
    I = ctypes.c_int
    for name, args in {
        "lgd_net_param_count": [I, P],
        "lgd_net_create": [I, I, I, I, I, I, P],
        "lgd_net_destroy": [P],
        "lgd_net_set_params": [P, P, ctypes.c_size_t],
        "lgd_net_get_params": [P, P, ctypes.c_size_t],
        "lgd_net_get_grads": [P, P, ctypes.c_size_t],
        "lgd_net_set_grads": [P, P, ctypes.c_size_t],
        "lgd_net_forward": [P, P, P, P],
        "lgd_net_backward": [P, P, P],
        "lgd_net_adam": [P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float],
        "lgd_net_advance": [P, P, P, I],
        "lgd_net_synchronize": [P],
        "lgd_net_stream": [P, P],
        "lgd_net_launch_count": [P, P],
        "lgd_net_set_variant": [P, I],
        "lgd_net_uses_tensor_core_path": [P, P],
    }.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = I
    return L


def param_count(channels: int = 24) -> int:
    n = ctypes.c_int64()
    lgd.check(_bind().lgd_net_param_count(channels, ctypes.byref(n)))
    return n.value


def init_params(channels: int = 24, seed: int = 0) -> np.ndarray:
    """He-style initialisation, last layer scaled by 0.1 (starts near the
    identity map u' = u)."""
    rng = np.random.default_rng(seed)
    out = []
    for li, (ci, co) in enumerate([(2, channels), (channels, channels), (channels, channels), (channels, 1)]):
        std = np.sqrt(2.0 / (27 * ci)) * (0.1 if li == 3 else 1.0)
        out.append(rng.normal(0.0, std, 27 * ci * co))
        out.append(np.zeros(co))
    return np.concatenate(out).astype(np.float32)


class SurrogateNet:
    """One network handle for grids of shape (batch, nz, ny, nx)."""

    def __init__(self, shape, batch: int = 1, channels: int = 24, training: bool = False):
        nz, ny, nx = shape
        self.shape = (batch, nz, ny, nx)
        self.channels = channels
        self.P = param_count(channels)
        self._L = _bind()
        self._h = ctypes.c_void_p()
        lgd.check(self._L.lgd_net_create(nx, ny, nz, batch, channels, int(training), ctypes.byref(self._h)))

    def close(self):
        if self._h:
            lgd.check(self._L.lgd_net_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_params(self, p: np.ndarray):
        a = np.ascontiguousarray(p, dtype=np.float32)
        assert a.size == self.P
        lgd.check(self._L.lgd_net_set_params(self._h, a.ctypes.data, a.size))

    def get_params(self) -> np.ndarray:
        a = np.empty(self.P, dtype=np.float32)
        lgd.check(self._L.lgd_net_get_params(self._h, a.ctypes.data, a.size))
        return a

    def get_grads(self) -> np.ndarray:
        a = np.empty(self.P, dtype=np.float32)
        lgd.check(self._L.lgd_net_get_grads(self._h, a.ctypes.data, a.size))
        return a

    def set_grads(self, g: np.ndarray):
        a = np.ascontiguousarray(g, dtype=np.float32)
        assert a.size == self.P
        lgd.check(self._L.lgd_net_set_grads(self._h, a.ctypes.data, a.size))

    def forward(self, u, kappa, du):
        lgd.check(self._L.lgd_net_forward(self._h, u.data_ptr(), kappa.data_ptr(), du.data_ptr()))

    def backward(self, target) -> float:
        loss = ctypes.c_double()
        lgd.check(self._L.lgd_net_backward(self._h, target.data_ptr(), ctypes.byref(loss)))
        return loss.value

    def adam(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        lgd.check(self._L.lgd_net_adam(self._h, lr, beta1, beta2, eps))

    def advance(self, u, kappa, calls: int = 1):
        lgd.check(self._L.lgd_net_advance(self._h, u.data_ptr(), kappa.data_ptr(), calls))

    def synchronize(self):
        lgd.check(self._L.lgd_net_synchronize(self._h))

    def stream(self) -> int:
        p = ctypes.c_void_p()
        lgd.check(self._L.lgd_net_stream(self._h, ctypes.byref(p)))
        return p.value

    def launch_count(self) -> int:
        n = ctypes.c_uint64()
        lgd.check(self._L.lgd_net_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def set_variant(self, variant: int):
        """0: tcgen05 layers where they apply (inference, C = 24, nx % 128 == 0,
        ny even); 1: mma.sync for every layer."""
        lgd.check(self._L.lgd_net_set_variant(self._h, variant))

    def uses_tensor_core_path(self) -> bool:
        y = ctypes.c_int()
        lgd.check(self._L.lgd_net_uses_tensor_core_path(self._h, ctypes.byref(y)))
        return bool(y.value)


class PlainStencil:
    """The plain var-coef stencil (LGD_CELL_VARCOEF_F32 on a torus) working
    on torch CUDA tensors: copy in, step, copy out.  n: the edge of a cube,
    or shape: (nz, ny, nx) of any torus."""

    def __init__(self, n: int = 0, precision: int = 4, shape=None):
        self.shape = tuple(shape) if shape is not None else (n, n, n)
        self.n = self.shape[-1]
        self.cells = int(np.prod(self.shape))
        self.cell = lgd.CELL_VARCOEF_F32 if precision == 4 else lgd.CELL_VARCOEF_F64
        self.g = lgd.Grid(self.cell, self.shape, periodic=7)
        self.elem = precision

    def close(self):
        self.g.close()

    def set_kappa(self, kappa):
        import torch
        torch.cuda.synchronize()
        self._call("lgd_gpu_upload_device", 1, 0, kappa)

    def run(self, u, steps: int):
        """u (torch CUDA tensor of the torus' shape) <- u after steps plain
        steps."""
        import torch
        torch.cuda.synchronize()
        self._call("lgd_gpu_upload_device", 0, 0, u)
        self.g.step(steps)
        self._call("lgd_gpu_download_device", 0, 0, u)

    def _call(self, name, member, which, t):
        assert t.is_contiguous() and t.numel() == self.cells and t.element_size() == self.elem
        fn = getattr(lgd.lib(), name)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]
        fn.restype = ctypes.c_int
        lgd.check(fn(self.g._h, member, which, t.data_ptr(), t.numel() * self.elem))


def grf_batch_torch(count: int, n: int, length: float, lo: float, hi: float, seed: int):
    """count periodic Gaussian random fields (n^3 each) on the GPU, mapped to
    [lo, hi] per field; same construction as workloads.gaussian_random_field
    (white noise filtered by exp(-k^2 length^2 / 2)), with torch's generator."""
    import torch
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    noise = torch.randn((count, n, n, n), generator=gen, device="cuda", dtype=torch.float64)
    k = 2.0 * np.pi * torch.fft.fftfreq(n, device="cuda", dtype=torch.float64)
    kr = 2.0 * np.pi * torch.fft.rfftfreq(n, device="cuda", dtype=torch.float64)
    k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + kr[None, None, :] ** 2
    filt = torch.exp(-0.5 * k2 * length * length)
    f = torch.fft.irfftn(torch.fft.rfftn(noise, dim=(1, 2, 3)) * filt, s=(n, n, n), dim=(1, 2, 3))
    fmin = f.amin(dim=(1, 2, 3), keepdim=True)
    fmax = f.amax(dim=(1, 2, 3), keepdim=True)
    return (lo + (hi - lo) * (f - fmin) / (fmax - fmin)).to(torch.float32)


def make_trajectories(count: int = 2000, n: int = 32, calls: int = 4, length: float = 16.0, seed: int = 7):
    """count plain-stencil trajectories on n^3 tori: returns (states, kappa)
    with states[j, c] the field after c surrogate calls' worth of plain
    steps (c = 0 .. calls)."""
    import torch
    kappa = grf_batch_torch(count, n, length, 0.02, 0.15, seed)
    u0 = grf_batch_torch(count, n, length, 0.0, 1.0, seed + 1)
    states = torch.empty((count, calls + 1, n, n, n), device="cuda", dtype=torch.float32)
    states[:, 0] = u0
    plain = PlainStencil(n)
    try:
        for j in range(count):
            plain.set_kappa(kappa[j].contiguous())
            u = u0[j].contiguous().clone()
            for c in range(calls):
                plain.run(u, STEPS_PER_CALL)
                states[j, c + 1] = u
    finally:
        plain.close()
    return states, kappa


def train(states, kappa, channels: int = 24, iters: int = 1500, batch: int = 8, lr: float = 1e-3, seed: int = 0,
          params: np.ndarray | None = None, log=None, comm=None):
    """Adam on the MSE of the one-call increment over random (trajectory,
    call) pairs; returns (params, loss history).

    comm (a libgeodecomp_gb300.slabs comm, several ranks): data-parallel
    training.  Every rank draws the same global batch of world x batch
    pairs and trains on its own slice; the ranks average their gradients
    (one all-reduce per iteration) before the Adam step, so the replicas
    stay identical and follow the single-rank run with the global batch
    (up to the order of the FP32 gradient sums)."""
    import torch
    count, calls1, n = states.shape[0], states.shape[1], states.shape[2]
    world, rank = (comm.world, comm.rank) if comm is not None else (1, 0)
    rng = np.random.default_rng(seed)
    net = SurrogateNet((n, n, n), batch=batch, channels=channels, training=True)
    net.set_params(init_params(channels, seed) if params is None else params)
    u = torch.empty((batch, n, n, n), device="cuda")
    k = torch.empty_like(u)
    tgt = torch.empty_like(u)
    du = torch.empty_like(u)
    hist = []
    try:
        for it in range(iters):
            j = rng.integers(0, count, batch * world)[rank * batch:(rank + 1) * batch]
            c = rng.integers(0, calls1 - 1, batch * world)[rank * batch:(rank + 1) * batch]
            ji = torch.as_tensor(j, device="cuda")
            ci = torch.as_tensor(c, device="cuda")
            u.copy_(states[ji, ci])
            k.copy_(kappa[ji])
            tgt.copy_(states[ji, ci + 1] - states[ji, ci])
            torch.cuda.synchronize()
            net.forward(u, k, du)
            loss = net.backward(tgt)
            if world > 1:
                net.set_grads(comm.allreduce_mean(net.get_grads()))
                loss = float(comm.allreduce_mean(np.array([loss]))[0])
            net.adam(lr=lr * (0.1 if it > 0.8 * iters else 1.0))
            hist.append(loss)
            if log and (it % 100 == 0 or it == iters - 1):
                log("iter %d loss %.3e" % (it, loss))
        net.synchronize()
        return net.get_params(), hist
    finally:
        net.close()


def one_call_errors(params, states, kappa, channels: int = 24):
    """Relative L2 error of one surrogate call and of the no-learning
    baseline (u unchanged) against the plain stencil, over all pairs."""
    import torch
    count, calls1, n = states.shape[0], states.shape[1], states.shape[2]
    net = SurrogateNet((n, n, n), batch=1, channels=channels)
    net.set_params(params)
    du = torch.empty((1, n, n, n), device="cuda")
    num_net = num_id = den = 0.0
    try:
        for j in range(count):
            for c in range(calls1 - 1):
                u = states[j, c].contiguous()
                net.forward(u, kappa[j].contiguous(), du)
                net.synchronize()
                target = states[j, c + 1]
                num_net += float(((u + du[0] - target) ** 2).sum())
                num_id += float(((u - target) ** 2).sum())
                den += float((target ** 2).sum())
    finally:
        net.close()
    return np.sqrt(num_net / den), np.sqrt(num_id / den)


def rel_l2(a, b) -> float:
    import torch
    return float(torch.linalg.vector_norm((a - b).double()) / torch.linalg.vector_norm(b.double()))


def run_plain(u0, kappa, steps: int):
    """FP32 plain stencil for steps steps; returns (u, seconds)."""
    import torch
    n = u0.shape[-1]
    plain = PlainStencil(n)
    try:
        plain.set_kappa(kappa)
        u = u0.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plain.run(u, steps)
        torch.cuda.synchronize()
        return u, time.perf_counter() - t0
    finally:
        plain.close()


def run_surrogate_with_judge(params, u0, kappa, steps: int, tol: float = 1e-4, channels: int = 24):
    """Surrogate plus judge to `steps` plain steps (a multiple of 16 * 8).
    Returns (u, seconds, stats)."""
    import torch
    n = u0.shape[-1]
    net = SurrogateNet((n, n, n), batch=1, channels=channels)
    net.set_params(params)
    plain = PlainStencil(n)
    stats = {"segments": 0, "fallbacks": 0, "judge_errors": []}
    try:
        plain.set_kappa(kappa)
        u = u0.clone()
        prev = torch.empty_like(u)
        seg_start = torch.empty_like(u)
        check = torch.empty_like(u)
        seg_steps = STEPS_PER_CALL * CALLS_PER_JUDGE
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps // seg_steps):
            seg_start.copy_(u)
            torch.cuda.synchronize()     # the copy (torch's stream) before the net's stream writes u
            net.advance(u, kappa, CALLS_PER_JUDGE - 1)
            net.synchronize()
            prev.copy_(u)
            torch.cuda.synchronize()
            net.advance(u, kappa, 1)
            net.synchronize()
            check.copy_(prev)
            plain.run(check, STEPS_PER_CALL)
            err = rel_l2(u, check)
            stats["judge_errors"].append(err)
            stats["segments"] += 1
            if not (err <= tol):     # a non-finite error fails the judge too

                stats["fallbacks"] += 1
                u.copy_(seg_start)
                plain.run(u, seg_steps)
        torch.cuda.synchronize()
        return u, time.perf_counter() - t0, stats
    finally:
        net.close()
        plain.close()


def time_calls(params, u0, kappa, calls: int = 8, channels: int = 24) -> float:
    """Milliseconds per network call (u <- u + net(u, kappa)), CUDA events on
    the network's stream, after one warm-up call."""
    import torch
    n = u0.shape[-1]
    net = SurrogateNet((n, n, n), batch=1, channels=channels)
    try:
        net.set_params(params)
        u = u0.clone()
        torch.cuda.synchronize()
        net.advance(u, kappa, 1)
        net.synchronize()
        st = torch.cuda.ExternalStream(net.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        net.advance(u, kappa, calls)
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / calls
    finally:
        net.close()
