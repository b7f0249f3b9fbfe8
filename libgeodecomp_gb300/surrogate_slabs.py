"""Inference of the learned surrogate, judge included, on z-slabs of the
torus, one per rank.

Every rank holds its slab of u and kappa plus G ghost planes on each side
and treats the local array as a torus along z as well (the network's
kernels and the plain stencil wrap every axis): what the wrap brings in at
the ghost zone's outer faces moves one plane per 3^3 layer, or per plain
step, towards the owned planes.  A network call runs four layers, so it
uses up four ghost planes; the judge's sixteen plain steps use up sixteen.
With G = 16 a rank refreshes its ghost planes (an exchange with its two
neighbours) whenever the next operation needs more ghost planes than are
left: every four calls, and before each block of sixteen plain steps.  The
owned planes therefore equal the single torus' bit for bit - a voxel's
arithmetic does not depend on where its slab lies - and the judge's
relative L2 error is summed over the owned planes of every rank (one
all-reduce of two numbers), so every rank takes the same fallback decision
as the single torus.

This is the ghost-zone model of the slab decomposition of the plain
stencils (libgeodecomp_gb300.slabs; the reference's HiParSimulator,
parallelization/hiparsimulator.h:60-72), with the ghost width set by the
network's depth.  The slab logic is host code: make_net and make_plain take
stand-ins, so it is tested on CPU ranks too.
"""
from __future__ import annotations

import time

import numpy as np

from . import slabs
from .surrogate import CALLS_PER_JUDGE, STEPS_PER_CALL

LAYERS = 4                   # 3^3 layers per call: ghost planes one call uses up
GHOST = STEPS_PER_CALL       # ghost planes per side: one judge run, or four calls


class SlabSurrogate:
    """One rank's slab of a surrogate run on a torus cut along z.

    params: the network's parameters; shape: the torus, (nz, ny, nx) or n
    for n^3 (the network's kernels want nx a multiple of 32 and ny of 4);
    comm: a slabs.TorchComm or
    slabs.InProcessComm (None: one rank, the whole torus); make_net(shape) /
    make_plain(shape): the network (advance(u, kappa, calls), synchronize(),
    close()) and the plain stencil (set_kappa(k), run(u, steps), close()) on
    the local torus - by default libgeodecomp_gb300.surrogate.SurrogateNet
    and PlainStencil on the GPU."""

    def __init__(self, params, shape, comm=None, ghost: int = GHOST, channels: int = 24, make_net=None,
                 make_plain=None):
        import torch
        self._torch = torch
        if ghost < STEPS_PER_CALL:
            raise ValueError("the ghost zone must hold one judge run of %d plain steps" % STEPS_PER_CALL)
        self.comm = comm
        world, rank = (comm.world, comm.rank) if comm is not None else (1, 0)
        self.shape = (int(shape),) * 3 if np.isscalar(shape) else tuple(int(s) for s in shape)
        self.layout = slabs.SlabLayout(self.shape[0], world, rank, ghost, periodic=True)
        self.local_shape = (self.layout.local_planes,) + self.shape[1:]
        if make_net is None or make_plain is None:
            from . import surrogate as S
            if make_net is None:
                def make_net(shape):
                    net = S.SurrogateNet(shape, batch=1, channels=channels)
                    net.set_params(params)
                    return net
            if make_plain is None:
                def make_plain(shape):
                    return S.PlainStencil(shape=shape)
        self.net = make_net(self.local_shape)
        try:
            self.plain = make_plain(self.local_shape)
        except Exception:
            self.net.close()
            raise
        self.kappa = None
        self.exchange_count = 0
        self._bufs = None
        self.stats = {"segments": 0, "fallbacks": 0, "judge_errors": []}

    # -------------------------------------------------------------- data
    def owned_slice(self):
        return slice(self.layout.ghost_lo, self.layout.ghost_lo + self.layout.owned)

    def cut(self, field, device=None):
        """This rank's local planes (ghost planes included, wrapped around
        the torus) of a global field, as a contiguous float32 tensor on
        device (default: the field's own device; numpy fields go to CUDA
        when it is available)."""
        torch = self._torch
        t = field if isinstance(field, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(field))
        if device is None:
            device = t.device if isinstance(field, torch.Tensor) else ("cuda" if torch.cuda.is_available() else "cpu")
        g0, g1 = self.layout.global_range()
        if tuple(t.shape) != self.shape:
            raise ValueError("field of shape %s for a torus of %s" % (tuple(t.shape), self.shape))
        idx = torch.as_tensor(np.arange(g0, g1) % self.shape[0], device=t.device)
        return t.index_select(0, idx).to(device=device, dtype=torch.float32).contiguous()

    def set_kappa(self, kappa):
        """The coefficient field: the global field, cut here."""
        self.kappa = self.cut(kappa)
        self._sync(self.kappa)
        self.plain.set_kappa(self.kappa)

    # ------------------------------------------------------------ ghosts
    def _sync(self, t):
        if t.is_cuda:
            self._torch.cuda.synchronize()

    def exchange(self, u):
        """u's G planes next to each neighbour into that neighbour's ghost
        zone, and the neighbours' into this rank's."""
        lay = self.layout
        if lay.world == 1:
            return
        torch = self._torch
        G = lay.ghost
        device = bool(self.comm.device)
        torch_bufs = getattr(self.comm, "torch_buffers", self.comm.dist is not None)
        planes = (G,) + self.local_shape[1:]
        if self._bufs is None:
            self._bufs = []
            for _ in lay.exchanges():
                if device:
                    self._bufs.append((torch.empty(planes, dtype=torch.float32, device=u.device),
                                       torch.empty(planes, dtype=torch.float32, device=u.device)))
                elif torch_bufs:
                    self._bufs.append((torch.empty(planes, dtype=torch.float32),
                                       torch.empty(planes, dtype=torch.float32)))
                else:
                    self._bufs.append((np.empty(planes, dtype=np.float32), np.empty(planes, dtype=np.float32)))
        self.net.synchronize()
        self._sync(u)
        sends, recvs, landing = [], [], []
        for (peer, s0, r0), (sbuf, rbuf) in zip(lay.exchanges(), self._bufs):
            src = u[s0:s0 + G]
            if device or torch_bufs:
                sbuf.copy_(src)
            else:
                sbuf[...] = src.cpu().numpy()
            sends.append((peer, sbuf))
            # a neighbour's lower-side planes (its first message) fill this
            # rank's upper ghost zone; messages between a pair of ranks
            # arrive in send order (two ranks on the torus are each other's
            # lower and upper neighbour), so receives post in reverse
            recvs.insert(0, (peer, rbuf))
            landing.append((r0, rbuf))
        self._sync(u)
        self.comm.exchange(sends, recvs)
        for r0, rbuf in landing:
            u[r0:r0 + G].copy_(rbuf if isinstance(rbuf, torch.Tensor) else torch.from_numpy(rbuf))
        self._sync(u)
        self.exchange_count += 1

    def _need(self, u, left, planes):
        """Refreshes u's ghost planes when fewer than planes are left;
        returns the ghost planes left after that."""
        if self.layout.world > 1 and left < planes:
            self.exchange(u)
            return self.layout.ghost
        return left

    # -------------------------------------------------------------- run
    def _rel_l2(self, a, b):
        own = self.owned_slice()
        d = (a[own] - b[own]).double()
        num = float((d * d).sum())
        den = float((b[own].double() ** 2).sum())
        if self.comm is not None and self.layout.world > 1:
            num, den = (float(v) for v in self.comm.allreduce_mean(np.array([num, den], dtype=np.float64)))
        with np.errstate(divide="ignore", invalid="ignore"):
            return float(np.sqrt(np.float64(num) / np.float64(den)))

    def run(self, u0, steps: int, tol: float = 1e-4):
        """Surrogate plus judge to `steps` plain steps (a multiple of 16 * 8)
        from u0 (the global field), in the single torus' scheme
        (libgeodecomp_gb300.surrogate.run_surrogate_with_judge): per segment
        seven calls, the state kept, an eighth call, the plain stencil's
        sixteen steps from the kept state as the judge, the segment redone
        with the plain stencil if the judge's error exceeds tol.  Returns
        (the owned planes, seconds, stats)."""
        torch = self._torch
        if self.kappa is None:
            raise RuntimeError("set_kappa() first")
        u = self.cut(u0, device=self.kappa.device)
        prev = torch.empty_like(u)
        seg_start = torch.empty_like(u)
        check = torch.empty_like(u)
        seg_steps = STEPS_PER_CALL * CALLS_PER_JUDGE
        # ghost planes whose values are exact: all of them after the cut
        left = float("inf") if self.layout.world == 1 else self.layout.ghost
        self._sync(u)
        t0 = time.perf_counter()
        for _ in range(steps // seg_steps):
            left = self._need(u, left, STEPS_PER_CALL)    # the fallback replays from here
            seg_start.copy_(u)
            self._sync(u)
            start_left = left
            for _ in range(CALLS_PER_JUDGE - 1):
                left = self._need(u, left, LAYERS)
                self.net.advance(u, self.kappa, 1)
                left -= LAYERS
            self.net.synchronize()
            left = self._need(u, left, STEPS_PER_CALL)    # the judge's steps start from prev
            prev.copy_(u)
            self._sync(u)
            prev_left = left
            self.net.advance(u, self.kappa, 1)
            left -= LAYERS
            self.net.synchronize()
            check.copy_(prev)
            if prev_left < STEPS_PER_CALL:           # _need above makes this impossible
                raise RuntimeError("the judge's state holds too few exact ghost planes")
            self.plain.run(check, STEPS_PER_CALL)
            err = self._rel_l2(u, check)
            self.stats["judge_errors"].append(err)
            self.stats["segments"] += 1
            if not (err <= tol):     # a non-finite error fails the judge too
                self.stats["fallbacks"] += 1
                u.copy_(seg_start)
                left = start_left
                for _ in range(CALLS_PER_JUDGE):
                    left = self._need(u, left, STEPS_PER_CALL)
                    self.plain.run(u, STEPS_PER_CALL)
                    left -= STEPS_PER_CALL
        self._sync(u)
        return u[self.owned_slice()].clone(), time.perf_counter() - t0, self.stats

    def describe(self) -> dict:
        lay = self.layout
        return {"ranks": lay.world, "planes_owned": lay.owned, "ghost_planes": lay.ghost,
                "local_planes": lay.local_planes, "exchanges": self.exchange_count,
                "path": "NCCL between device buffers" if (self.comm is not None and self.comm.device)
                else "host buffers"}

    def close(self):
        try:
            self.net.close()
        finally:
            self.plain.close()
