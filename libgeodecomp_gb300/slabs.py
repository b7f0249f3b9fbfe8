"""Slab decomposition of a structured grid over ranks, one GPU per rank.

The grid is cut along its slowest axis (z in 3D, y in 2D) into one slab per
rank.  Every rank holds its slab plus G ghost planes on each side that
faces another rank, and advances its whole local grid; after T = G / R
steps (R the stencil radius, 1 here) the ghost planes are stale, and the
ranks exchange the G planes next to each neighbour before stepping on.
This is the ghost-zone model of the reference's HiParSimulator
(parallelization/hiparsimulator.h:60-72: ghostZoneWidth, the inner and
outer ghost zones its steppers update; the patch links of
communication/patchlink.h carry them), for the library's whole-grid steps:
the owned planes stay exact for T steps because wrong values spread one
plane per step from the ghost zone's outer face.

Results equal a single grid's bit for bit: the cells update from the same
neighbours in the same order, and a fixed-point grid keeps one exponent on
every rank (pinned: the automatic lowering of a single grid is per grid).

Exchanges move raw planes (the device representation, row padding
included) through lgd_gpu_copy_planes: with NCCL straight between device
buffers, with gloo through host memory.  The slab logic itself - the
partition, the ghost widths and the exchange plan - is host code with no
GPU in it, so it is tested on CPU ranks with a stand-in stepper.
"""
from __future__ import annotations

import numpy as np


def partition(n: int, world: int, rank: int):
    """Owned planes [p0, p1) of a rank: an even split, the first n % world
    ranks one plane more."""
    base, extra = divmod(n, world)
    p0 = rank * base + min(rank, extra)
    return p0, p0 + base + (1 if rank < extra else 0)


class SlabLayout:
    """Where a rank's planes lie and what it exchanges.

    n_planes: the global grid's planes along the cut axis; ghost: G, the
    ghost planes per side that faces another rank; periodic: the cut axis
    wraps (the first and last rank are neighbours)."""

    def __init__(self, n_planes: int, world: int, rank: int, ghost: int, periodic: bool):
        if world < 1 or not 0 <= rank < world:
            raise ValueError("rank outside the world")
        if ghost < 1:
            raise ValueError("ghost width must be at least one plane")
        self.n_planes, self.world, self.rank, self.ghost = n_planes, world, rank, ghost
        self.periodic = periodic
        self.p0, self.p1 = partition(n_planes, world, rank)
        if world > 1 and (self.p1 - self.p0) < ghost:
            raise ValueError("every rank needs at least %d planes (the ghost width)" % ghost)
        if world == 1:
            self.lower = self.upper = None
        else:
            self.lower = rank - 1 if rank > 0 else (world - 1 if periodic else None)
            self.upper = rank + 1 if rank < world - 1 else (0 if periodic else None)
        self.ghost_lo = ghost if self.lower is not None else 0
        self.ghost_hi = ghost if self.upper is not None else 0
        self.owned = self.p1 - self.p0
        self.local_planes = self.ghost_lo + self.owned + self.ghost_hi
        # the local grid wraps along the cut axis only when one rank holds
        # the whole periodic axis
        self.local_periodic = periodic and world == 1

    def global_range(self):
        """Global planes [g0, g1) of the local grid (g0 may be negative and
        g1 beyond the grid on a periodic axis: those wrap)."""
        return self.p0 - self.ghost_lo, self.p1 + self.ghost_hi

    def exchanges(self):
        """(neighbour, local planes to send [s0, s0 + G), local planes to
        receive into [r0, r0 + G)) per neighbour, lower side first.  With two
        ranks on a periodic axis the same neighbour appears on both sides."""
        out = []
        G = self.ghost
        if self.lower is not None:
            out.append((self.lower, self.ghost_lo, 0))
        if self.upper is not None:
            out.append((self.upper, self.ghost_lo + self.owned - G, self.ghost_lo + self.owned))
        return out


class TorchComm:
    """Point-to-point byte exchange over torch.distributed: NCCL between
    device buffers, gloo through host buffers."""

    def __init__(self, dist, device: bool):
        self.dist = dist
        self.device = device
        self.world = dist.get_world_size()
        self.rank = dist.get_rank()

    def exchange(self, sends, recvs):
        """sends: [(peer, tensor)], recvs: [(peer, tensor)], posted as one
        batch: with NCCL the operations of a batch run as one group, so a
        receive queued ahead of a send cannot block it (pairs of ranks that
        each receive first would deadlock otherwise), and operations to the
        same peer are matched in the order they were posted."""
        ops = [self.dist.P2POp(self.dist.irecv, t, peer) for peer, t in recvs]
        ops += [self.dist.P2POp(self.dist.isend, t, peer) for peer, t in sends]
        if not ops:
            return
        for r in self.dist.batch_isend_irecv(ops):
            r.wait()

    def allgather(self, send, recvs):
        """recvs[q] <- rank q's send (equal sizes), every rank."""
        self.dist.all_gather(recvs, send)

    def allreduce_mean(self, a: np.ndarray) -> np.ndarray:
        """The mean over ranks of a host array, on every rank."""
        import torch
        t = torch.from_numpy(np.ascontiguousarray(a))
        if self.device:
            t = t.cuda()
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return (t.cpu().numpy() / self.world).astype(a.dtype)

    def max_int(self, v: int) -> int:
        import torch
        t = torch.tensor([v], dtype=torch.int64, device="cuda" if self.device else "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return int(t.item())

    def max_float(self, v: float) -> float:
        import torch
        t = torch.tensor([v], dtype=torch.float64, device="cuda" if self.device else "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())


class InProcessComm:
    """Ranks as threads of one process (several slabs of one grid on one
    GPU, or CPU tests): the same exchange through a shared mailbox.  Build
    one per rank from a shared InProcessComm.Hub(world)."""

    class Hub:
        def __init__(self, world: int):
            import threading
            self.world = world
            self.box = {}
            self.lock = threading.Lock()
            self.barrier = threading.Barrier(world)

    def __init__(self, hub: "InProcessComm.Hub", rank: int, device: bool = False):
        """device: the exchange buffers are CUDA tensors filled and drained by
        device-to-device plane copies (the path NCCL ranks take)."""
        self.hub = hub
        self.world = hub.world
        self.rank = rank
        self.device = device
        self.torch_buffers = device
        self.dist = None

    def exchange(self, sends, recvs):
        # a (src, dst) pair can carry two messages (two ranks on a periodic
        # axis are each other's lower and upper neighbour): keep their order
        with self.hub.lock:
            for k, (peer, t) in enumerate(sends):
                self.hub.box.setdefault((self.rank, peer), []).append(
                    t.clone() if self.device else np.array(t, copy=True))
        self.hub.barrier.wait()
        with self.hub.lock:
            for peer, t in recvs:
                msg = self.hub.box[(peer, self.rank)].pop(0)
                if self.device:
                    t.copy_(msg)
                else:
                    t[...] = msg
        self.hub.barrier.wait()

    def allgather(self, send, recvs):
        with self.hub.lock:
            self.hub.box[("gather", self.rank)] = send.clone() if self.device else np.array(send, copy=True)
        self.hub.barrier.wait()
        for q in range(self.world):
            msg = self.hub.box[("gather", q)]
            if self.device:
                recvs[q].copy_(msg)
            else:
                recvs[q][...] = msg
        self.hub.barrier.wait()

    def allreduce_mean(self, a: np.ndarray) -> np.ndarray:
        """The mean over ranks of a host array, summed in rank order."""
        parts = [p for _, p in sorted(self._reduce((self.rank, np.array(a, copy=True)), list),
                                      key=lambda rp: rp[0])]
        acc = parts[0].copy()
        for p in parts[1:]:
            acc = acc + p
        return (acc / self.world).astype(a.dtype)

    def _reduce(self, v, fn):
        with self.hub.lock:
            self.hub.box.setdefault("reduce", []).append(v)
        self.hub.barrier.wait()
        out = fn(self.hub.box["reduce"])
        self.hub.barrier.wait()
        if self.rank == 0:
            with self.hub.lock:
                del self.hub.box["reduce"]
        self.hub.barrier.wait()
        return out

    def max_int(self, v: int) -> int:
        return self._reduce(int(v), max)

    def max_float(self, v: float) -> float:
        return self._reduce(float(v), max)


class SlabGrid:
    """One rank's slab of a structured grid with its ghost zones.

    make_grid(local_shape, periodic_mask) creates the local grid: a
    libgeodecomp_gb300.lgd.Grid on the GPU, or any object with step(n),
    save_planes(p0, n), load_planes(p0, data), plane_bytes(), and for
    fixed-point cells fixed_point_exponent() / set_fixed_point_exponent(e,
    pin).  shape is the global (nz, ny, nx) or (ny, nx); periodic the global
    mask (bit 0 x, 1 y, 2 z)."""

    def __init__(self, cell, shape, comm, periodic: int = 0, ghost: int = 8, time_block: int = 0,
                 make_grid=None, fixed_point: bool | None = None):
        shape = tuple(int(s) for s in shape)
        self.shape = shape
        self.dim = len(shape)
        if self.dim not in (2, 3):
            raise ValueError("slabs cut 2D and 3D grids")
        self.cut_bit = 1 << (self.dim - 1)          # z in 3D, y in 2D
        self.comm = comm
        world, rank = (comm.world, comm.rank) if comm is not None else (1, 0)
        self.layout = SlabLayout(shape[0], world, rank, ghost, bool(periodic & self.cut_bit))
        local_mask = periodic & ~self.cut_bit
        if periodic & self.cut_bit:
            # one rank: the whole periodic axis wraps locally.  Several: every
            # face of every slab is a ghost face, and what lies beyond a ghost
            # zone never reaches the owned planes between two exchanges, so
            # the local grid may wrap there too - which keeps the torus fast
            # paths (Game of Life's bit-sliced passes, the var-coef TMA ring)
            local_mask |= self.cut_bit
        self.local_shape = (self.layout.local_planes,) + shape[1:]
        if make_grid is None:
            from libgeodecomp_gb300 import lgd

            def make_grid(local_shape, mask):
                return lgd.Grid(cell, local_shape, periodic=mask)
            if fixed_point is None:
                fixed_point = cell == lgd.CELL_JACOBI7_F64_FIX
        self.fixed_point = bool(fixed_point)
        self.grid = make_grid(self.local_shape, local_mask)
        if time_block and hasattr(self.grid, "set_time_block"):
            self.grid.set_time_block(time_block)
        self.period = ghost                       # steps between exchanges (radius 1)
        self.since = self.period                  # ghosts are stale until the first exchange
        self.exchange_count = 0
        self._bufs = {}

    # -------------------------------------------------------------- data
    def owned_slice(self):
        return slice(self.layout.ghost_lo, self.layout.ghost_lo + self.layout.owned)

    def _local_rows(self, values: np.ndarray):
        """The global array's planes of this rank's local grid (ghosts
        wrapped on a periodic axis)."""
        g0, g1 = self.layout.global_range()
        idx = np.arange(g0, g1) % self.shape[0]
        return np.ascontiguousarray(values[idx])

    def _agree_exponent(self, local_max: float):
        """A fixed-point grid takes the exponent of the global maximum on
        every rank, pinned, before values are converted."""
        if not self.fixed_point:
            return
        m = self.comm.max_float(local_max) if self.comm is not None else local_max
        e = int(np.frexp(m)[1]) if m > 0 else 0
        self.grid.set_fixed_point_exponent(e, True)

    def upload(self, member: int, values: np.ndarray):
        """Loads this rank's part of a global array (shape = the grid's)."""
        values = np.asarray(values)
        if values.shape != self.shape:
            raise ValueError("values have shape %s, the grid %s" % (values.shape, self.shape))
        local = self._local_rows(values)
        if member == 0:
            self._agree_exponent(float(np.max(np.abs(values))) if values.size else 0.0)
        self.grid.upload(member, local)
        self.since = self.period

    def fill_uniform(self, seed: int = 42, stream: int = 1):
        """The library's seeded U[0,1) fill of the global grid, each rank
        generating its own planes (the values depend on the global index
        only, so this equals a fill of the whole grid)."""
        self._agree_exponent(1.0 - 2.0 ** -53)
        from libgeodecomp_gb300 import workloads
        # generate on the host per plane range: index = global plane offset
        n_plane = int(np.prod(self.shape[1:]))
        g0, g1 = self.layout.global_range()
        planes = np.arange(g0, g1) % self.shape[0]
        out = np.empty((len(planes),) + self.shape[1:])
        for i, p in enumerate(planes):
            out[i] = workloads.uniform(seed, stream, n_plane, offset=int(p) * n_plane).reshape(self.shape[1:])
        self.grid.upload(0, out)
        self.since = self.period

    def fill_bernoulli(self, p: float, seed: int = 42, stream: int = 1):
        """Bernoulli(p) 0/1 cells of the global grid (value i = 1 if the
        library's uniform i < p), each rank generating its own planes."""
        from libgeodecomp_gb300 import workloads
        n_plane = int(np.prod(self.shape[1:]))
        g0, g1 = self.layout.global_range()
        planes = np.arange(g0, g1) % self.shape[0]
        out = np.empty((len(planes),) + self.shape[1:], dtype=np.uint8)
        for i, q in enumerate(planes):
            u = workloads.uniform(seed, stream, n_plane, offset=int(q) * n_plane)
            out[i] = (u < p).astype(np.uint8).reshape(self.shape[1:])
        self.grid.upload(0, out)
        self.since = self.period

    def download_owned(self, member: int = 0) -> np.ndarray:
        return self.grid.download(member)[self.owned_slice()]

    def gather(self, member: int = 0) -> np.ndarray | None:
        """The whole grid on rank 0 (None elsewhere), through the comm's
        host path; for tests and small grids."""
        own = self.download_owned(member)
        if self.comm is None:
            return own
        import torch
        dist = self.comm.dist
        parts = None
        if self.comm.rank == 0:
            parts = [own]
            for r in range(1, self.comm.world):
                p0, p1 = partition(self.shape[0], self.comm.world, r)
                t = torch.empty(((p1 - p0),) + self.shape[1:], dtype=torch.from_numpy(own[:0]).dtype)
                dist.recv(t, src=r)
                parts.append(t.numpy())
            return np.concatenate(parts, axis=0)
        dist.send(torch.from_numpy(np.ascontiguousarray(own)), dst=0)
        return None

    # ------------------------------------------------------------- steps
    def exchange(self):
        """Each rank's G planes next to a neighbour into that neighbour's
        ghost zone (raw planes, device representation)."""
        lay = self.layout
        if lay.world == 1 or not lay.exchanges():
            self.since = 0
            return
        G = lay.ghost
        pb = self.grid.plane_bytes()
        device = self.comm.device
        torch_bufs = getattr(self.comm, "torch_buffers", self.comm.dist is not None)
        if torch_bufs:
            import torch
        sends, recvs, landing = [], [], []
        for k, (peer, s0, r0) in enumerate(lay.exchanges()):
            if k not in self._bufs:
                if torch_bufs:
                    dev = "cuda" if device else "cpu"
                    self._bufs[k] = (torch.empty(G * pb, dtype=torch.uint8, device=dev),
                                     torch.empty(G * pb, dtype=torch.uint8, device=dev))
                else:
                    self._bufs[k] = (np.empty(G * pb, dtype=np.uint8), np.empty(G * pb, dtype=np.uint8))
            sbuf, rbuf = self._bufs[k]
            if device:
                self.grid.copy_planes_device(s0, G, sbuf.data_ptr(), to_grid=False)
            else:
                self.grid.save_planes(s0, G, out=sbuf.numpy() if torch_bufs else sbuf)
            sends.append((peer, sbuf))
            # receives post in the opposite order: messages between a pair
            # of ranks arrive in send order, and a neighbour's lower-side
            # planes (its first message) fill this rank's upper ghost zone
            # (two ranks on a periodic axis are each other's lower and upper
            # neighbour)
            recvs.insert(0, (peer, rbuf))
            landing.append((r0, rbuf))
        if device:
            torch.cuda.synchronize()
        self.comm.exchange(sends, recvs)
        if device:
            torch.cuda.synchronize()
        for r0, rbuf in landing:
            if device:
                self.grid.copy_planes_device(r0, G, rbuf.data_ptr(), to_grid=True)
            else:
                self.grid.load_planes(r0, rbuf.numpy() if torch_bufs else rbuf)
        self.exchange_count += 1
        self.since = 0

    def step(self, n: int):
        """n time steps of the global grid."""
        while n > 0:
            if self.since >= self.period:
                self.exchange()
            k = min(n, self.period - self.since)
            self.grid.step(k)
            self.since += k
            n -= k

    def synchronize(self):
        if hasattr(self.grid, "synchronize"):
            self.grid.synchronize()

    def launch_count(self) -> int:
        return self.grid.launch_count() if hasattr(self.grid, "launch_count") else 0

    def describe(self) -> dict:
        lay = self.layout
        return {"ranks": lay.world, "planes_owned": lay.owned, "ghost_planes": lay.ghost,
                "local_planes": lay.local_planes, "exchange_every_steps": self.period,
                "exchanges": self.exchange_count,
                "path": "NCCL between device buffers" if (self.comm is not None and self.comm.device)
                else "host buffers (gloo)"}

    def close(self):
        if hasattr(self.grid, "close"):
            self.grid.close()
