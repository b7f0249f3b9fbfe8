"""Row-block decomposition of a SELL-C-sigma diffusion grid over ranks, one
GPU per rank.

Every rank holds the matrix (built from the same CSR, so every rank has the
same sigma-sorted physical order) and both node-value buffers.  A step
updates the rank's own block of physical rows - whole chunks, so warps never
straddle two ranks - into the next buffer (lgd_sell_update_rows), then the
ranks gather every block of the next buffer (one all-gather per step, the
path's only communication) and swap.  A row's sum runs over its entries in
the same order on every rank as in one grid, so the result equals one
grid's bit for bit.

This is the unstructured counterpart of the structured slabs
(libgeodecomp_gb300.slabs): the reference's HiParSimulator gives each node
a region of the grid and trades the neighbour values its region reads
through patch links (parallelization/hiparsimulator.h,
communication/patchlink.h).  Here the halo is every block: with targets
drawn uniformly at random (the configuration's graph) a block of half the
rows reads about 99.7% of all nodes, so gathering the set of columns a
block reads would move nearly the whole vector anyway, at the cost of an
index list per peer.  The matrix is held whole on every rank (0.8 GB for
the 4.19 M-node configuration); a rank that stores only its rows' entries
needs the same gather.

make_grid() returns the local grid: a libgeodecomp_gb300.lgd.SellGrid, or
any object with update_rows(r0, r1), swap(), download(logical, which),
upload(x, logical, which) and n (the CPU tests' numpy stand-in); with
device=True comms the next buffer is gathered device to device through
x_device().
"""
from __future__ import annotations

import numpy as np


class RowBlocks:
    """Chunk-aligned blocks of physical rows: rank r updates rows
    [r * B, min((r + 1) * B, n)), B = ceil(chunks / world) * C; the last
    ranks' blocks may be short or empty."""

    def __init__(self, n: int, C: int, world: int):
        self.n, self.C, self.world = n, C, world
        n_chunks = (n + C - 1) // C
        self.block = ((n_chunks + world - 1) // world) * C
        self.ranges = [(min(r * self.block, n), min((r + 1) * self.block, n)) for r in range(world)]

    def rows(self, rank: int):
        return self.ranges[rank]


class ShardedSell:
    """One rank's share of the steps of a SELL-C-sigma diffusion grid."""

    def __init__(self, grid, comm, C: int, precision: int = 8):
        self.grid = grid
        self.comm = comm
        self.world, self.rank = (comm.world, comm.rank) if comm is not None else (1, 0)
        self.blocks = RowBlocks(grid.n, C, self.world)
        self.precision = precision
        self.gathers = 0
        self._bufs = None

    # --------------------------------------------------------- exchange
    def _gather_host(self):
        """The next buffer's blocks through host memory (gloo, or threads)."""
        B = self.blocks.block
        dtype = np.float64
        xn = self.grid.download(logical=False, which=1)
        r0, r1 = self.blocks.rows(self.rank)
        torch_bufs = getattr(self.comm, "dist", None) is not None
        if self._bufs is None:
            if torch_bufs:
                import torch
                self._bufs = (torch.zeros(B, dtype=torch.float64),
                              [torch.zeros(B, dtype=torch.float64) for _ in range(self.world)])
            else:
                self._bufs = (np.zeros(B, dtype=dtype), [np.zeros(B, dtype=dtype) for _ in range(self.world)])
        send, recvs = self._bufs
        sv = send.numpy() if torch_bufs else send
        sv[:r1 - r0] = xn[r0:r1]
        self.comm.allgather(send, recvs)
        for q, (q0, q1) in enumerate(self.blocks.ranges):
            if q != self.rank and q1 > q0:
                rv = recvs[q].numpy() if torch_bufs else recvs[q]
                xn[q0:q1] = rv[:q1 - q0]
        self.grid.upload(xn, logical=False, which=1)

    def _gather_device(self):
        """The next buffer's blocks device to device (NCCL, or threads
        sharing one GPU)."""
        import torch
        B = self.blocks.block
        dt = torch.float64 if self.precision == 8 else torch.float32
        ptr, rows_padded = self.grid.x_device(1)
        xn = _device_view(ptr, rows_padded, dt)
        if self._bufs is None:
            self._bufs = (torch.zeros(B, dtype=dt, device="cuda"),
                          [torch.zeros(B, dtype=dt, device="cuda") for _ in range(self.world)])
        send, recvs = self._bufs
        r0, r1 = self.blocks.rows(self.rank)
        self.grid.synchronize()
        send[:r1 - r0].copy_(xn[r0:r1])
        torch.cuda.synchronize()
        self.comm.allgather(send, recvs)
        for q, (q0, q1) in enumerate(self.blocks.ranges):
            if q != self.rank and q1 > q0:
                xn[q0:q1].copy_(recvs[q][:q1 - q0])
        torch.cuda.synchronize()

    # ------------------------------------------------------------ steps
    def step(self, n: int = 1):
        r0, r1 = self.blocks.rows(self.rank)
        for _ in range(n):
            if r1 > r0:
                self.grid.update_rows(r0, r1)
            if self.world > 1:
                if getattr(self.comm, "device", False):
                    self._gather_device()
                else:
                    self._gather_host()
                self.gathers += 1
            self.grid.swap()

    def synchronize(self):
        if hasattr(self.grid, "synchronize"):
            self.grid.synchronize()

    def describe(self) -> dict:
        r0, r1 = self.blocks.rows(self.rank)
        return {"ranks": self.world, "rows_of_rank": r1 - r0, "block_rows": self.blocks.block,
                "gathers": self.gathers,
                "path": "all-gather between device buffers" if getattr(self.comm, "device", False)
                else "all-gather through host memory"}


class _CudaArray:
    """A raw device allocation seen by torch (__cuda_array_interface__)."""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3,
                                         "strides": None}


def _device_view(ptr: int, n: int, dtype):
    import torch
    typestr = "<f8" if dtype == torch.float64 else "<f4"
    return torch.as_tensor(_CudaArray(ptr, n, typestr), device="cuda")
