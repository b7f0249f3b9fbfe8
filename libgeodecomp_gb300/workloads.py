"""Seeded synthetic inputs for the cell-update workloads.

Every workload draws from one counter-based generator, SplitMix64: the i-th
output of stream ``s`` under seed ``seed`` is ``mix(key + (i + 1) * GAMMA)``
with ``key = mix(seed * 256 + s)``.  A uniform double in [0, 1) is the top 53
bits of that output times 2**-53.  Because each value depends only on its
index, the device fill kernel (``lgd_gpu_fill_uniform``) produces the same
numbers as this module, and large grids can be generated on the GPU.

Logical cell order is x-fastest everywhere: ``idx = (z * ny + y) * nx + x``.

The reference ships no dataset for this path; these generators stand in for
the benchmark configurations' inputs (their shapes, sizes and value
distributions).
"""
from __future__ import annotations

import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

# stream ids, one per quantity drawn
STREAM_GRID = 1
STREAM_DEGREE = 2
STREAM_TARGET = 3
STREAM_WEIGHT = 4
STREAM_VALUE = 5
STREAM_EDGE = 6
STREAM_OMEGA = 7
STREAM_GRF_A = 8
STREAM_GRF_B = 9


def _mix(z: np.ndarray) -> np.ndarray:
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def stream_key(seed: int, stream: int) -> int:
    """Key of one stream: mix(seed * 256 + stream) (64-bit wrap-around)."""
    v = np.array([(int(seed) * 256 + int(stream)) & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64)
    return int(_mix(v)[0])


def splitmix64(seed: int, stream: int, n: int, offset: int = 0) -> np.ndarray:
    """Raw 64-bit outputs ``offset .. offset + n - 1`` of one stream."""
    key = np.uint64(stream_key(seed, stream))
    idx = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return _mix(key + idx * GAMMA)


def uniform(seed: int, stream: int, n: int, offset: int = 0) -> np.ndarray:
    """Doubles in [0, 1): (splitmix64 >> 11) * 2**-53."""
    r = splitmix64(seed, stream, n, offset)
    return (r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


# ----------------------------------------------------------------- Jacobi-7
def jacobi_initial(nx: int, ny: int, nz: int, seed: int = 42) -> np.ndarray:
    """U[0,1) FP64 temperatures, shape (nz, ny, nx)."""
    return uniform(seed, STREAM_GRID, nx * ny * nz).reshape(nz, ny, nx)


# ------------------------------------------------------------ Game of Life
def gol_initial(nx: int, ny: int, seed: int = 42, p: float = 0.3) -> np.ndarray:
    """Bernoulli(p) alive cells as uint8 0/1, shape (ny, nx)."""
    return (uniform(seed, STREAM_GRID, nx * ny) < p).astype(np.uint8).reshape(ny, nx)


# ------------------------------------------------------- SELL-C-sigma graph
def powerlaw_graph(n: int, seed: int = 42, dmin: int = 4, dmax: int = 64, alpha: float = 2.0):
    """Random directed graph with out-degrees from a truncated power law.

    Degree: d = floor(x) with x drawn from the continuous Pareto law
    p(x) ~ x**-alpha on [dmin, dmax + 1) by inverse transform, clipped to
    [dmin, dmax].  Targets: uniform over [0, n), sorted and made distinct
    within a row.  Weights: U[0,1) normalised so each row sums to 0.9.

    Returns ``(row_ptr int64[n+1], col int32[nnz], w float64[nnz])`` in CSR
    order (rows ascending, columns ascending within a row).
    """
    if dmax >= n:
        raise ValueError("dmax must be below the node count")
    u = uniform(seed, STREAM_DEGREE, n)
    a1 = alpha - 1.0
    lo = float(dmin)
    hi = float(dmax + 1)
    x = lo * (1.0 - u * (1.0 - (lo / hi) ** a1)) ** (-1.0 / a1)
    deg = np.clip(np.floor(x), dmin, dmax).astype(np.int64)
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(deg, out=row_ptr[1:])
    nnz = int(row_ptr[-1])
    rows = np.repeat(np.arange(n, dtype=np.int64), deg)
    k = np.arange(nnz, dtype=np.int64) - row_ptr[rows]

    r = splitmix64(seed, STREAM_TARGET, nnz)
    t = ((r >> np.uint64(32)) * np.uint64(n) >> np.uint64(32)).astype(np.int64)
    # sort targets within each row
    order = np.lexsort((t, rows))
    t = t[order]
    # strictly increasing within a row: t'[k] = max_{j<=k}(t[j] - j) + k
    big = np.int64(1) << np.int64(34)
    v = t - k + rows * big
    np.maximum.accumulate(v, out=v)
    t = v - rows * big + k
    # keep below n: t''[k] = min(t'[k], n - d + k)
    t = np.minimum(t, n - deg[rows] + k)

    uw = uniform(seed, STREAM_WEIGHT, nnz)
    rowsum = np.add.reduceat(uw, row_ptr[:-1])
    w = 0.9 * uw / rowsum[rows]
    return row_ptr, t.astype(np.int32), w


def sell_values(n: int, seed: int = 42) -> np.ndarray:
    """U[0,1) FP64 node values."""
    return uniform(seed, STREAM_VALUE, n)


# ------------------------------------------------------------ LBM ensemble
def lbm_ensemble(count: int = 512, seed: int = 42, edge_min: int = 32, edge_max: int = 192,
                 omega_min: float = 1.0, omega_max: float = 1.9):
    """Per-instance cube edge (uniform integer in [edge_min, edge_max]) and
    relaxation rate omega (uniform in [omega_min, omega_max))."""
    ue = uniform(seed, STREAM_EDGE, count)
    edges = edge_min + np.floor(ue * (edge_max - edge_min + 1)).astype(np.int64)
    edges = np.minimum(edges, edge_max)
    omegas = omega_min + (omega_max - omega_min) * uniform(seed, STREAM_OMEGA, count)
    return edges.astype(np.int32), omegas


# ------------------------------------------------ Gaussian random fields
def gaussian_random_field(n: int, length: float, seed: int, stream: int,
                          lo: float, hi: float) -> np.ndarray:
    """Periodic Gaussian random field on an n^3 torus, shape (n, n, n).

    White noise (Box-Muller from two uniform streams) is filtered in Fourier
    space by exp(-|k|^2 length^2 / 2) (Gaussian covariance with the given
    length scale in cells), then mapped linearly onto [lo, hi] by its min and
    max.
    """
    m = n * n * n
    u1 = uniform(seed, stream, m)
    u2 = uniform(seed, stream, m, offset=m)
    g = np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)
    g = g.reshape(n, n, n)
    k = 2.0 * np.pi * np.fft.fftfreq(n)
    kz = k[:, None, None]
    ky = k[None, :, None]
    kx = np.fft.rfftfreq(n)[None, None, :] * 2.0 * np.pi
    filt = np.exp(-0.5 * (kx * kx + ky * ky + kz * kz) * length * length)
    field = np.fft.irfftn(np.fft.rfftn(g) * filt, s=(n, n, n), axes=(0, 1, 2))
    fmin = field.min()
    fmax = field.max()
    return lo + (hi - lo) * (field - fmin) / (fmax - fmin)


def varcoef_fields(n: int = 256, seed: int = 42, length: float = 16.0):
    """(u0, kappa) for the variable-coefficient diffusion: u0 a GRF on
    [0, 1], kappa a separate GRF on [0.02, 0.15]."""
    kappa = gaussian_random_field(n, length, seed, STREAM_GRF_A, 0.02, 0.15)
    u0 = gaussian_random_field(n, length, seed, STREAM_GRF_B, 0.0, 1.0)
    return u0, kappa
