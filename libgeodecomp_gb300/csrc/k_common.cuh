// Device-side helpers shared by the kernels: pitched grid views, boundary
// handling (constant edge cell or periodic wrap, the reference's Cube and
// Torus topologies, geometry/topologies.h:179-278) and the per-cell update
// rules used by the generic (region) kernels.
#ifndef LGD_K_COMMON_CUH
#define LGD_K_COMMON_CUH

#include <stdint.h>

namespace lgd {

// A pitched 3D array: element (x, y, z) at p[(z * ny + y) * pitch + x].
template<typename T>
struct View {
    T *p;
    long pitch;
    int nx, ny, nz;
    __host__ __device__ T *row(int y, int z) const { return p + ((long)z * ny + y) * pitch; }
    __host__ __device__ T& at(int x, int y, int z) const { return p[((long)z * ny + y) * pitch + x]; }
};

__device__ __forceinline__ int wrap_axis(int i, int n)
{
    return (i < 0) ? i + n : ((i >= n) ? i - n : i);
}

// Value at (x, y, z) for a neighbour at most one cell outside the box:
// wrapped on periodic axes, the edge value on the others.
template<typename T>
__device__ __forceinline__ T load_bc(const View<const T>& v, int x, int y, int z, int periodic, T edge)
{
    if (x < 0 || x >= v.nx) {
        if (!(periodic & 1)) return edge;
        x = wrap_axis(x, v.nx);
    }
    if (y < 0 || y >= v.ny) {
        if (!(periodic & 2)) return edge;
        y = wrap_axis(y, v.ny);
    }
    if (z < 0 || z >= v.nz) {
        if (!(periodic & 4)) return edge;
        z = wrap_axis(z, v.nz);
    }
    return v.at(x, y, z);
}

// ---- SplitMix64 (matches libgeodecomp_gb300/workloads.py)
__host__ __device__ __forceinline__ uint64_t splitmix_mix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ double splitmix_uniform(uint64_t key, uint64_t i)
{
    uint64_t r = splitmix_mix(key + (i + 1) * 0x9E3779B97F4A7C15ull);
    return (double)(r >> 11) * (1.0 / 9007199254740992.0);
}

// ---- fixed-point representation of the FP64 Jacobi grid
// value = k * 2^(scale_exp - LGD_FIX_BITS), k a signed 64-bit integer,
// |value| < 2^scale_exp, so |k| < 2^56.  The averaging stencil maps
// [-S, S] into itself, so 7 * 2^56 bounds every neighbour sum, and 49 * 2^56
// < 2^62 every exact two-step sum (the temporally blocked pass): nothing
// overflows.  56 fraction bits: each rounding adds at most 2^(scale_exp - 57),
// e.g. 6.9e-18 for values in [0, 1).
#define LGD_FIX_BITS 56

__device__ __forceinline__ long long fx_div7_round(long long sum)
{
    // round(sum / 7) (no ties exist), via an unsigned offset so that the
    // division is one multiply-high: for n < 7 * 2^57 + 3 (and far beyond),
    // floor(n / 7) = floor(n * ceil(2^65 / 7) / 2^65) exactly (the error
    // term n * (3/7) / 2^65 stays below 1/7)
    const unsigned long long off = 7ull << LGD_FIX_BITS;
    const unsigned long long n = (unsigned long long)(sum + 3) + off;
    const unsigned long long q = __umul64hi(n, 0x4924924924924925ull) >> 1;
    return (long long)(q - (1ull << LGD_FIX_BITS));
}

__device__ __forceinline__ long long fx_div49_round(long long sum)
{
    // round(sum / 49) for |sum| < 49 * 2^56 (no ties: sum + 24 is never a
    // multiple of 49 plus a half).  n = sum + 24 + 49 * 2^56 < 98 * 2^56 + 25;
    // floor(n / 49) = floor(n * M / 2^69), M = ceil(2^69 / 49): with
    // M * 49 - 2^69 = 34, the error term n * 34 / (49 * 2^69) stays below
    // 1/49 for n < 2^69 / 34
    const unsigned long long off = 49ull << LGD_FIX_BITS;
    const unsigned long long n = (unsigned long long)(sum + 24) + off;
    const unsigned long long q = __umul64hi(n, 0xa72f05397829cbc2ull) >> 5;
    return (long long)(q - (1ull << LGD_FIX_BITS));
}

}  // namespace lgd

#endif
