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
// |value| < 2^scale_exp, so |k| < 2^57.  The averaging stencil maps
// [-S, S] into itself, so 7 * 2^57 < 2^60 bounds every neighbour sum, and
// 49 * 2^57 < 2^63 every exact two-step sum (the temporally blocked pass):
// nothing overflows.  57 fraction bits: each rounding adds at most
// 2^(scale_exp - 58), e.g. 3.5e-18 for values in [0, 1).
#define LGD_FIX_BITS 57

// The cell multiplies its neighbour sum by the double nearest 1/7,
// fl(1/7) = LGD_FIX_C7 * 2^-54 exactly (0x3FC2492492492492), which is
// 5.55e-17 (relatively) below 1/7.  The fixed-point steps multiply the exact
// sum by that same constant, so they follow the reference's arithmetic
// without the drift an exact division by 7 would accumulate against it
// (1.1e-12 relative after 20,000 steps).
//   single step: round(|sum| * fl(1/7)) = (hi64(|sum| * M7) + 1) >> 1 with
//     M7 = fl(1/7) * 2^65 = LGD_FIX_C7 << 11 (exact, below 2^63): the +1 in
//     the high word is the half unit, and the low word cannot carry into
//     the result because it is below 2^64 = half of 2^65;
//   two steps (exact sum of exact sums): round(|sum| * fl(1/7)^2) =
//     (hi64(|sum| * M49) + 16) >> 5 with M49 = fl(1/7)^2 * 2^69 rounded to
//     an integer (relative error below 2^-64: the product differs from the
//     exact one by less than 0.006 units for |sum| < 49 * 2^57).
// Rounding is to nearest, ties away from zero, and symmetric in the sign
// like an IEEE multiplication.
#define LGD_FIX_C7 2573485501354569ull
#define LGD_FIX_M7 0x4924924924924800ull
#define LGD_FIX_M49 0xa72f05397829c688ull

// 0 <= sum < 7 * 2^57
__device__ __forceinline__ long long fx_mul7_round_nonneg(long long sum)
{
    return (long long)((__umul64hi((unsigned long long)sum, LGD_FIX_M7) + 1ull) >> 1);
}

__device__ __forceinline__ long long fx_mul7_round(long long sum)
{
    const long long s = sum >> 63;                    // 0 or -1
    const long long q = fx_mul7_round_nonneg((sum ^ s) - s);
    return (q ^ s) - s;
}

// 0 <= sum < 49 * 2^57
__device__ __forceinline__ long long fx_mul49_round_nonneg(long long sum)
{
    return (long long)((__umul64hi((unsigned long long)sum, LGD_FIX_M49) + 16ull) >> 5);
}

__device__ __forceinline__ long long fx_mul49_round(long long sum)
{
    const long long s = sum >> 63;
    const long long q = fx_mul49_round_nonneg((sum ^ s) - s);
    return (q ^ s) - s;
}

}  // namespace lgd

#endif
