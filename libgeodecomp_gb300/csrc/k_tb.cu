// Jacobi-7 with temporal blocking: TB time steps per pass over memory.
// (The fixed-point cell's pass of two keeps exact neighbour sums at its
// first level and rounds once at the second; see Jacobi7FixTwoStep.)
//
// A CTA owns a box of 64 x BH cells of every z plane of its z chunk and
// marches in z.  One thread streams the box's input planes into a ring of
// shared-memory slots with cp.async.bulk.tensor (D planes ahead, an
// mbarrier per slot, zero fill outside the grid = the constant-zero edge
// cell).  Every lane owns two x-neighbouring cells of ROWS rows at every
// level t = 0 .. TB, and at iteration i (input plane i has landed) level t
// computes its plane i - t from level t - 1:
//   - the z neighbours and the centre come from the thread's own registers
//     (three planes of each level rotate through v[t][i % 3]),
//   - the x neighbours from the adjacent lanes by shuffle,
//   - the y neighbours from the thread's own rows, except the rows just
//     above and below its block, which come from the previous level's plane
//     in shared memory (the input ring for level 1; a two-slot ring per
//     intermediate level, written one iteration earlier).
// One __syncthreads per input plane orders all of it.  Intermediate levels
// hold the edge value (zero) outside the grid, so every cell sees exactly
// the neighbours a single-step update would: the result is bit-identical to
// TB single steps.  Level TB stores the inner tile (64 - 2 XP) x (BH - 2 TB)
// to global memory; the rim of the box is recomputed by the neighbouring
// CTAs.  Input planes are read once per pass (the rims mostly from L2), so
// HBM traffic per pass stays 2 x sizeof(cell) per cell for TB steps.
//
// Waits on the mbarriers are bounded; a CTA that gives up sets the handle's
// error word, waits (bounded) for its copies in flight and leaves.
#include <cuda.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <type_traits>

#include "lgd_internal.h"
#include "k_cells.cuh"
#include "k_tma.cuh"

namespace lgd {
namespace tbk {

using tmak::lds_pair;
using tmak::mbar_expect_tx;
using tmak::mbar_init;
using tmak::mbar_wait_bounded;
using tmak::smem_addr;
using tmak::st_pair;
using tmak::tma_load_3d;

constexpr int BW = 64;     // box width in cells: 32 lanes x 2

// TB steps per pass; WY warps, each owning ROWS rows of the box
template<typename T, int TB, int WY, int ROWS>
struct Geo {
    static constexpr int ALIGN = 16 / (int)sizeof(T);              // cells per 16 bytes
    static constexpr int XP = (TB + ALIGN - 1) / ALIGN * ALIGN;    // x halo; keeps every copy's x 16-byte aligned
    static constexpr int BH = ROWS * WY;
    static constexpr int OX = BW - 2 * XP;                         // output tile
    static constexpr int OY = BH - 2 * TB;
    static constexpr int THREADS = 32 * WY;
    static constexpr int PLANE = BW * BH * (int)sizeof(T);         // one staged plane (a multiple of 128 bytes)
    static constexpr int D = 2;                                    // input planes in flight ahead
    static constexpr int S = D + 2;                                // input ring: planes i - 1, i, and D ahead
    static constexpr int SMEM = (S + 2 * (TB - 1)) * PLANE;
    static_assert(OX > 0 && OY > 0, "box too small for the blocking depth");
    static_assert((OX * (int)sizeof(T)) % 16 == 0, "tile origins must stay 16-byte aligned");
};

// The rule a level applies: the cell's own rule at every level, except for
// the two-step fixed-point cell, whose first level keeps exact sums and
// whose last level rounds once
template<typename CELL>
struct TBOps {
    typedef typename CELL::T T;
    // boxes inside the grid skip the intermediate level's edge masks (a
    // separate code path: it pays for the fixed-point cell, 495 against 483
    // GLUPS at 512^3, and costs the FP32 cell, 1079 against 1122)
    static constexpr bool INTERIOR_PATH = false;
    static __device__ __forceinline__ T level(bool last, T c, T n, T s, T e, T w, T t, T b)
    {
        return CELL::apply(c, n, s, e, w, t, b);
    }
    // the lane's two x-neighbouring cells: (c0, n0, ...) and (c1, n1, ...)
    static __device__ __forceinline__ void pair(bool last, T c0, T c1, T n0, T n1, T s0, T s1, T e0, T e1, T w0, T w1,
                                                T t0, T t1, T b0, T b1, T& r0, T& r1)
    {
        r0 = level(last, c0, n0, s0, e0, w0, t0, b0);
        r1 = level(last, c1, n1, s1, e1, w1, t1, b1);
    }
};

// FP32 Jacobi-7 on both cells at once in packed FP32 arithmetic: the same
// additions in the same order as Jacobi7F32::apply, each rounded to nearest,
// so the results are bit-identical to the single-step kernels'.
template<>
struct TBOps<Jacobi7F32> {
    typedef float T;
    static constexpr bool INTERIOR_PATH = false;
    static __device__ __forceinline__ void pair(bool, T c0, T c1, T n0, T n1, T s0, T s1, T e0, T e1, T w0, T w1,
                                                T t0, T t1, T b0, T b1, T& r0, T& r1)
    {
        float2 a = __fadd2_rn(make_float2(c0, c1), make_float2(n0, n1));
        a = __fadd2_rn(a, make_float2(s0, s1));
        a = __fadd2_rn(a, make_float2(e0, e1));
        a = __fadd2_rn(a, make_float2(w0, w1));
        a = __fadd2_rn(a, make_float2(t0, t1));
        a = __fadd2_rn(a, make_float2(b0, b1));
        a = __fmul2_rn(a, make_float2(1.0f / 7.0f, 1.0f / 7.0f));
        r0 = a.x;
        r1 = a.y;
    }
};

template<bool NONNEG>
struct TBOps<Jacobi7FixTwoStepT<NONNEG> > {
    typedef long long T;
    typedef Jacobi7FixTwoStepT<NONNEG> C;
    static constexpr bool INTERIOR_PATH = true;
    static __device__ __forceinline__ T level(bool last, T c, T n, T s, T e, T w, T t, T b)
    {
        return last ? C::last(c, n, s, e, w, t, b) : C::inner(c, n, s, e, w, t, b);
    }
    static __device__ __forceinline__ void pair(bool last, T c0, T c1, T n0, T n1, T s0, T s1, T e0, T e1, T w0, T w1,
                                                T t0, T t1, T b0, T b1, T& r0, T& r1)
    {
        r0 = level(last, c0, n0, s0, e0, w0, t0, b0);
        r1 = level(last, c1, n1, s1, e1, w1, t1, b1);
    }
};

template<typename CELL, int TB, int WY, int ROWS>
__global__ void __launch_bounds__(32 * WY)
jacobi7_tb_kernel(const __grid_constant__ CUtensorMap in_map, typename CELL::T *__restrict__ out, long pitch, int nx,
                  int ny, int nz, int zchunk, int *err)
{
    typedef typename CELL::T T;
    typedef Geo<T, TB, WY, ROWS> G;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[G::S];
    __shared__ int s_fail;
    __shared__ int s_issued;    // input planes issued so far

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const int x0 = blockIdx.x * G::OX;
    const int y0 = blockIdx.y * G::OY;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, nz);
    if (z0 >= z1) return;                       // uniform across the CTA
    const int nq = (z1 - z0) + 2 * TB;          // input plane q is z = z0 - TB + q
    const int bx0 = x0 - G::XP;                 // grid coordinates of box cell (0, 0)
    const int by0 = y0 - TB;
    unsigned char *const lvl = smem + G::S * G::PLANE;   // level t's slot s: lvl + ((t - 1) * 2 + s) * PLANE

    if (tid == 0) {
        for (int s = 0; s < G::S; ++s) mbar_init(smem_addr(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
        const int first = min(G::D, nq);
        for (int q = 0; q < first; ++q) {
            const uint32_t bar = smem_addr(&bars[q % G::S]);
            mbar_expect_tx(bar, G::PLANE);
            tma_load_3d(smem_addr(smem + (q % G::S) * G::PLANE), &in_map, bx0, by0, z0 - TB + q, bar);
        }
        s_issued = first;
    }
    __syncthreads();

    const int r0 = warp * ROWS;                 // the thread's first box row
    const int cx = 2 * lane;                    // box x of its first cell
    const int gx = bx0 + cx;
    const bool xin0 = gx >= 0 && gx < nx;
    const bool xin1 = gx + 1 >= 0 && gx + 1 < nx;
    unsigned ymask = 0;
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        const int gy = by0 + r0 + r;
        if (gy >= 0 && gy < ny) ymask |= 1u << r;
    }
    const int rn = max(r0 - 1, 0);              // rim rows, clamped to the box (the clamped
    const int rs = min(r0 + ROWS, G::BH - 1);   // values only reach cells outside the tile)
    const bool xout = cx >= G::XP && cx < G::XP + G::OX && gx < nx;
    const bool box_in =
        TBOps<CELL>::INTERIOR_PATH && bx0 >= 0 && bx0 + BW <= nx && by0 >= 0 && by0 + G::BH <= ny;
    const long plane_elems = pitch * ny;

    T v[TB][3][ROWS][2];                        // level t's planes, rotating by i % 3
    int waited = -1;                            // highest input plane this thread has waited for

    auto iteration = [&](auto phase, int i) {
        constexpr int P = decltype(phase)::value;          // i % 3
        constexpr int PC = (P + 2) % 3;                    // plane i - 1 of a level
        constexpr int PB = (P + 1) % 3;                    // plane i - 2
        const uint32_t bar = smem_addr(&bars[i % G::S]);
        // the whole warp goes on or stops together (the compute shuffles)
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(bar, (uint32_t)((i / G::S) & 1)))) {
            s_fail = 1;
            return;
        }
        waited = i;
        const unsigned char *sl = smem + (i % G::S) * G::PLANE;
        const unsigned char *slp = smem + ((i + G::S - 1) % G::S) * G::PLANE;
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            lds_pair<T>(sl + ((r0 + r) * BW + cx) * (int)sizeof(T), v[0][P][r][0], v[0][P][r][1]);
        }
#pragma unroll
        for (int t = 1; t <= TB; ++t) {
            if (i < 2 * t) break;                           // uniform: level t has no plane yet
            const unsigned char *src = (t == 1) ? slp : lvl + ((t - 2) * 2 + ((i - 1) & 1)) * G::PLANE;
            T nr0, nr1, sr0, sr1;
            lds_pair<T>(src + (rn * BW + cx) * (int)sizeof(T), nr0, nr1);
            lds_pair<T>(src + (rs * BW + cx) * (int)sizeof(T), sr0, sr1);
            T res[ROWS][2];
#pragma unroll
            for (int r = 0; r < ROWS; ++r) {
                const T c0 = v[t - 1][PC][r][0];
                const T c1 = v[t - 1][PC][r][1];
                const T n0 = (r == 0) ? nr0 : v[t - 1][PC][r - 1][0];
                const T n1 = (r == 0) ? nr1 : v[t - 1][PC][r - 1][1];
                const T s0 = (r == ROWS - 1) ? sr0 : v[t - 1][PC][r + 1][0];
                const T s1 = (r == ROWS - 1) ? sr1 : v[t - 1][PC][r + 1][1];
                const T w0 = __shfl_up_sync(0xffffffffu, c1, 1);
                const T e1 = __shfl_down_sync(0xffffffffu, c0, 1);
                TBOps<CELL>::pair(t == TB, c0, c1, n0, n1, s0, s1, c1, e1, w0, c0, v[t - 1][P][r][0],
                                  v[t - 1][P][r][1], v[t - 1][PB][r][0], v[t - 1][PB][r][1], res[r][0], res[r][1]);
            }
            if (t < TB) {
                // outside the grid an intermediate level keeps the edge
                // value; a plane of a box inside the grid needs no masks
                // (the branch is uniform across the CTA; cells whose
                // INTERIOR_PATH is off always take the masked one)
                const int gz = z0 - TB + i - t;
                const bool zin = gz >= 0 && gz < nz;
                unsigned char *dst = lvl + ((t - 1) * 2 + (i & 1)) * G::PLANE;
                if (box_in && zin) {
#pragma unroll
                    for (int r = 0; r < ROWS; ++r) {
                        v[t][P][r][0] = res[r][0];
                        v[t][P][r][1] = res[r][1];
                        st_pair<T>(dst + ((r0 + r) * BW + cx) * (int)sizeof(T), res[r][0], res[r][1]);
                    }
                } else {
#pragma unroll
                    for (int r = 0; r < ROWS; ++r) {
                        const bool yin = zin && ((ymask >> r) & 1u);
                        v[t][P][r][0] = (yin && xin0) ? res[r][0] : T(0);
                        v[t][P][r][1] = (yin && xin1) ? res[r][1] : T(0);
                        st_pair<T>(dst + ((r0 + r) * BW + cx) * (int)sizeof(T), v[t][P][r][0], v[t][P][r][1]);
                    }
                }
            } else if (xout) {
                const int gz = z0 - 2 * TB + i;                 // in [z0, z1): level TB's plane
                T *orow = out + (long)gz * plane_elems + gx;
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    const int ly = r0 + r;
                    const int gy = by0 + ly;
                    if (ly < TB || ly >= TB + G::OY || gy >= ny) continue;
                    T *o = orow + (long)gy * pitch;
                    if (gx + 1 < nx) {
                        st_pair<T>(o, res[r][0], res[r][1]);
                    } else {
                        o[0] = res[r][0];
                    }
                }
            }
        }
    };

    for (int i = 0; i < nq; i += 3) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int ii = i + k;
            if (ii >= nq) break;                            // uniform
            __syncthreads();                                // plane ii - 2's slots are free again
            if (s_fail) goto done;                          // uniform: read after the barrier
            if (tid == 0 && ii + G::D < nq) {
                const int qn = ii + G::D;
                const uint32_t bar = smem_addr(&bars[qn % G::S]);
                mbar_expect_tx(bar, G::PLANE);
                tma_load_3d(smem_addr(smem + (qn % G::S) * G::PLANE), &in_map, bx0, by0, z0 - TB + qn, bar);
                s_issued = qn + 1;
            }
            if (k == 0) iteration(std::integral_constant<int, 0>(), ii);
            else if (k == 1) iteration(std::integral_constant<int, 1>(), ii);
            else iteration(std::integral_constant<int, 2>(), ii);
        }
    }
done:
    __syncthreads();            // every thread has left the loop: s_fail and s_issued are final
    if (s_fail) {
        if (tid == 0) atomicExch(err, 1);
        for (int q = waited + 1; q < s_issued; ++q) {
            if (!mbar_wait_bounded(smem_addr(&bars[q % G::S]), (uint32_t)((q / G::S) & 1))) break;
        }
    }
}

}  // namespace tbk

// ------------------------------------------------------------ host side

long long fix_edge(const Grid& g);

static long long resident_ctas_tb(const void *fn, int threads, int smem)
{
    int dev = 0, sms = 0, per_sm = 0;
    LGD_CHECK_CUDA(cudaGetDevice(&dev));
    LGD_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    LGD_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
    return (long long)sms * std::max(1, per_sm);
}

// resident CTAs of a pass kernel on the device, set up once (the shared
// memory limit and the query also load the kernel, which CUDA otherwise
// does at its first launch)
template<typename CELL, int TB, int WY, int ROWS>
static long long tb_resident()
{
    typedef tbk::Geo<typename CELL::T, TB, WY, ROWS> G;
    static PerDevice<long long> setup;
    return setup.get([] {
        LGD_CHECK_CUDA(cudaFuncSetAttribute(tbk::jacobi7_tb_kernel<CELL, TB, WY, ROWS>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM));
        return resident_ctas_tb((const void *)tbk::jacobi7_tb_kernel<CELL, TB, WY, ROWS>, G::THREADS, G::SMEM);
    });
}

// Planes per CTA: minimise waves of resident CTAs times input planes per CTA
// (the chunk plus the 2 TB halo planes); chunks of at least 8 planes.
static int pick_zchunk_tb(long long xy, int nz, long long resident, int halo)
{
    int best_chunk = nz;
    double best = 1e300;
    const int max_split = std::max(1, nz / 8);
    for (int split = 1; split <= max_split; ++split) {
        const int chunk = (nz + split - 1) / split;
        const int s = (nz + chunk - 1) / chunk;
        const long long waves = (xy * s + resident - 1) / resident;
        const double t = (double)waves * (chunk + halo);
        if (t < best * 0.999) {
            best = t;
            best_chunk = chunk;
        }
    }
    return best_chunk;
}

template<typename CELL, int TB, int WY, int ROWS>
static void launch_tb_typed(Grid& g, int dtype)
{
    typedef typename CELL::T T;
    typedef tbk::Geo<T, TB, WY, ROWS> G;
    const int src = g.cur;
    void *base = g.m[0].buf[src];
    if (!g.tbmap_ready[src] || g.tbmap_base[src] != base || g.tbmap_rows[src] != G::BH) {
        const uint64_t dims[3] = {(uint64_t)g.desc.nx, (uint64_t)g.desc.ny, (uint64_t)g.desc.nz};
        const uint64_t strides[2] = {(uint64_t)g.pitch_bytes[0], (uint64_t)g.pitch_bytes[0] * g.desc.ny};
        const uint32_t box[3] = {(uint32_t)tbk::BW, (uint32_t)G::BH, 1};
        encode_tensor_map(g.tbmap[src], dtype, 3, base, dims, strides, box);
        g.tbmap_ready[src] = true;
        g.tbmap_base[src] = base;
        g.tbmap_rows[src] = G::BH;
    }
    const long long resident = tb_resident<CELL, TB, WY, ROWS>();
    const int bx = (g.desc.nx + G::OX - 1) / G::OX;
    const int by = (g.desc.ny + G::OY - 1) / G::OY;
    const int zchunk = pick_zchunk_tb((long long)bx * by, g.desc.nz, resident, 2 * TB);
    const int zsplit = (g.desc.nz + zchunk - 1) / zchunk;
    const CUtensorMap *map = reinterpret_cast<const CUtensorMap *>(g.tbmap[src]);
    tbk::jacobi7_tb_kernel<CELL, TB, WY, ROWS><<<dim3(bx, by, zsplit), G::THREADS, G::SMEM, g.stream>>>(
        *map, (T *)g.m[0].buf[1 - src], (long)(g.pitch_bytes[0] / sizeof(T)), g.desc.nx, g.desc.ny, g.desc.nz, zchunk,
        g.d_err);
}

// Temporal blocking serves what the single-step TMA kernel serves (Jacobi
// cells on cube grids with a zero edge cell) in 3D, for the integer
// (fixed-point) and FP32 cells; the IEEE FP64 cell is bound by the FP64 rate,
// not by memory, and keeps one step per pass.
bool tb_applicable(const Grid& g)
{
    if (g.desc.dim != 3 || g.desc.periodic != 0) return false;
    switch (g.desc.cell) {
    case LGD_CELL_JACOBI7_F32:
        return g.desc.edge[0] == 0.0;
    case LGD_CELL_JACOBI7_F64_FIX:
        return fix_edge(g) == 0;
    default:
        return false;
    }
}

// Default depth per cell, measured at 512^3 on GB300: FP32 (packed pairs)
// 754 GLUPS at depth 1, 932 at 2, 1100 at 3 (16x4), 1026 at 4; fixed point
// 403 at depth 1 (95% of HBM
// bandwidth), 482 at depth 2 with exact two-step sums (a pass of two
// single-rounding steps took as long as two HBM-bound single steps: the
// per-step division by 7 costs a 64-bit multiply-high).
int tb_default_depth(const Grid& g)
{
    return g.desc.cell == LGD_CELL_JACOBI7_F32 ? 3 : 2;
}

// One pass of depth steps with box shape `shape` (0 = the fastest measured
// on GB300 for the cell and depth; 1, 2 = alternatives; warps x rows per
// warp; a shape that does not exist for a depth runs shape 0):
//   fixed point  depth 2 (exact two-step sums, one rounding): 16x4, 8x4, 16x2
//   FP32         depth 2: 8x4, 16x4, 16x2     depth 3: 16x4, 8x4, 16x2
//                depth 4: 16x4, 8x4, 16x2
// every pass kernel set up once, on the first pass of any grid
static void prepare_tb_kernels()
{
    static PerDevice<bool> setup;
    setup.get([] {
        (void)tb_resident<Jacobi7FixTwoStep, 2, 16, 4>();
        (void)tb_resident<Jacobi7FixTwoStep, 2, 8, 4>();
        (void)tb_resident<Jacobi7FixTwoStep, 2, 16, 2>();
        (void)tb_resident<Jacobi7FixTwoStepNonNeg, 2, 16, 4>();
        (void)tb_resident<Jacobi7FixTwoStepNonNeg, 2, 8, 4>();
        (void)tb_resident<Jacobi7FixTwoStepNonNeg, 2, 16, 2>();
        (void)tb_resident<Jacobi7F32, 2, 8, 4>();
        (void)tb_resident<Jacobi7F32, 2, 16, 4>();
        (void)tb_resident<Jacobi7F32, 2, 16, 2>();
        (void)tb_resident<Jacobi7F32, 3, 16, 4>();
        (void)tb_resident<Jacobi7F32, 3, 8, 4>();
        (void)tb_resident<Jacobi7F32, 3, 16, 2>();
        (void)tb_resident<Jacobi7F32, 4, 16, 4>();
        (void)tb_resident<Jacobi7F32, 4, 8, 4>();
        (void)tb_resident<Jacobi7F32, 4, 16, 2>();
        return true;
    });
}

void launch_jacobi7_tb(Grid& g, int depth, int shape)
{
    prepare_tb_kernels();
    const int i64 = CU_TENSOR_MAP_DATA_TYPE_INT64;
    const int f32 = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    if (g.desc.cell == LGD_CELL_JACOBI7_F64_FIX) {
        LGD_REQUIRE(depth == 2, LGD_ERR_INVALID, "the fixed-point cell fuses two steps per pass");
        // grids without negative values skip the sign handling (same results)
        if (g.fix_nonneg) {
            switch (shape) {
            case 1: launch_tb_typed<Jacobi7FixTwoStepNonNeg, 2, 8, 4>(g, i64); break;
            case 2: launch_tb_typed<Jacobi7FixTwoStepNonNeg, 2, 16, 2>(g, i64); break;
            default: launch_tb_typed<Jacobi7FixTwoStepNonNeg, 2, 16, 4>(g, i64); break;
            }
        } else {
            switch (shape) {
            case 1: launch_tb_typed<Jacobi7FixTwoStep, 2, 8, 4>(g, i64); break;
            case 2: launch_tb_typed<Jacobi7FixTwoStep, 2, 16, 2>(g, i64); break;
            default: launch_tb_typed<Jacobi7FixTwoStep, 2, 16, 4>(g, i64); break;
            }
        }
    } else if (g.desc.cell == LGD_CELL_JACOBI7_F32) {
        switch (depth * 10 + shape) {
        case 21: launch_tb_typed<Jacobi7F32, 2, 16, 4>(g, f32); break;
        case 22: launch_tb_typed<Jacobi7F32, 2, 16, 2>(g, f32); break;
        case 31: launch_tb_typed<Jacobi7F32, 3, 8, 4>(g, f32); break;
        case 32: launch_tb_typed<Jacobi7F32, 3, 16, 2>(g, f32); break;
        case 41: launch_tb_typed<Jacobi7F32, 4, 8, 4>(g, f32); break;
        case 42: launch_tb_typed<Jacobi7F32, 4, 16, 2>(g, f32); break;
        default:
            switch (depth) {
            case 2: launch_tb_typed<Jacobi7F32, 2, 8, 4>(g, f32); break;
            case 3: launch_tb_typed<Jacobi7F32, 3, 16, 4>(g, f32); break;
            case 4: launch_tb_typed<Jacobi7F32, 4, 16, 4>(g, f32); break;
            default: throw Error(LGD_ERR_INVALID, "temporal blocking depth out of range");
            }
        }
    } else {
        throw Error(LGD_ERR_UNSUPPORTED, "temporal blocking serves the fixed-point and FP32 Jacobi cells");
    }
    check_launch("jacobi7 temporal blocking");
    ++g.launches;
    g.cur = 1 - g.cur;
}

// Deepest Jacobi pass of a cell: the fixed-point cell's exact two-step sums
// stay below 2^63 (49 * 2^57), deeper fusion would need fewer fraction bits;
// the FP32 kernel is instantiated up to 4.
int tb_max_depth(const Grid& g)
{
    return g.desc.cell == LGD_CELL_JACOBI7_F64_FIX ? 2 : 4;
}

}  // namespace lgd
