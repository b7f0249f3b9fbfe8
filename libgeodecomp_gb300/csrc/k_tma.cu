// Jacobi-7 with TMA-fed shared-memory planes (default whole-grid kernel on
// cube grids whose edge cell is zero - the Jacobi configuration).
//
// A CTA owns a 64 x 16 tile of every z plane of its z chunk.  One thread
// issues cp.async.bulk.tensor loads of the tile plus its one-cell rim
// ((64 + 2 pad) x 18 cells) into a ring of shared-memory slots, D = 3 planes
// ahead of the plane being computed; each slot has an mbarrier that the
// copy completes (expect_tx / complete_tx).  The tensor map's
// out-of-bounds fill (zeros) is the constant-zero edge cell, so no thread
// tests a boundary.  Threads compute from shared memory - two x-neighbouring
// cells per lane, four rows per warp, west/east/north/south/top/bottom from
// the staged planes - and store 16-byte pairs.  Traffic per time step: every
// cell read once through TMA (plus the rim, mostly L2 hits) and written
// once: 16 B per cell for 8-byte cells.
//
// The x coordinate of every copy is a multiple of 16 bytes (tile origin
// minus 16 / sizeof(T) cells), as TMA requires.  Waits on the mbarriers are
// bounded (about two seconds of clock cycles); a CTA that gives up sets the
// handle's error word, drains its copies and leaves, and the host reports
// LGD_ERR_TIMEOUT at the next synchronisation.
#include <cuda.h>

#include <mutex>

#include "lgd_internal.h"
#include "k_cells.cuh"

namespace lgd {
namespace tmak {

constexpr int TX = 64;         // cells per tile in x (32 lanes x 2)
constexpr int TY = 16;         // rows per tile (4 warps x 4 rows)
constexpr int ROWS = 4;
constexpr int THREADS = 128;
constexpr int D = 3;           // prefetch distance in planes
constexpr int S = D + 2;       // ring slots: planes q-1, q, q+1 in use, D ahead
constexpr long long WAIT_CYCLES = 4000000000LL;

template<typename T>
struct Box {
    static constexpr int XPAD = 16 / (int)sizeof(T);   // keeps the copy's x at 16 bytes
    static constexpr int W = TX + 2 * XPAD;
    static constexpr int H = TY + 2;
    static constexpr int BYTES = W * H * (int)sizeof(T);
    static constexpr int SLOT = (BYTES + 127) / 128 * 128;
};

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > WAIT_CYCLES) return false;
    }
    return true;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

template<typename T>
__device__ __forceinline__ void lds_pair(const unsigned char *p, T& a, T& b)
{
    if (sizeof(T) == 8) {
        const longlong2 v = *reinterpret_cast<const longlong2 *>(p);
        a = *reinterpret_cast<const T *>(&v.x);
        b = *reinterpret_cast<const T *>(&v.y);
    } else {
        const int2 v = *reinterpret_cast<const int2 *>(p);
        a = *reinterpret_cast<const T *>(&v.x);
        b = *reinterpret_cast<const T *>(&v.y);
    }
}

template<typename CELL>
__global__ void __launch_bounds__(THREADS)
jacobi7_tma_kernel(const __grid_constant__ CUtensorMap in_map, typename CELL::T *__restrict__ out, long pitch, int nx,
                   int ny, int nz, int zchunk, int *err)
{
    typedef typename CELL::T T;
    typedef Box<T> B;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[S];
    __shared__ int s_fail;
    __shared__ int s_issued;    // planes issued so far (0 .. nplanes)

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const int x0 = blockIdx.x * TX;
    const int y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, nz);
    if (z0 >= z1) return;                       // uniform across the CTA
    const int nplanes = (z1 - z0) + 2;          // plane q is z = z0 - 1 + q

    if (tid == 0) {
        for (int s = 0; s < S; ++s) mbar_init(smem_addr(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
        const int first = min(D, nplanes - 1);
        for (int q = 0; q <= first; ++q) {
            const uint32_t bar = smem_addr(&bars[q % S]);
            mbar_expect_tx(bar, B::BYTES);
            tma_load_3d(smem_addr(smem + (q % S) * B::SLOT), &in_map, x0 - B::XPAD, y0 - 1, z0 - 1 + q, bar);
        }
        s_issued = first + 1;
    }
    __syncthreads();

    int waited = -1;    // highest plane this thread has waited for
    for (int q = 0; q < 2; ++q) {
        if (!mbar_wait_bounded(smem_addr(&bars[q % S]), (q / S) & 1)) s_fail = 1;
        waited = q;
    }

    const int lx = 2 * lane;
    const int gx = x0 + lx;
    const int rw = warp * ROWS;
    const long plane = pitch * ny;

    for (int z = z0; z < z1; ++z) {
        const int q = z - z0 + 1;               // centre plane
        __syncthreads();                        // plane q - 2's slot is free again
        if (s_fail) break;                      // uniform: read after the barrier
        if (tid == 0 && q + D < nplanes) {
            const int qn = q + D;
            const uint32_t bar = smem_addr(&bars[qn % S]);
            mbar_expect_tx(bar, B::BYTES);
            tma_load_3d(smem_addr(smem + (qn % S) * B::SLOT), &in_map, x0 - B::XPAD, y0 - 1, z0 - 1 + qn, bar);
            s_issued = qn + 1;
        }
        if (!mbar_wait_bounded(smem_addr(&bars[(q + 1) % S]), ((q + 1) / S) & 1)) {
            s_fail = 1;
            continue;
        }
        waited = q + 1;

        const unsigned char *pb = smem + ((q - 1) % S) * B::SLOT;
        const unsigned char *pc = smem + (q % S) * B::SLOT;
        const unsigned char *pt = smem + ((q + 1) % S) * B::SLOT;
        // element (by, bx) of a slot at (by * W + bx) * sizeof(T); tile
        // cell (ly, lx) at by = ly + 1, bx = lx + XPAD
        auto off = [&](int ly, int lxx) { return ((ly + 1) * B::W + lxx + B::XPAD) * (int)sizeof(T); };
        T c[ROWS + 2][2];
#pragma unroll
        for (int j = -1; j <= ROWS; ++j) lds_pair<T>(pc + off(rw + j, lx), c[j + 1][0], c[j + 1][1]);
        T* orow = out + (long)z * plane + (long)(y0 + rw) * pitch + gx;
#pragma unroll
        for (int j = 0; j < ROWS; ++j) {
            const int ly = rw + j;
            T ta, tb, ba, bb;
            lds_pair<T>(pt + off(ly, lx), ta, tb);
            lds_pair<T>(pb + off(ly, lx), ba, bb);
            const T w0 = *reinterpret_cast<const T *>(pc + off(ly, lx - 1));
            const T e1 = *reinterpret_cast<const T *>(pc + off(ly, lx + 2));
            const T o0 = CELL::apply(c[j + 1][0], c[j][0], c[j + 2][0], c[j + 1][1], w0, ta, ba);
            const T o1 = CELL::apply(c[j + 1][1], c[j][1], c[j + 2][1], e1, c[j + 1][0], tb, bb);
            const int gy = y0 + ly;
            if (gy < ny) {
                T *o = orow + (long)j * pitch;
                if (gx + 1 < nx) {
                    if (sizeof(T) == 8) {
                        longlong2 v;
                        v.x = *reinterpret_cast<const long long *>(&o0);
                        v.y = *reinterpret_cast<const long long *>(&o1);
                        *reinterpret_cast<longlong2 *>(o) = v;
                    } else {
                        int2 v;
                        v.x = *reinterpret_cast<const int *>(&o0);
                        v.y = *reinterpret_cast<const int *>(&o1);
                        *reinterpret_cast<int2 *>(o) = v;
                    }
                } else if (gx < nx) {
                    o[0] = o0;
                }
            }
        }
    }

    __syncthreads();            // every thread has left the loop: s_fail and s_issued are final
    if (s_fail) {
        // report, then wait (bounded) for every copy still in flight before
        // the shared memory is released
        if (tid == 0) atomicExch(err, 1);
        for (int q = waited + 1; q < s_issued; ++q) {
            if (!mbar_wait_bounded(smem_addr(&bars[q % S]), (q / S) & 1)) break;
        }
    }
}

// -------------------------------------------------------------- host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess) {
            fn = reinterpret_cast<EncodeTiledFn>(p);
        } else {
            cudaGetLastError();
        }
    });
    return fn;
}

template<typename T>
static void encode(CUtensorMap *map, void *base, const Grid& g, CUtensorMapDataType dt)
{
    EncodeTiledFn fn = encode_fn();
    LGD_REQUIRE(fn != nullptr, LGD_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[3] = {(cuuint64_t)g.desc.nx, (cuuint64_t)g.desc.ny, (cuuint64_t)g.desc.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)g.pitch_bytes[0], (cuuint64_t)g.pitch_bytes[0] * g.desc.ny};
    const cuuint32_t box[3] = {(cuuint32_t)Box<T>::W, (cuuint32_t)Box<T>::H, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, dt, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    LGD_REQUIRE(r == CUDA_SUCCESS, LGD_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

}  // namespace tmak

long long fix_edge(const Grid& g);

// The TMA kernel serves Jacobi cells on cube grids whose edge cell is zero
// (the tensor map's zero fill is the edge value there).
bool tma_applicable(const Grid& g)
{
    if (g.desc.periodic != 0) return false;
    switch (g.desc.cell) {
    case LGD_CELL_JACOBI7_F64:
    case LGD_CELL_JACOBI7_F32:
        return g.desc.edge[0] == 0.0;
    case LGD_CELL_JACOBI7_F64_FIX:
        return fix_edge(g) == 0;
    default:
        return false;
    }
}

template<typename CELL>
static void launch_tma_typed(Grid& g, CUtensorMapDataType dt)
{
    typedef typename CELL::T T;
    const int src = g.cur;
    if (!g.tmap_ready[src] || g.tmap_base[src] != g.m[0].buf[src]) {
        tmak::encode<T>(reinterpret_cast<CUtensorMap *>(g.tmap[src]), g.m[0].buf[src], g, dt);
        g.tmap_ready[src] = true;
        g.tmap_base[src] = g.m[0].buf[src];
    }
    const int smem = tmak::S * tmak::Box<T>::SLOT;
    static bool configured = false;
    if (!configured) {
        LGD_CHECK_CUDA(cudaFuncSetAttribute(tmak::jacobi7_tma_kernel<CELL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            smem));
        configured = true;
    }
    const int bx = (g.desc.nx + tmak::TX - 1) / tmak::TX;
    const int by = (g.desc.ny + tmak::TY - 1) / tmak::TY;
    const long long xy = (long long)bx * by;
    // about four waves of four resident CTAs per SM
    int zsplit = (int)((152LL * 16 + xy - 1) / xy);
    zsplit = std::max(1, std::min(zsplit, (g.desc.nz + 15) / 16));
    int zchunk = (g.desc.nz + zsplit - 1) / zsplit;
    zsplit = (g.desc.nz + zchunk - 1) / zchunk;
    const CUtensorMap *map = reinterpret_cast<const CUtensorMap *>(g.tmap[src]);
    tmak::jacobi7_tma_kernel<CELL><<<dim3(bx, by, zsplit), tmak::THREADS, smem, g.stream>>>(
        *map, (T *)g.m[0].buf[1 - src], (long)(g.pitch_bytes[0] / sizeof(T)), g.desc.nx, g.desc.ny, g.desc.nz, zchunk,
        g.d_err);
}

void launch_jacobi7_tma(Grid& g)
{
    switch (g.desc.cell) {
    case LGD_CELL_JACOBI7_F64:
        launch_tma_typed<Jacobi7F64>(g, CU_TENSOR_MAP_DATA_TYPE_FLOAT64);
        break;
    case LGD_CELL_JACOBI7_F32:
        launch_tma_typed<Jacobi7F32>(g, CU_TENSOR_MAP_DATA_TYPE_FLOAT32);
        break;
    case LGD_CELL_JACOBI7_F64_FIX:
        launch_tma_typed<Jacobi7Fix>(g, CU_TENSOR_MAP_DATA_TYPE_INT64);
        break;
    default:
        throw Error(LGD_ERR_UNSUPPORTED, "not a Jacobi cell");
    }
    check_launch("jacobi7 tma");
    ++g.launches;
    g.cur = 1 - g.cur;
}

}  // namespace lgd
