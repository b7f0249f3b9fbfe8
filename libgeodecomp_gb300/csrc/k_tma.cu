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
#include <type_traits>

#include "lgd_internal.h"
#include "k_cells.cuh"
#include "k_tma.cuh"

namespace lgd {
namespace tmak {

constexpr int TX = 64;         // cells per tile in x (32 lanes x 2)
constexpr int TY = 16;         // rows per tile (4 warps x 4 rows)
constexpr int ROWS = 4;
constexpr int THREADS = 128;
constexpr int D = 3;           // prefetch distance in planes
constexpr int S = D + 2;       // ring slots: planes q-1, q, q+1 in use, D ahead
// the var-coef kernel's ring (two fields per slot): prefetch distance and
// slots, and whether FP32 pairs update in packed FP32 arithmetic.  Four
// slots of 13.6 KB (FP32) leave room for four CTAs per SM; at 256^3 FP32
// distance 2 measured 386 GLUPS against 368 for 3 (three CTAs per SM) and
// 282 for 1, and the packed arithmetic 368 against 333 for scalar.  Carrying
// the lane's own cells of planes z - 1 and z in registers (two shared loads
// fewer per field and row, 87 registers) measured slower: 369.
constexpr int VC_D = 2;
constexpr int VC_S = VC_D + 2;
constexpr bool VC_PACKED = true;

template<typename T>
struct Box {
    static constexpr int XPAD = 16 / (int)sizeof(T);   // keeps the copy's x at 16 bytes
    static constexpr int W = TX + 2 * XPAD;
    static constexpr int H = TY + 2;
    static constexpr int BYTES = W * H * (int)sizeof(T);
    static constexpr int SLOT = (BYTES + 127) / 128 * 128;
};

// wait_cycles bounds every mbarrier wait; skip_plane >= 0 (tests of the
// timeout path only, lgd_gpu_test_bounded_waits) makes CTA (0, 0, 0) leave
// that plane's copy unissued, so the wait for it runs out: the CTA sets the
// error word, drains the copies it did issue and returns
template<typename CELL>
__global__ void __launch_bounds__(THREADS)
jacobi7_tma_kernel(const __grid_constant__ CUtensorMap in_map, typename CELL::T *__restrict__ out, long pitch, int nx,
                   int ny, int nz, int zchunk, int *err, long long wait_cycles, int skip_plane)
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

    const int skip = (blockIdx.x | blockIdx.y | blockIdx.z) == 0 ? skip_plane : -1;
    if (tid == 0) {
        for (int s = 0; s < S; ++s) mbar_init(smem_addr(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
        const int first = min(D, nplanes - 1);
        for (int q = 0; q <= first; ++q) {
            if (q == skip) continue;
            const uint32_t bar = smem_addr(&bars[q % S]);
            mbar_expect_tx(bar, B::BYTES);
            tma_load_3d(smem_addr(smem + (q % S) * B::SLOT), &in_map, x0 - B::XPAD, y0 - 1, z0 - 1 + q, bar);
        }
        s_issued = first + 1;
    }
    __syncthreads();

    int waited = -1;    // highest plane this thread has waited for
    for (int q = 0; q < 2; ++q) {
        if (!mbar_wait_bounded(smem_addr(&bars[q % S]), (q / S) & 1, wait_cycles)) s_fail = 1;
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
            if (qn != skip) {
                const uint32_t bar = smem_addr(&bars[qn % S]);
                mbar_expect_tx(bar, B::BYTES);
                tma_load_3d(smem_addr(smem + (qn % S) * B::SLOT), &in_map, x0 - B::XPAD, y0 - 1, z0 - 1 + qn, bar);
            }
            s_issued = qn + 1;
        }
        if (!mbar_wait_bounded(smem_addr(&bars[(q + 1) % S]), ((q + 1) / S) & 1, wait_cycles)) {
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
            if (q == skip) continue;            // never issued
            if (!mbar_wait_bounded(smem_addr(&bars[q % S]), (q / S) & 1, wait_cycles)) break;
        }
    }
}

// Variable-coefficient diffusion with the same plane ring, carrying u and k
// and supporting wrapping axes.  Per plane and field the CTA copies the
// main box ((64 + 2 pad) x 18 cells, out-of-bounds cells zero) and, where
// an axis wraps and the tile touches the domain's edge, the wrapped
// neighbours into separate areas of the slot: the row y = ny - 1 (north of
// y = 0), the row y = 0 (south of y = ny - 1), a 16-byte column ending at
// x = nx - 1 (west of x = 0) and one starting at x = 0 (east of x = nx - 1).
// Wrapped z planes come from the plane index modulo nz.  Rows and columns
// are picked warp-uniformly (per row) or per lane when the compute reads
// its neighbours.  Traffic: u and k read once, u written once (12 B per
// cell for FP32).
namespace vc {

template<typename T>
struct Lay {
    typedef Box<T> B;
    static constexpr int MAIN = (B::W * B::H * (int)sizeof(T) + 127) / 128 * 128;
    static constexpr int ROW = (B::W * (int)sizeof(T) + 127) / 128 * 128;
    static constexpr int COL = (B::XPAD * B::H * (int)sizeof(T) + 127) / 128 * 128;
    // field block: main, north row, south row, west column, east column
    static constexpr int ROWN = MAIN;
    static constexpr int ROWS_ = MAIN + ROW;
    static constexpr int COLW = MAIN + 2 * ROW;
    static constexpr int COLE = MAIN + 2 * ROW + COL;
    static constexpr int FIELD = MAIN + 2 * ROW + 2 * COL;
    static constexpr int SLOT = 2 * FIELD;
};

// tensor maps of one step: [field][main, row, col]
struct Maps {
    CUtensorMap m[2][3];
};

}  // namespace vc

template<typename R>
__global__ void __launch_bounds__(THREADS)
varcoef_tma_kernel(const __grid_constant__ vc::Maps maps, R *__restrict__ out, long pitch, int nx, int ny, int nz,
                   int periodic, int zchunk, int *err)
{
    typedef Box<R> B;
    typedef vc::Lay<R> Y;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[VC_S];
    __shared__ int s_fail;
    __shared__ int s_issued;

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const int x0 = blockIdx.x * TX;
    const int y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, nz);
    if (z0 >= z1) return;
    const int nplanes = (z1 - z0) + 2;
    const bool xw = (periodic & 1) != 0;
    const bool yw = (periodic & 2) != 0;
    const bool zw = (periodic & 4) != 0;
    // which wrapped areas this tile needs (uniform across the CTA)
    const bool need_n = yw && y0 == 0;
    const bool need_s = yw && y0 + TY >= ny;
    const bool need_w = xw && x0 == 0;
    const bool need_e = xw && x0 + TX >= nx;
    const uint32_t bytes = 2u * (uint32_t)(B::W * B::H * sizeof(R) + (need_n + need_s) * B::W * sizeof(R) +
                                           (need_w + need_e) * B::XPAD * B::H * sizeof(R));

    auto issue = [&](int q) {
        const uint32_t bar = smem_addr(&bars[q % VC_S]);
        int z = z0 - 1 + q;
        if (zw) z = (z + nz) % nz;
        mbar_expect_tx(bar, bytes);
        unsigned char *slot = smem + (q % VC_S) * Y::SLOT;
#pragma unroll
        for (int f = 0; f < 2; ++f) {
            unsigned char *fb = slot + f * Y::FIELD;
            tma_load_3d(smem_addr(fb), &maps.m[f][0], x0 - B::XPAD, y0 - 1, z, bar);
            if (need_n) tma_load_3d(smem_addr(fb + Y::ROWN), &maps.m[f][1], x0 - B::XPAD, ny - 1, z, bar);
            if (need_s) tma_load_3d(smem_addr(fb + Y::ROWS_), &maps.m[f][1], x0 - B::XPAD, 0, z, bar);
            if (need_w) tma_load_3d(smem_addr(fb + Y::COLW), &maps.m[f][2], nx - B::XPAD, y0 - 1, z, bar);
            if (need_e) tma_load_3d(smem_addr(fb + Y::COLE), &maps.m[f][2], 0, y0 - 1, z, bar);
        }
    };

    if (tid == 0) {
        for (int s = 0; s < VC_S; ++s) mbar_init(smem_addr(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
        const int first = min(VC_D, nplanes - 1);
        for (int q = 0; q <= first; ++q) issue(q);
        s_issued = first + 1;
    }
    __syncthreads();

    int waited = -1;
    for (int q = 0; q < 2; ++q) {
        if (!mbar_wait_bounded(smem_addr(&bars[q % VC_S]), (q / VC_S) & 1)) s_fail = 1;
        waited = q;
    }

    const int lx = 2 * lane;
    const int gx = x0 + lx;
    const int rw = warp * ROWS;
    const long plane = pitch * ny;
    // element offsets (bytes) inside a field block
    auto mo = [&](int ly, int lxx) { return ((ly + 1) * B::W + lxx + B::XPAD) * (int)sizeof(R); };
    auto ld = [&](const unsigned char *p) { return *reinterpret_cast<const R *>(p); };

    for (int z = z0; z < z1; ++z) {
        const int q = z - z0 + 1;
        __syncthreads();
        if (s_fail) break;
        if (tid == 0 && q + VC_D < nplanes) {
            issue(q + VC_D);
            s_issued = q + VC_D + 1;
        }
        if (!mbar_wait_bounded(smem_addr(&bars[(q + 1) % VC_S]), ((q + 1) / VC_S) & 1)) {
            s_fail = 1;
            continue;
        }
        waited = q + 1;

        const unsigned char *sb = smem + ((q - 1) % VC_S) * Y::SLOT;
        const unsigned char *sc = smem + (q % VC_S) * Y::SLOT;
        const unsigned char *st = smem + ((q + 1) % VC_S) * Y::SLOT;
        R *orow = out + (long)z * plane + (long)(y0 + rw) * pitch + gx;
#pragma unroll
        for (int j = 0; j < ROWS; ++j) {
            const int ly = rw + j;
            const int gy = y0 + ly;
            if (gy >= ny) break;                        // warp-uniform
            R c[2][2], nb[2][2], sb2[2][2], tp[2][2], bt[2][2], we[2], ea[2];
#pragma unroll
            for (int f = 0; f < 2; ++f) {
                const unsigned char *cf = sc + f * Y::FIELD;
                lds_pair<R>(cf + mo(ly, lx), c[f][0], c[f][1]);
                if (need_n && gy == 0) {
                    lds_pair<R>(cf + Y::ROWN + (lx + B::XPAD) * (int)sizeof(R), nb[f][0], nb[f][1]);
                } else {
                    lds_pair<R>(cf + mo(ly - 1, lx), nb[f][0], nb[f][1]);
                }
                if (need_s && gy == ny - 1) {
                    lds_pair<R>(cf + Y::ROWS_ + (lx + B::XPAD) * (int)sizeof(R), sb2[f][0], sb2[f][1]);
                } else {
                    lds_pair<R>(cf + mo(ly + 1, lx), sb2[f][0], sb2[f][1]);
                }
                lds_pair<R>(st + f * Y::FIELD + mo(ly, lx), tp[f][0], tp[f][1]);
                lds_pair<R>(sb + f * Y::FIELD + mo(ly, lx), bt[f][0], bt[f][1]);
                // west of the lane's first cell, east of its second (or of
                // the first when the second lies beyond nx)
                we[f] = (need_w && gx == 0) ? ld(cf + Y::COLW + ((ly + 1) * B::XPAD + B::XPAD - 1) * (int)sizeof(R))
                                            : ld(cf + mo(ly, lx - 1));
                const int ex = (gx + 1 < nx) ? gx + 2 : gx + 1;     // global x of the east neighbour
                ea[f] = (need_e && ex == nx) ? ld(cf + Y::COLE + (ly + 1) * B::XPAD * (int)sizeof(R))
                                             : ld(cf + mo(ly, ex - x0));
            }
            if (gx >= nx) continue;
            R *o = orow + (long)j * pitch;
            if (VC_PACKED && sizeof(R) == 4 && gx + 1 < nx) {
                // both cells in packed FP32 arithmetic
                auto p2 = [](R a, R b) { return make_float2((float)a, (float)b); };
                const float2 r2 = varcoef_pair_f32(
                    p2(c[0][0], c[0][1]), p2(c[1][0], c[1][1]), p2(we[0], c[0][0]), p2(we[1], c[1][0]),
                    p2(c[0][1], ea[0]), p2(c[1][1], ea[1]), p2(nb[0][0], nb[0][1]), p2(nb[1][0], nb[1][1]),
                    p2(sb2[0][0], sb2[0][1]), p2(sb2[1][0], sb2[1][1]), p2(bt[0][0], bt[0][1]), p2(bt[1][0], bt[1][1]),
                    p2(tp[0][0], tp[0][1]), p2(tp[1][0], tp[1][1]));
                *reinterpret_cast<float2 *>(o) = r2;
            } else if (gx + 1 < nx) {
                const R o0 = VarCoef<R>::apply(c[0][0], c[1][0], we[0], we[1], c[0][1], c[1][1], nb[0][0], nb[1][0],
                                               sb2[0][0], sb2[1][0], bt[0][0], bt[1][0], tp[0][0], tp[1][0]);
                const R o1 = VarCoef<R>::apply(c[0][1], c[1][1], c[0][0], c[1][0], ea[0], ea[1], nb[0][1], nb[1][1],
                                               sb2[0][1], sb2[1][1], bt[0][1], bt[1][1], tp[0][1], tp[1][1]);
                if (sizeof(R) == 8) {
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
            } else {
                o[0] = VarCoef<R>::apply(c[0][0], c[1][0], we[0], we[1], ea[0], ea[1], nb[0][0], nb[1][0], sb2[0][0],
                                         sb2[1][0], bt[0][0], bt[1][0], tp[0][0], tp[1][0]);
            }
        }
    }

    __syncthreads();
    if (s_fail) {
        if (tid == 0) atomicExch(err, 1);
        for (int q = waited + 1; q < s_issued; ++q) {
            if (!mbar_wait_bounded(smem_addr(&bars[q % VC_S]), (q / VC_S) & 1)) break;
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
static void encode(CUtensorMap *map, void *base, const Grid& g, CUtensorMapDataType dt, int member = 0,
                   int box_w = Box<T>::W, int box_h = Box<T>::H)
{
    EncodeTiledFn fn = encode_fn();
    LGD_REQUIRE(fn != nullptr, LGD_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[3] = {(cuuint64_t)g.desc.nx, (cuuint64_t)g.desc.ny, (cuuint64_t)g.desc.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)g.pitch_bytes[member], (cuuint64_t)g.pitch_bytes[member] * g.desc.ny};
    const cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, dt, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    LGD_REQUIRE(r == CUDA_SUCCESS, LGD_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

}  // namespace tmak

void encode_tensor_map(void *map, int dtype, int rank, void *base, const uint64_t *dims, const uint64_t *strides,
                       const uint32_t *box)
{
    tmak::EncodeTiledFn fn = tmak::encode_fn();
    LGD_REQUIRE(fn != nullptr, LGD_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    LGD_REQUIRE(rank >= 1 && rank <= 5, LGD_ERR_INVALID, "tensor map rank out of range");
    cuuint64_t d[5], s[4];
    cuuint32_t b[5], e[5];
    for (int i = 0; i < rank; ++i) {
        d[i] = dims[i];
        b[i] = box[i];
        e[i] = 1;
        if (i + 1 < rank) s[i] = strides[i];
    }
    CUresult r = fn(reinterpret_cast<CUtensorMap *>(map), (CUtensorMapDataType)dtype, (cuuint32_t)rank, base, d, s, b, e,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    LGD_REQUIRE(r == CUDA_SUCCESS, LGD_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

namespace tmak {

// Planes per CTA of a z-marching launch over xy tiles per plane: the split
// that minimises the modelled time, waves of resident CTAs times planes per
// CTA (including the two halo planes), with chunks of at least 8 planes.
// A partial last wave costs a whole wave: the kernels are bound by the
// copies each CTA keeps in flight, so fewer CTAs move fewer bytes.
static int pick_zchunk(long long xy, int nz, long long resident)
{
    int best_chunk = nz;
    double best = 1e300;
    const int max_split = std::max(1, nz / 8);
    for (int split = 1; split <= max_split; ++split) {
        const int chunk = (nz + split - 1) / split;
        const int s = (nz + chunk - 1) / chunk;
        const long long waves = (xy * s + resident - 1) / resident;
        const double t = (double)waves * (chunk + 2);
        if (t < best * 0.999) {
            best = t;
            best_chunk = chunk;
        }
    }
    return best_chunk;
}

// Planes per CTA for a kernel bound by its arithmetic pipe (the IEEE FP64
// cell: the FP64 pipe, not HBM): the split whose CTAs fill whole waves of
// resident CTAs best, modelled time = waves x planes per CTA, chunks of at
// least 8 planes.  A partial last wave leaves SMs idle while the others
// finish, which an arithmetic-bound kernel pays in full (512^3: 10 chunks
// of 52 planes make 4.2 waves, 19 chunks of 27 make 8.0).
static int pick_zchunk_compute(long long xy, int nz, long long resident)
{
    int best_chunk = nz;
    double best = 1e300;
    const int max_split = std::max(1, nz / 8);
    for (int split = 1; split <= max_split; ++split) {
        const int chunk = (nz + split - 1) / split;
        const int s = (nz + chunk - 1) / chunk;
        const long long waves = (xy * s + resident - 1) / resident;
        const double t = (double)waves * chunk;
        if (t < best * 0.999) {
            best = t;
            best_chunk = chunk;
        }
    }
    return best_chunk;
}

// resident CTAs of a kernel on the whole device
static long long resident_ctas(const void *fn, int threads, int smem)
{
    int dev = 0, sms = 0, per_sm = 0;
    LGD_CHECK_CUDA(cudaGetDevice(&dev));
    LGD_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    LGD_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
    return (long long)sms * std::max(1, per_sm);
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
    static PerDevice<long long> setup;
    const long long resident = setup.get([smem] {
        LGD_CHECK_CUDA(cudaFuncSetAttribute(tmak::jacobi7_tma_kernel<CELL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            smem));
        return tmak::resident_ctas((const void *)tmak::jacobi7_tma_kernel<CELL>, tmak::THREADS, smem);
    });
    const int bx = (g.desc.nx + tmak::TX - 1) / tmak::TX;
    const int by = (g.desc.ny + tmak::TY - 1) / tmak::TY;
    const long long xy = (long long)bx * by;
    int zchunk, zsplit;
    if (std::is_same<CELL, Jacobi7F64>::value) {
        // bound by the FP64 pipe: whole waves
        zchunk = tmak::pick_zchunk_compute(xy, g.desc.nz, resident);
    } else {
        // about 16 CTAs per SM over the launch (several waves of three
        // resident ones): at 94% of HBM bandwidth the kernel is bound by
        // DRAM, not by the copies a CTA has in flight, and short z chunks
        // keep the tail of the launch short (measured: 400 GLUPS at 512^3
        // against 387 with the wave-count model the var-coef kernel uses)
        zsplit = (int)((152LL * 16 + xy - 1) / xy);
        zsplit = std::max(1, std::min(zsplit, (g.desc.nz + 15) / 16));
        zchunk = (g.desc.nz + zsplit - 1) / zsplit;
    }
    zsplit = (g.desc.nz + zchunk - 1) / zchunk;
    const CUtensorMap *map = reinterpret_cast<const CUtensorMap *>(g.tmap[src]);
    tmak::jacobi7_tma_kernel<CELL><<<dim3(bx, by, zsplit), tmak::THREADS, smem, g.stream>>>(
        *map, (T *)g.m[0].buf[1 - src], (long)(g.pitch_bytes[0] / sizeof(T)), g.desc.nx, g.desc.ny, g.desc.nz, zchunk,
        g.d_err, g.test_wait_cycles > 0 ? g.test_wait_cycles : tmak::WAIT_CYCLES, g.test_skip_plane - 1);
}

// The var-coef TMA kernel: 3D grids whose non-wrapping axes have zero edge
// values for u and k, and - when x wraps - rows whose length is a multiple
// of 16 bytes (the west column's copy starts at x = nx - 16 / sizeof(T)).
bool varcoef_tma_applicable(const Grid& g)
{
    if (g.desc.dim != 3) return false;
    const int elem = (g.desc.cell == LGD_CELL_VARCOEF_F32) ? 4 : 8;
    if (g.desc.cell != LGD_CELL_VARCOEF_F32 && g.desc.cell != LGD_CELL_VARCOEF_F64) return false;
    if (g.desc.periodic != 7 && (g.desc.edge[0] != 0.0 || g.desc.edge[1] != 0.0)) return false;
    if ((g.desc.periodic & 1) && ((long long)g.desc.nx * elem) % 16 != 0) return false;
    return g.pitch_bytes[0] == g.pitch_bytes[1];
}

template<typename R>
static void launch_varcoef_tma_typed(Grid& g, CUtensorMapDataType dt)
{
    typedef tmak::Box<R> B;
    const int src = g.cur;
    void *ubuf = g.m[0].buf[src];
    void *kbuf = g.m[1].buf[0];
    tmak::vc::Maps *maps = reinterpret_cast<tmak::vc::Maps *>(g.vtmap[src]);
    if (!g.vtmap_ready[src] || g.vtmap_base[src][0] != ubuf || g.vtmap_base[src][1] != kbuf) {
        void *bases[2] = {ubuf, kbuf};
        for (int f = 0; f < 2; ++f) {
            tmak::encode<R>(&maps->m[f][0], bases[f], g, dt, f, B::W, B::H);
            tmak::encode<R>(&maps->m[f][1], bases[f], g, dt, f, B::W, 1);
            tmak::encode<R>(&maps->m[f][2], bases[f], g, dt, f, B::XPAD, B::H);
        }
        g.vtmap_ready[src] = true;
        g.vtmap_base[src][0] = ubuf;
        g.vtmap_base[src][1] = kbuf;
    }
    const int smem = tmak::VC_S * tmak::vc::Lay<R>::SLOT;
    static PerDevice<long long> setup;
    const long long resident = setup.get([smem] {
        LGD_CHECK_CUDA(cudaFuncSetAttribute(tmak::varcoef_tma_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        return tmak::resident_ctas((const void *)tmak::varcoef_tma_kernel<R>, tmak::THREADS, smem);
    });
    const int bx = (g.desc.nx + tmak::TX - 1) / tmak::TX;
    const int by = (g.desc.ny + tmak::TY - 1) / tmak::TY;
    const int zchunk = tmak::pick_zchunk((long long)bx * by, g.desc.nz, resident);
    const int zsplit = (g.desc.nz + zchunk - 1) / zchunk;
    tmak::varcoef_tma_kernel<R><<<dim3(bx, by, zsplit), tmak::THREADS, smem, g.stream>>>(
        *maps, (R *)g.m[0].buf[1 - src], (long)(g.pitch_bytes[0] / sizeof(R)), g.desc.nx, g.desc.ny, g.desc.nz,
        g.desc.periodic, zchunk, g.d_err);
}

void launch_varcoef_tma(Grid& g)
{
    if (g.desc.cell == LGD_CELL_VARCOEF_F32) {
        launch_varcoef_tma_typed<float>(g, CU_TENSOR_MAP_DATA_TYPE_FLOAT32);
    } else {
        launch_varcoef_tma_typed<double>(g, CU_TENSOR_MAP_DATA_TYPE_FLOAT64);
    }
    check_launch("varcoef tma");
    ++g.launches;
    g.cur = 1 - g.cur;
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
        // grids without negative values skip the sign handling (same results)
        if (g.fix_nonneg) {
            launch_tma_typed<Jacobi7FixNonNeg>(g, CU_TENSOR_MAP_DATA_TYPE_INT64);
        } else {
            launch_tma_typed<Jacobi7Fix>(g, CU_TENSOR_MAP_DATA_TYPE_INT64);
        }
        break;
    default:
        throw Error(LGD_ERR_UNSUPPORTED, "not a Jacobi cell");
    }
    check_launch("jacobi7 tma");
    ++g.launches;
    g.cur = 1 - g.cur;
}

}  // namespace lgd
