// Surrogate convolution C -> C (C = 24) on the fifth-generation tensor
// cores: tcgen05.mma with BF16 operands in shared memory and the FP32
// accumulator in tensor memory.
//
// Activations for this path are "ghosted": BF16 [batch][nz+2][ny+2][nx+2][32],
// the torus' wrapped neighbours stored in a one-voxel ghost layer (written
// by the producing layer's epilogue), channels 24..31 zero.  A CTA owns a
// 128 x 2 tile of output voxels of every plane of its z chunk and keeps:
//   - the layer's weights, 27 taps x 32 x 32 BF16 (54 KiB, one bulk copy),
//     as the MMA's B operand in the canonical K-major layout without
//     swizzle: element (tap, cin, cout) at ((tap * 4 + cin / 8) * 32 + cout)
//     * 16 B + cin % 8;
//   - a ring of five input planes, each 4 channel groups x 4 rows x 130
//     voxels x 8 channels, laid out [group][row][voxel][8 ch], i.e. voxels
//     16 B apart: the canonical K-major layout of the A operand (8-voxel core
//     matrices 128 B apart = SBO, channel groups one group block apart =
//     LBO).  A tap shifts the A start address by whole voxels (16 B) and
//     rows; no data moves.
// Warp-specialised pipeline, no CTA-wide barrier inside the plane loop:
//   - warps 9..12 (loaders) copy input planes into the ring with cp.async,
//     16 B per request, each warp instruction 32 consecutive voxels of one
//     channel group (the four groups of a voxel back to back, so the three
//     re-reads of a 64-byte voxel hit L1); two planes in flight, each
//     published to the MMA thread through the slot's "full" mbarrier (after
//     a generic-to-async proxy fence) before the loader waits for the next
//     free slot.  (A tensor-map copy would land the same
//     layout, but its 16-byte box rows run at about one row per 7.5 cycles
//     per SM, four times slower than the MMAs.)
//   - warp 0, one thread: per output plane i it waits for input planes
//     i .. i+2 and for the epilogue to have emptied TMEM accumulator buffer
//     i % 2, issues 2 rows x 27 taps x 2 K-steps of M=128 (voxels), N=32
//     (output channels), K=16 MMAs into that buffer and commits them to the
//     buffer's mbarrier and to the "empty" mbarrier of input plane i's slot
//     (plane i has no later reader);
//   - warps 1..8 (the epilogue): each owns one TMEM lane quarter (32 voxels)
//     and one output row; per plane it waits for the commit, reads its 32
//     accumulator columns (tcgen05.ld), hands the buffer back and then
//     applies bias, GELU, BF16 rounding and stores the voxel and its ghost
//     copies.
// Every wait is bounded and gives up early once another role has failed; a
// CTA that gives up sets the error word, lets its copies and MMAs finish and
// frees its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>

#include "lgd_internal.h"

namespace lgd {
namespace sur {

namespace tc {

constexpr int TXO = 128;                    // output voxels per row tile (MMA M)
constexpr int TYO = 2;                      // output rows per tile
constexpr int R = TYO + 2;                  // halo rows per plane
constexpr int HXV = TXO + 2;                // halo voxels per row
constexpr int CP = 32;                      // channels stored per voxel
constexpr int G = CP / 8;                   // 16-byte channel groups
constexpr int GROUP_BYTES = R * HXV * 16;   // 8320
constexpr int SLOT = G * GROUP_BYTES;       // 33280
constexpr int S = 5;                        // ring slots
constexpr int W_BYTES = 27 * G * CP * 16;   // 55296
constexpr int SMEM = 128 + W_BYTES + S * SLOT;
constexpr int EPI_WARPS = 8;                // epilogue warps: 4 lane quarters x 2 rows
constexpr int LOAD_WARPS = 4;               // cp.async loaders
constexpr int LOAD0 = 1 + EPI_WARPS;        // first loader warp
constexpr int THREADS = 32 * (1 + EPI_WARPS + LOAD_WARPS);
constexpr int TMEM_COLS = 128;              // 2 buffers x 2 rows x 32 columns
constexpr long long WAIT_CYCLES = 4000000000LL;

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both
// K-major, N = 32, M = 128
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(CP >> 3) << 17) | ((uint32_t)(TXO >> 4) << 24);

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, no swizzle: start, leading (K) and
// stride (M/N) byte offsets in 16-byte units, descriptor version 1
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
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

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    if (mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try(bar, parity)) {
        if (clock64() - t0 > WAIT_CYCLES) return false;
    }
    return true;
}

__device__ __forceinline__ void tma_4d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void bulk_copy(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t acc)
{
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(IDESC), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16(lo)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(hi)) << 16);
}

struct Params {
    int nx, ny, nz, batch, zchunk;
};

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// bounded wait that also gives up as soon as another role has failed
__device__ __forceinline__ bool mbar_wait_or_fail(uint32_t bar, uint32_t parity, volatile int *fail)
{
    if (mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try(bar, parity)) {
        if (*fail || clock64() - t0 > WAIT_CYCLES) return false;
    }
    return true;
}

__global__ void __launch_bounds__(THREADS, 1)
conv_tc_kernel(const __nv_bfloat16 *__restrict__ in, const __nv_bfloat16 *__restrict__ wpacked,
               const float *__restrict__ bias, __nv_bfloat16 *__restrict__ out, Params p, int *err)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar_w;
    __shared__ __align__(8) uint64_t bar_full[S];     // input plane in its slot (one arrive per loader warp)
    __shared__ __align__(8) uint64_t bar_empty[S];    // input slot no longer read (MMA commit)
    __shared__ __align__(8) uint64_t bar_mma[2];      // accumulator buffer written (MMA commit)
    __shared__ __align__(8) uint64_t bar_free[2];     // accumulator buffer read by the epilogue
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail;
    volatile int *fail = &s_fail;

    unsigned char *smem = smem_raw + ((128 - (saddr(smem_raw) & 127)) & 127);
    unsigned char *wsm = smem;
    unsigned char *ring = smem + W_BYTES;

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const int x0 = blockIdx.x * TXO;
    const int y0 = blockIdx.y * TYO;
    const int zsplit = (p.nz + p.zchunk - 1) / p.zchunk;
    const int b = blockIdx.z / zsplit;
    const int z0 = (blockIdx.z % zsplit) * p.zchunk;
    const int z1 = min(z0 + p.zchunk, p.nz);
    const int n = z1 - z0;                  // output planes; input planes q = 0 .. n+1
    const int zg0 = b * (p.nz + 2) + z0;    // ghosted z of input plane q = 0

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&s_tmem)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // MMA-thread state (thread 0 only)
    int waited = 0;         // input planes waited for
    int committed = 0;      // output planes whose MMAs were committed
    bool w_ready = false;
    if (tid == 0) {
        s_fail = 0;
        mbar_init(saddr(&bar_w), 1);
        for (int s = 0; s < S; ++s) {
            mbar_init(saddr(&bar_full[s]), LOAD_WARPS);
            mbar_init(saddr(&bar_empty[s]), 1);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(saddr(&bar_mma[s]), 1);
            mbar_init(saddr(&bar_free[s]), EPI_WARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbar_expect_tx(saddr(&bar_w), W_BYTES);
        bulk_copy(saddr(wsm), wpacked, W_BYTES, saddr(&bar_w));
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s_tmem;

    if (warp == 0) {
        if (lane == 0) {
            bool ok = mbar_wait_or_fail(saddr(&bar_w), 0, fail);
            w_ready = ok;
            const uint32_t rbase = saddr(ring);
            const uint64_t wd = sdesc(saddr(wsm), CP * 16, 128);
            for (int i = 0; ok && i < n; ++i) {
                while (ok && waited <= i + 2) {
                    ok = mbar_wait_or_fail(saddr(&bar_full[waited % S]), (uint32_t)((waited / S) & 1), fail);
                    if (ok) ++waited;
                }
                if (ok && i >= 2) ok = mbar_wait_or_fail(saddr(&bar_free[i & 1]), (uint32_t)(((i - 2) >> 1) & 1), fail);
                if (!ok) break;
                fence_after();
                // descriptors: one base per input slot, every MMA adds a
                // compile-time offset (16-byte units) to the address field
                // (addresses stay below 2^18, so nothing carries out of it)
                uint64_t sd[3];
                const int i_slot = i % S;
#pragma unroll
                for (int dz = 0; dz < 3; ++dz) {
                    const int sl = (i_slot + dz >= S) ? i_slot + dz - S : i_slot + dz;
                    sd[dz] = sdesc(rbase + (uint32_t)(sl * SLOT), GROUP_BYTES, 128);
                }
#pragma unroll
                for (int r = 0; r < TYO; ++r) {
                    const uint32_t d = tmem + (uint32_t)((i & 1) * 64 + r * 32);
#pragma unroll
                    for (int tap = 0; tap < 27; ++tap) {
                        const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
#pragma unroll
                        for (int s = 0; s < 2; ++s) {
                            const uint64_t a = sd[dz] + (uint64_t)(((2 * s) * R + r + dy) * HXV + dx);
                            const uint64_t bw = wd + (uint64_t)((tap * G + 2 * s) * CP);
                            mma(d, a, bw, (tap | s) ? 1u : 0u);
                        }
                    }
                }
                mma_commit(saddr(&bar_mma[i & 1]));
                mma_commit(saddr(&bar_empty[i % S]));     // plane i has no later reader
                committed = i + 1;
            }
            if (!ok) s_fail = 1;
        }
        __syncwarp();
    } else if (warp >= LOAD0) {
        // loaders: input plane q into slot q % S, [group][row][voxel][8 ch]
        const int lt = tid - LOAD0 * 32;
        const long long gnx = p.nx + 2;
        int published = 0;
        bool ok = true;
        auto publish = [&](int upto) {          // planes published .. upto-1 have landed
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            for (; published < upto; ++published) {
                if (lane == 0) mbar_arrive(saddr(&bar_full[published % S]));
            }
        };
        for (int q = 0; q <= n + 1; ++q) {
            const int slot = q % S;
            // publish what has landed before waiting for a slot: plane q-2
            // (all groups but the newest are complete), so the MMAs of the
            // plane that frees this slot never wait on this loader
            if (q >= 2) {
                asm volatile("cp.async.wait_group 1;" ::: "memory");
                publish(q - 1);
            }
            if (q >= S) {
                const bool got = mbar_wait_or_fail(saddr(&bar_empty[slot]), (uint32_t)(((q - S) / S) & 1), fail);
                if (!__all_sync(0xffffffffu, got)) {
                    ok = false;
                    break;
                }
            }
            unsigned char *dst = ring + slot * SLOT;
            const long long base = ((long long)(zg0 + q) * (p.ny + 2) + y0) * gnx + x0;   // ghosted voxel (row 0, voxel 0)
            for (int v = lt; v < R * HXV; v += LOAD_WARPS * 32) {
                const int yy = v / HXV;
                const int xx = v - yy * HXV;
                const __nv_bfloat16 *src = in + (base + (long long)yy * gnx + xx) * CP;
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const uint32_t d = saddr(dst + ((g * R + yy) * HXV + xx) * 16);
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src + 8 * g) : "memory");
                }
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        if (ok) publish(n + 2);
        else if (lane == 0) s_fail = 1;
    } else {
        // epilogue: lane quarter qd (TMEM lanes 32 qd .. 32 qd + 31 = voxels),
        // output row r of the tile
        const int qd = warp & 3;
        const int r = (warp - 1) >> 2;
        const int x = x0 + qd * 32 + lane;
        const int y = y0 + r;
        int xs[3], ys[3];         // an axis of extent 1 has both ghost copies
        int nxs = 1, nys = 1;
        xs[0] = x + 1;
        if (x == 0) xs[nxs++] = p.nx + 1;
        if (x == p.nx - 1) xs[nxs++] = 0;
        ys[0] = y + 1;
        if (y == 0) ys[nys++] = p.ny + 1;
        if (y == p.ny - 1) ys[nys++] = 0;
        float bv[24];
#pragma unroll
        for (int c = 0; c < 24; ++c) bv[c] = __ldg(bias + c);
        for (int j = 0; j < n; ++j) {
            const bool ok = mbar_wait_or_fail(saddr(&bar_mma[j & 1]), (uint32_t)((j >> 1) & 1), fail);
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) s_fail = 1;
                break;
            }
            fence_after();
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)((j & 1) * 64 + r * 32), v);
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(saddr(&bar_free[j & 1]));
            uint32_t w[12];
#pragma unroll
            for (int c = 0; c < 12; ++c) w[c] = pack_bf16(gelu(v[2 * c] + bv[2 * c]), gelu(v[2 * c + 1] + bv[2 * c + 1]));
            const int zz = z0 + j;
            int zs[3];
            int nzs = 1;
            zs[0] = zz + 1;
            if (zz == 0) zs[nzs++] = p.nz + 1;
            if (zz == p.nz - 1) zs[nzs++] = 0;
            for (int a = 0; a < nzs; ++a) {
                for (int bb = 0; bb < nys; ++bb) {
                    for (int c = 0; c < nxs; ++c) {
                        const long long vox =
                            (((long long)b * (p.nz + 2) + zs[a]) * (p.ny + 2) + ys[bb]) * (p.nx + 2) + xs[c];
                        uint4 *o = reinterpret_cast<uint4 *>(out + vox * CP);
                        o[0] = make_uint4(w[0], w[1], w[2], w[3]);
                        o[1] = make_uint4(w[4], w[5], w[6], w[7]);
                        o[2] = make_uint4(w[8], w[9], w[10], w[11]);
                        o[3] = make_uint4(0u, 0u, 0u, 0u);
                    }
                }
            }
        }
    }

    fence_before();
    __syncthreads();            // every role has left its loop; no copy is in flight
    fence_after();
    if (s_fail) {
        // report, then wait (bounded) for the MMAs and the weight copy
        if (tid == 0) {
            atomicExch(err, 1);
            if (committed > 0) mbar_wait(saddr(&bar_mma[(committed - 1) & 1]), ((committed - 1) >> 1) & 1);
            if (!w_ready) mbar_wait(saddr(&bar_w), 0);
        }
        fence_before();
        __syncthreads();
        fence_after();
    }
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// FP32 W[tap][cin][cout] (cin = cout = 24) -> BF16 B operand layout
__global__ void pack_tc_weights_kernel(const float *__restrict__ w, __nv_bfloat16 *__restrict__ out)
{
    const int total = 27 * G * CP * 8;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int k8 = i & 7;
        const int co = (i >> 3) & (CP - 1);
        const int g = (i >> 8) & (G - 1);
        const int tap = i >> 10;
        const int ci = g * 8 + k8;
        const float v = (ci < 24 && co < 24) ? w[(tap * 24 + ci) * 24 + co] : 0.f;
        out[i] = __float2bfloat16(v);
    }
}

}  // namespace tc

bool tc_applicable(int nx, int ny, int channels)
{
    return channels == 24 && nx % tc::TXO == 0 && ny % tc::TYO == 0;
}

size_t tc_weight_bytes() { return tc::W_BYTES; }

void tc_pack_weights(const float *w, void *out, cudaStream_t stream)
{
    tc::pack_tc_weights_kernel<<<27, 256, 0, stream>>>(w, (__nv_bfloat16 *)out);
    check_launch("pack tensor-core weights");
}

// one C -> C layer: ghosted BF16 in -> ghosted BF16 out (GELU(conv + bias))
void tc_conv(void *map_cache, const void *in, void *out, const void *wpacked, const float *bias, int nx, int ny, int nz,
             int batch, cudaStream_t stream, int *d_err)
{
    static PerDevice<long long> setup;
    const long long resident = setup.get([] {
        LGD_CHECK_CUDA(cudaFuncSetAttribute(tc::conv_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM));
        int dev = 0, sms = 0;
        LGD_CHECK_CUDA(cudaGetDevice(&dev));
        LGD_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        return (long long)sms;
    });
    (void)map_cache;
    // z chunks: whole waves of one CTA per SM
    const long long xy = (long long)(nx / tc::TXO) * (ny / tc::TYO) * batch;
    int best_chunk = nz;
    double best = 1e300;
    for (int split = 1; split <= std::max(1, nz / 4); ++split) {
        const int chunk = (nz + split - 1) / split;
        const int s = (nz + chunk - 1) / chunk;
        const long long waves = (xy * s + resident - 1) / resident;
        const double t = (double)waves * (chunk + 2);
        if (t < best * 0.999) {
            best = t;
            best_chunk = chunk;
        }
    }
    tc::Params p;
    p.nx = nx;
    p.ny = ny;
    p.nz = nz;
    p.batch = batch;
    p.zchunk = best_chunk;
    const int zsplit = (nz + best_chunk - 1) / best_chunk;
    dim3 grid(nx / tc::TXO, ny / tc::TYO, batch * zsplit);
    tc::conv_tc_kernel<<<grid, tc::THREADS, tc::SMEM, stream>>>((const __nv_bfloat16 *)in,
                                                                 (const __nv_bfloat16 *)wpacked, bias,
                                                                 (__nv_bfloat16 *)out, p, d_err);
    check_launch("tensor-core convolution");
}

}  // namespace sur
}  // namespace lgd
