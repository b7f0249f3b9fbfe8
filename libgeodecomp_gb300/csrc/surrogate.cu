// Learned surrogate for variable-coefficient diffusion: a 4-layer 3D
// convolutional network (channels 2 -> C -> C -> C -> 1, 3x3x3 kernels on
// the torus, GELU after the first three layers, residual u' = u + net), with
// its forward pass, backward pass and Adam update as hand-written kernels.
// No counterpart in the reference library.
//
// Convolutions are implicit GEMMs on the tensor cores (mma.sync
// m16n8k16, BF16 operands, FP32 accumulation): one CTA computes a
// TX x 4 x 1 tile of output voxels; the input halo (TX+2) x 6 x 3 voxels x
// CIN channels and the layer's weights (pre-packed in mma fragment order)
// are staged in shared memory, every warp owns one row of the tile
// (TX / 16 M-tiles) and walks K = 27 * CIN (tap-major, channel-minor,
// padded to 16).  Activations are channels-last BF16, [batch][z][y][x][C].
//
// The input gradient of a layer is the same convolution with the taps
// mirrored and the channel roles swapped (weights re-packed); the weight
// gradient is a GEMM over the voxels of a tile (M = 27 * CIN, N = COUT,
// K = voxels) accumulated in FP32 and added to the global gradient with
// atomics.  Parameters stay in FP32 (master copy), Adam runs in FP32 and
// re-packs the BF16 fragments after every update.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "lgd_internal.h"
#include "../../include/lgd_surrogate.h"

namespace lgd {
namespace sur {

typedef __nv_bfloat16 bf16;

static const int TYT = 4;        // rows per tile (one per warp)
static const int THREADS = 128;

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi)
{
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ float gelu_f(float z)
{
    return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}

__device__ __forceinline__ float gelu_grad_f(float z)
{
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * expf(-0.5f * z * z) * 0.39894228040143268f;
}

__host__ __device__ constexpr int ceil_div(int a, int b) { return (a + b - 1) / b; }

struct Geo {
    int nx, ny, nz, batch;
};

// Halo tile of the layer input for the CTA at (x0, y0, z, b): (TX+2) x 6 x 3
// voxels, wrapped on the torus, CIN BF16 channels each (CIN even).  GIN:
// the input is ghosted ([batch][nz+2][ny+2][nx+2][32], the wrapped
// neighbours stored in the ghost layer), else dense [V][CIN].
template<int CIN, int TX, bool GIN = false>
__device__ __forceinline__ void load_halo(uint32_t *halo, const bf16 *__restrict__ in, const Geo& g, int x0, int y0,
                                          int z, int b)
{
    constexpr int HX = TX + 2;
    constexpr int HY = TYT + 2;
    constexpr int WORDS = CIN / 2;
    const int total = 3 * HY * HX * WORDS;
    const uint32_t *src = reinterpret_cast<const uint32_t *>(in);
    for (int i = threadIdx.x; i < total; i += THREADS) {
        const int w = i % WORDS;
        const int vox = i / WORDS;
        const int hx = vox % HX;
        const int hy = (vox / HX) % HY;
        const int hz = vox / (HX * HY);
        int gx = x0 - 1 + hx;
        int gy = y0 - 1 + hy;
        int gz = z - 1 + hz;
        if (GIN) {
            const long long v = (((long long)b * (g.nz + 2) + gz + 1) * (g.ny + 2) + gy + 1) * (g.nx + 2) + gx + 1;
            halo[i] = src[v * 16 + w];
        } else {
            gx = (gx < 0) ? gx + g.nx : (gx >= g.nx ? gx - g.nx : gx);
            gy = (gy < 0) ? gy + g.ny : (gy >= g.ny ? gy - g.ny : gy);
            gz = (gz < 0) ? gz + g.nz : (gz >= g.nz ? gz - g.nz : gz);
            const long long v = (((long long)b * g.nz + gz) * g.ny + gy) * g.nx + gx;
            halo[i] = src[v * WORDS + w];
        }
    }
}

// BF16 pair (channels co, co+1) of voxel (x, y, z, b) into a ghosted
// activation buffer, at its own position and its ghost copies
__device__ __forceinline__ void store_ghosted(bf16 *__restrict__ out, const Geo& g, int x, int y, int z, int b, int co,
                                              uint32_t pair)
{
    int xs[3], ys[3], zs[3];
    int nxs = 1, nys = 1, nzs = 1;
    xs[0] = x + 1;
    if (x == 0) xs[nxs++] = g.nx + 1;
    if (x == g.nx - 1) xs[nxs++] = 0;
    ys[0] = y + 1;
    if (y == 0) ys[nys++] = g.ny + 1;
    if (y == g.ny - 1) ys[nys++] = 0;
    zs[0] = z + 1;
    if (z == 0) zs[nzs++] = g.nz + 1;
    if (z == g.nz - 1) zs[nzs++] = 0;
    for (int a = 0; a < nzs; ++a) {
        for (int c = 0; c < nys; ++c) {
            for (int d = 0; d < nxs; ++d) {
                const long long v = (((long long)b * (g.nz + 2) + zs[a]) * (g.ny + 2) + ys[c]) * (g.nx + 2) + xs[d];
                *reinterpret_cast<uint32_t *>(out + v * 32 + co) = pair;
            }
        }
    }
}

// ------------------------------------------------------------ forward conv
// MODE 0: out_h = gelu(acc + bias) in BF16 (COUT even), out_z = acc + bias
//         in FP32 when non-null.  MODE 1: out_f = acc (+ bias when
//         non-null) in FP32 for co < COUT.  MODE 2: as MODE 0 without
//         out_z, into a ghosted buffer (own position and ghost copies).
// GIN: the input is ghosted (see load_halo).
template<int CIN, int COUT, int TX, int MODE, bool GIN = false>
__global__ void __launch_bounds__(THREADS)
conv_fwd_kernel(const bf16 *__restrict__ in, const uint2 *__restrict__ wfrag, const float *__restrict__ bias, Geo g,
                bf16 *__restrict__ out_h, float *__restrict__ out_z, float *__restrict__ out_f)
{
    constexpr int K = 27 * CIN;
    constexpr int KS = ceil_div(K, 16);
    constexpr int NT = ceil_div(COUT, 8);
    constexpr int MT = TX / 16;
    constexpr int HX = TX + 2;
    constexpr int HY = TYT + 2;
    extern __shared__ uint32_t smem[];
    uint32_t *halo = smem;                                        // 3 * HY * HX * CIN / 2 words
    uint2 *wsm = reinterpret_cast<uint2 *>(smem + ((3 * HY * HX * CIN / 2 + 3) & ~3));   // 16-byte aligned
    // MODE 2: the tile's output voxels, 16 words (32 BF16 channels) each
    uint32_t *otile = reinterpret_cast<uint32_t *>(wsm + KS * NT * 32);

    const int x0 = blockIdx.x * TX;
    const int y0 = blockIdx.y * TYT;
    const int z = blockIdx.z % g.nz;
    const int b = blockIdx.z / g.nz;
    load_halo<CIN, TX, GIN>(halo, in, g, x0, y0, z, b);
    for (int i = threadIdx.x; i < KS * NT * 32; i += THREADS) wsm[i] = wfrag[i];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int gq = lane >> 2;
    const int tq = lane & 3;
    const bf16 *hb = reinterpret_cast<const bf16 *>(halo);

    float acc[MT][NT][4];
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int n = 0; n < NT; ++n)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[m][n][r] = 0.f;

    for (int ks = 0; ks < KS; ++ks) {
        int base[2];
        int ci[2];
        bool valid[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = ks * 16 + 2 * tq + 8 * h;
            const int tap = k / CIN;
            ci[h] = k - tap * CIN;
            valid[h] = k < K;
            const int dz = tap / 9 - 1;
            const int dy = (tap / 3) % 3 - 1;
            const int dx = tap % 3 - 1;
            base[h] = ((dz + 1) * HY + (warp + 1 + dy)) * HX + (1 + dx);
        }
        uint2 bf[NT];
#pragma unroll
        for (int n = 0; n < NT; ++n) bf[n] = wsm[(ks * NT + n) * 32 + lane];
#pragma unroll
        for (int m = 0; m < MT; ++m) {
            const int xr = m * 16 + gq;
            uint32_t a[4];
            a[0] = valid[0] ? *reinterpret_cast<const uint32_t *>(hb + (base[0] + xr) * CIN + ci[0]) : 0u;
            a[1] = valid[0] ? *reinterpret_cast<const uint32_t *>(hb + (base[0] + xr + 8) * CIN + ci[0]) : 0u;
            a[2] = valid[1] ? *reinterpret_cast<const uint32_t *>(hb + (base[1] + xr) * CIN + ci[1]) : 0u;
            a[3] = valid[1] ? *reinterpret_cast<const uint32_t *>(hb + (base[1] + xr + 8) * CIN + ci[1]) : 0u;
#pragma unroll
            for (int n = 0; n < NT; ++n) mma_bf16(acc[m][n], a, bf[n].x, bf[n].y);
        }
    }

    const int y = y0 + warp;
#pragma unroll
    for (int m = 0; m < MT; ++m) {
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int x = x0 + m * 16 + gq + 8 * half;
            const long long v = (((long long)b * g.nz + z) * g.ny + y) * g.nx + x;
#pragma unroll
            for (int n = 0; n < NT; ++n) {
                const int co = n * 8 + 2 * tq;
                const float r0 = acc[m][n][2 * half];
                const float r1 = acc[m][n][2 * half + 1];
                if (MODE == 0) {
                    if (co < COUT) {
                        const float z0 = r0 + bias[co];
                        const float z1 = r1 + bias[co + 1];
                        if (out_z) {
                            out_z[v * COUT + co] = z0;
                            out_z[v * COUT + co + 1] = z1;
                        }
                        *reinterpret_cast<uint32_t *>(out_h + v * COUT + co) =
                            pack2(__float2bfloat16(gelu_f(z0)), __float2bfloat16(gelu_f(z1)));
                    }
                } else if (MODE == 2) {
                    const int vt = warp * TX + (x - x0);
                    if (co < COUT) {
                        const float z0 = r0 + bias[co];
                        const float z1 = r1 + bias[co + 1];
                        otile[vt * 16 + co / 2] = pack2(__float2bfloat16(gelu_f(z0)), __float2bfloat16(gelu_f(z1)));
                    } else if (co < 32) {
                        otile[vt * 16 + co / 2] = 0u;
                    }
                } else {
                    if (co < COUT) out_f[v * COUT + co] = r0 + (bias ? bias[co] : 0.f);
                    if (co + 1 < COUT) out_f[v * COUT + co + 1] = r1 + (bias ? bias[co + 1] : 0.f);
                }
            }
        }
    }
    if (MODE == 2) {
        // channels COUT .. 31 of the staged voxels (the n-tiles stop at COUT)
        for (int i = threadIdx.x; i < TYT * TX * (16 - NT * 4); i += THREADS) {
            const int per = 16 - NT * 4;
            otile[(i / per) * 16 + NT * 4 + i % per] = 0u;
        }
        __syncthreads();
        // one 64-byte record per voxel, at its position and its ghost copies
        for (int vt = threadIdx.x; vt < TYT * TX; vt += THREADS) {
            const uint4 *src = reinterpret_cast<const uint4 *>(otile + vt * 16);
            const uint4 q0 = src[0], q1 = src[1], q2 = src[2], q3 = src[3];
            const int x = x0 + vt % TX;
            const int yv = y0 + vt / TX;
            int xs[3], ys[3], zs[3];     // an axis of extent 1 has both ghost copies
            int nxs = 1, nys = 1, nzs = 1;
            xs[0] = x + 1;
            if (x == 0) xs[nxs++] = g.nx + 1;
            if (x == g.nx - 1) xs[nxs++] = 0;
            ys[0] = yv + 1;
            if (yv == 0) ys[nys++] = g.ny + 1;
            if (yv == g.ny - 1) ys[nys++] = 0;
            zs[0] = z + 1;
            if (z == 0) zs[nzs++] = g.nz + 1;
            if (z == g.nz - 1) zs[nzs++] = 0;
            for (int a = 0; a < nzs; ++a) {
                for (int c = 0; c < nys; ++c) {
                    for (int d = 0; d < nxs; ++d) {
                        const long long v =
                            (((long long)b * (g.nz + 2) + zs[a]) * (g.ny + 2) + ys[c]) * (g.nx + 2) + xs[d];
                        uint4 *o = reinterpret_cast<uint4 *>(out_h + v * 32);
                        o[0] = q0;
                        o[1] = q1;
                        o[2] = q2;
                        o[3] = q3;
                    }
                }
            }
        }
    }
}

// ------------------------------------------------------ weight gradient
// dW[(tap * CIN + ci) * COUT + co] += sum over the tile's voxels v of
// in[v + off(tap)][ci] * dz[v][co]; dz is [V][COUTP] BF16 (COUTP = COUT
// rounded up to even).
template<int CIN, int COUT, int TX>
__global__ void __launch_bounds__(THREADS)
conv_wgrad_kernel(const bf16 *__restrict__ in, const bf16 *__restrict__ dz, Geo g, float *__restrict__ dW)
{
    constexpr int M = 27 * CIN;
    constexpr int MT = ceil_div(M, 16);
    constexpr int NT = ceil_div(COUT, 8);
    constexpr int COUTP = (COUT + 1) & ~1;
    constexpr int HX = TX + 2;
    constexpr int HY = TYT + 2;
    constexpr int KS = TYT * TX / 16;
    extern __shared__ uint32_t smem[];
    uint32_t *halo = smem;
    bf16 *dzt = reinterpret_cast<bf16 *>(smem + 3 * HY * HX * CIN / 2);   // [TYT * TX][COUTP]

    const int x0 = blockIdx.x * TX;
    const int y0 = blockIdx.y * TYT;
    const int z = blockIdx.z % g.nz;
    const int b = blockIdx.z / g.nz;
    load_halo<CIN, TX>(halo, in, g, x0, y0, z, b);
    for (int i = threadIdx.x; i < TYT * TX * COUTP; i += THREADS) {
        const int c = i % COUTP;
        const int t = i / COUTP;
        const int xx = t % TX;
        const int yy = t / TX;
        const long long v = (((long long)b * g.nz + z) * g.ny + (y0 + yy)) * g.nx + (x0 + xx);
        dzt[i] = dz[v * COUTP + c];
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int gq = lane >> 2;
    const int tq = lane & 3;
    const bf16 *hb = reinterpret_cast<const bf16 *>(halo);
    const bf16 zero = __float2bfloat16(0.f);

    for (int mt = warp; mt < MT; mt += THREADS / 32) {
        int off[2];
        bool mv[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int m = mt * 16 + gq + 8 * h;
            mv[h] = m < M;
            const int tap = mv[h] ? m / CIN : 0;
            const int ci = mv[h] ? m - tap * CIN : 0;
            const int dz_ = tap / 9 - 1;
            const int dy = (tap / 3) % 3 - 1;
            const int dx = tap % 3 - 1;
            off[h] = (((dz_ + 1) * HY + (1 + dy)) * HX + (1 + dx)) * CIN + ci;
        }
        float acc[NT][4];
#pragma unroll
        for (int n = 0; n < NT; ++n)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[n][r] = 0.f;
        for (int ks = 0; ks < KS; ++ks) {
            const int k0 = ks * 16 + 2 * tq;    // the 16 voxels of a step share one tile row
            const int yy = k0 / TX;
            const int xx = k0 - yy * TX;
            const int vo = (yy * HX + xx) * CIN;
            uint32_t a[4];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const bf16 *p = hb + off[h] + vo;
                a[h] = mv[h] ? pack2(p[0], p[CIN]) : 0u;                   // voxels k0, k0 + 1
                a[2 + h] = mv[h] ? pack2(p[8 * CIN], p[9 * CIN]) : 0u;     // voxels k0 + 8, k0 + 9
            }
#pragma unroll
            for (int n = 0; n < NT; ++n) {
                const int co = n * 8 + gq;
                const bf16 *q = dzt + k0 * COUTP + co;
                const bool cv = co < COUT;
                const uint32_t b0 = cv ? pack2(q[0], q[COUTP]) : pack2(zero, zero);
                const uint32_t b1 = cv ? pack2(q[8 * COUTP], q[9 * COUTP]) : pack2(zero, zero);
                mma_bf16(acc[n], a, b0, b1);
            }
        }
#pragma unroll
        for (int n = 0; n < NT; ++n) {
            const int co = n * 8 + 2 * tq;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int m = mt * 16 + gq + 8 * h;
                if (m < M) {
                    if (co < COUT) atomicAdd(&dW[m * COUT + co], acc[n][2 * h]);
                    if (co + 1 < COUT) atomicAdd(&dW[m * COUT + co + 1], acc[n][2 * h + 1]);
                }
            }
        }
    }
}

// ------------------------------------------------------- elementwise parts
__global__ void pack_input_kernel(const float *__restrict__ u, const float *__restrict__ k, bf16 *__restrict__ x,
                                  long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        *reinterpret_cast<uint32_t *>(x + 2 * i) = pack2(__float2bfloat16(u[i]), __float2bfloat16(k[i]));
    }
}

// dz = dh * gelu'(z) in BF16, and db[c] += sum of dz over the voxels
template<int C>
__global__ void gelu_bwd_kernel(const float *__restrict__ dh, const float *__restrict__ zv, bf16 *__restrict__ dz,
                                float *__restrict__ db, long long nvox)
{
    __shared__ float red[C];
    for (int c = threadIdx.x; c < C; c += blockDim.x) red[c] = 0.f;
    __syncthreads();
    float part[C];
#pragma unroll
    for (int c = 0; c < C; ++c) part[c] = 0.f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < C; c += 2) {
            const float g0 = dh[v * C + c] * gelu_grad_f(zv[v * C + c]);
            const float g1 = dh[v * C + c + 1] * gelu_grad_f(zv[v * C + c + 1]);
            part[c] += g0;
            part[c + 1] += g1;
            *reinterpret_cast<uint32_t *>(dz + v * C + c) = pack2(__float2bfloat16(g0), __float2bfloat16(g1));
        }
    }
#pragma unroll
    for (int c = 0; c < C; ++c) atomicAdd(&red[c], part[c]);
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) atomicAdd(&db[c], red[c]);
}

// MSE loss of du against target: g = 2 (du - t) / N as the BF16 gradient of
// the last layer ([V][2], channel 1 zero), db4 += sum g, loss += sum diff^2
__global__ void loss_kernel(const float *__restrict__ du, const float *__restrict__ target, bf16 *__restrict__ dz4,
                            float *__restrict__ db4, double *__restrict__ loss, long long nvox)
{
    __shared__ double sl[256];
    __shared__ float sg[256];
    double l = 0.0;
    float gs = 0.f;
    const float scale = 2.0f / (float)nvox;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x) {
        const float d = du[v] - target[v];
        l += (double)d * d;
        const float gv = scale * d;
        gs += gv;
        *reinterpret_cast<uint32_t *>(dz4 + 2 * v) = pack2(__float2bfloat16(gv), __float2bfloat16(0.f));
    }
    sl[threadIdx.x] = l;
    sg[threadIdx.x] = gs;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sl[threadIdx.x] += sl[threadIdx.x + s];
            sg[threadIdx.x] += sg[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(loss, sl[0]);
        atomicAdd(db4, sg[0]);
    }
}

__global__ void add_inplace_kernel(float *__restrict__ u, const float *__restrict__ du, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        u[i] += du[i];
    }
}

// Fragment packing.  Forward: B[k][n] = W[k][n] (W flat [27 * CIN][COUT]).
// Input-gradient convolution: CIN' = COUTP, COUT' = CIN,
// B'[k'][n'] = W[((26 - tap') * CIN + n') * COUT + co] with k' = tap' * CIN' + co.
__global__ void pack_frag_kernel(const float *__restrict__ w, uint2 *__restrict__ frag, int cin, int cout, int mirror,
                                 int cin_eff, int cout_eff)
{
    // cin_eff / cout_eff: the convolution's own channel counts (K = 27 * cin_eff)
    const int K = 27 * cin_eff;
    const int KS = (K + 15) / 16;
    const int NT = (cout_eff + 7) / 8;
    const int total = KS * NT * 32;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int lane = i % 32;
        const int nt = (i / 32) % NT;
        const int ks = i / (32 * NT);
        const int gq = lane >> 2;
        const int tq = lane & 3;
        const int n = nt * 8 + gq;
        float vals[4];
        const int ks4[4] = {ks * 16 + 2 * tq, ks * 16 + 2 * tq + 1, ks * 16 + 2 * tq + 8, ks * 16 + 2 * tq + 9};
        for (int j = 0; j < 4; ++j) {
            const int k = ks4[j];
            float v = 0.f;
            if (k < K && n < cout_eff) {
                const int tap = k / cin_eff;
                const int c = k - tap * cin_eff;
                if (!mirror) {
                    v = w[(tap * cin + c) * cout + n];
                } else if (c < cout) {
                    // c is the layer's output channel, n its input channel
                    v = w[((26 - tap) * cin + n) * cout + c];
                }
            }
            vals[j] = v;
        }
        uint2 r;
        r.x = pack2(__float2bfloat16(vals[0]), __float2bfloat16(vals[1]));
        r.y = pack2(__float2bfloat16(vals[2]), __float2bfloat16(vals[3]));
        frag[i] = r;
    }
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                            float *__restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                            float c2)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float g = gr[i];
        const float mi = b1 * m[i] + (1.f - b1) * g;
        const float vi = b2 * v[i] + (1.f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// ------------------------------------------------------------- network
struct Layer {
    int cin, cout;
    long long w_off, b_off;     // offsets into the flat parameter vector
    uint2 *frag;                // forward fragments
    uint2 *frag_t;              // input-gradient fragments
    int frag_n, frag_t_n;
};

struct Net {
    Geo g;
    int C;
    int TX;
    bool training;
    long long V;
    long long P;
    float *params, *grads, *m, *v;
    Layer L[4];
    bf16 *x0;           // [V][2]
    bf16 *h[3];         // [V][C]
    float *zb[3];       // [V][C] pre-activations (training)
    float *du;          // [V]
    float *dh;          // [V][C] FP32 input gradient
    bf16 *dzb;          // [V][C] BF16 gradient
    bf16 *dz4;          // [V][2]
    double *d_loss;
    int t;              // Adam step
    cudaStream_t stream;
    uint64_t launches;
    // tensor-core (tcgen05) inference path: C = 24, nx % 128 == 0, ny even,
    // no training buffers; layers 2 and 3 on tcgen05, 1 and 4 on mma.sync
    bool fast;
    int variant;        // 0: tcgen05 path where it applies; 1: mma.sync for every layer
    bf16 *hg[2];        // ghosted activations [batch][nz+2][ny+2][nx+2][32]
    void *wtc[2];       // weights of layers 2 and 3 in the tcgen05 B layout
    int *d_err;         // bounded waits of the tcgen05 kernel
    alignas(64) unsigned char tmap[128];
};

bool tc_applicable(int nx, int ny, int channels);
size_t tc_weight_bytes();
void tc_pack_weights(const float *w, void *out, cudaStream_t stream);
void tc_conv(void *map_cache, const void *in, void *out, const void *wpacked, const float *bias, int nx, int ny, int nz,
             int batch, cudaStream_t stream, int *d_err);
bool last_conv_applicable(int nx, int ny, int channels);
void last_conv(const void *h, const float *w, const float *bias, float *out, bool add_to_u, int nx, int ny, int nz,
               int batch, cudaStream_t stream);

static int layer_frag_words(int cin, int cout)
{
    return ceil_div(27 * cin, 16) * ceil_div(cout, 8) * 32;
}

template<int CIN, int COUT, int TX, int MODE = 0>
static size_t fwd_smem()
{
    // MODE 2 adds the staged output tile (TYT x TX voxels x 32 BF16 channels)
    return (size_t)(((3 * (TYT + 2) * (TX + 2) * CIN / 2 + 3) & ~3) * 4 + layer_frag_words(CIN, COUT) * 8) +
           (MODE == 2 ? (size_t)TYT * TX * 64 : 0);
}

template<int CIN, int COUT, int TX>
static size_t wgrad_smem()
{
    return (size_t)(3 * (TYT + 2) * (TX + 2) * CIN / 2) * 4 + (size_t)TYT * TX * ((COUT + 1) & ~1) * 2;
}

template<int CIN, int COUT, int TX, int MODE, bool GIN = false>
static void run_fwd(Net& n, const bf16 *in, const uint2 *frag, const float *bias, bf16 *oh, float *oz, float *of)
{
    const size_t sm = fwd_smem<CIN, COUT, TX, MODE>();
    static PerDevice<bool> setup;             // per instantiation, per device
    setup.get([sm] {
        LGD_CHECK_CUDA(cudaFuncSetAttribute(conv_fwd_kernel<CIN, COUT, TX, MODE, GIN>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        return true;
    });
    dim3 grid(n.g.nx / TX, n.g.ny / TYT, n.g.nz * n.g.batch);
    conv_fwd_kernel<CIN, COUT, TX, MODE, GIN><<<grid, THREADS, sm, n.stream>>>(in, frag, bias, n.g, oh, oz, of);
    check_launch("conv forward");
    ++n.launches;
}

template<int CIN, int COUT, int TX>
static void run_wgrad(Net& n, const bf16 *in, const bf16 *dz, float *dW)
{
    const size_t sm = wgrad_smem<CIN, COUT, TX>();
    static PerDevice<bool> setup;
    setup.get([sm] {
        LGD_CHECK_CUDA(cudaFuncSetAttribute(conv_wgrad_kernel<CIN, COUT, TX>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        return true;
    });
    dim3 grid(n.g.nx / TX, n.g.ny / TYT, n.g.nz * n.g.batch);
    conv_wgrad_kernel<CIN, COUT, TX><<<grid, THREADS, sm, n.stream>>>(in, dz, n.g, dW);
    check_launch("conv weight gradient");
    ++n.launches;
}

static int grid_blocks(long long n)
{
    long long b = (n + 255) / 256;
    return (int)std::min<long long>(b, 152LL * 16);
}

static void repack(Net& n)
{
    for (int l = 0; l < 4; ++l) {
        Layer& L = n.L[l];
        pack_frag_kernel<<<64, 256, 0, n.stream>>>(n.params + L.w_off, L.frag, L.cin, L.cout, 0, L.cin, L.cout);
        const int coutp = (L.cout + 1) & ~1;
        pack_frag_kernel<<<64, 256, 0, n.stream>>>(n.params + L.w_off, L.frag_t, L.cin, L.cout, 1, coutp, L.cin);
        n.launches += 2;
    }
    check_launch("pack fragments");
    if (n.fast) {
        tc_pack_weights(n.params + n.L[1].w_off, n.wtc[0], n.stream);
        tc_pack_weights(n.params + n.L[2].w_off, n.wtc[1], n.stream);
        n.launches += 2;
    }
}

// Inference with the tcgen05 layers: input packing, layer 1 (mma.sync) into
// a ghosted buffer, layers 2 and 3 on tcgen05 between the two ghosted
// buffers, layer 4 from the ghosted buffer into du (the tap-product kernel
// of conv_last.cu where the tile fits, else mma.sync).  With add_to_u the
// last layer adds its result to u instead (u <- u + du, the residual step).
// Returns whether it did.
template<int TX>
static bool forward_fast_impl(Net& n, const float *u, const float *k, float *du, bool add_to_u)
{
    pack_input_kernel<<<grid_blocks(n.V), 256, 0, n.stream>>>(u, k, n.x0, n.V);
    ++n.launches;
    run_fwd<2, 24, TX, 2>(n, n.x0, n.L[0].frag, n.params + n.L[0].b_off, n.hg[0], nullptr, nullptr);
    tc_conv(n.tmap, n.hg[0], n.hg[1], n.wtc[0], n.params + n.L[1].b_off, n.g.nx, n.g.ny, n.g.nz, n.g.batch, n.stream,
            n.d_err);
    ++n.launches;
    tc_conv(n.tmap, n.hg[1], n.hg[0], n.wtc[1], n.params + n.L[2].b_off, n.g.nx, n.g.ny, n.g.nz, n.g.batch, n.stream,
            n.d_err);
    ++n.launches;
    if (last_conv_applicable(n.g.nx, n.g.ny, n.C)) {
        last_conv(n.hg[0], n.params + n.L[3].w_off, n.params + n.L[3].b_off, add_to_u ? const_cast<float *>(u) : du,
                  add_to_u, n.g.nx, n.g.ny, n.g.nz, n.g.batch, n.stream);
        ++n.launches;
        return add_to_u;
    }
    run_fwd<24, 1, TX, 1, true>(n, n.hg[0], n.L[3].frag, n.params + n.L[3].b_off, nullptr, nullptr, du);
    return false;
}

// the network's channel count is a template parameter of the kernels; the
// library is built for C = 24 (the configured surrogate) and C = 8 (tests)
template<int C, int TX>
static void forward_impl(Net& n, const float *u, const float *k, float *du)
{
    pack_input_kernel<<<grid_blocks(n.V), 256, 0, n.stream>>>(u, k, n.x0, n.V);
    ++n.launches;
    float *z0 = n.training ? n.zb[0] : nullptr;
    float *z1 = n.training ? n.zb[1] : nullptr;
    float *z2 = n.training ? n.zb[2] : nullptr;
    // without training, two BF16 buffers alternate
    bf16 *h1 = n.h[0];
    bf16 *h2 = n.h[1];
    bf16 *h3 = n.training ? n.h[2] : n.h[0];
    run_fwd<2, C, TX, 0>(n, n.x0, n.L[0].frag, n.params + n.L[0].b_off, h1, z0, nullptr);
    run_fwd<C, C, TX, 0>(n, h1, n.L[1].frag, n.params + n.L[1].b_off, h2, z1, nullptr);
    run_fwd<C, C, TX, 0>(n, h2, n.L[2].frag, n.params + n.L[2].b_off, h3, z2, nullptr);
    run_fwd<C, 1, TX, 1>(n, h3, n.L[3].frag, n.params + n.L[3].b_off, nullptr, nullptr, du);
}

template<int C, int TX>
static void backward_impl(Net& n, const float *target, double *loss_out)
{
    LGD_CHECK_CUDA(cudaMemsetAsync(n.grads, 0, sizeof(float) * n.P, n.stream));
    LGD_CHECK_CUDA(cudaMemsetAsync(n.d_loss, 0, sizeof(double), n.stream));
    loss_kernel<<<grid_blocks(n.V), 256, 0, n.stream>>>(n.du, target, n.dz4, n.grads + n.L[3].b_off, n.d_loss, n.V);
    ++n.launches;
    // layer 4: dW4, then dH3 = conv_t(dz4)
    run_wgrad<C, 1, TX>(n, n.h[2], n.dz4, n.grads + n.L[3].w_off);
    run_fwd<2, C, TX, 1>(n, n.dz4, n.L[3].frag_t, nullptr, nullptr, nullptr, n.dh);
    gelu_bwd_kernel<C><<<grid_blocks(n.V), 256, 0, n.stream>>>(n.dh, n.zb[2], n.dzb, n.grads + n.L[2].b_off, n.V);
    ++n.launches;
    // layer 3
    run_wgrad<C, C, TX>(n, n.h[1], n.dzb, n.grads + n.L[2].w_off);
    run_fwd<C, C, TX, 1>(n, n.dzb, n.L[2].frag_t, nullptr, nullptr, nullptr, n.dh);
    gelu_bwd_kernel<C><<<grid_blocks(n.V), 256, 0, n.stream>>>(n.dh, n.zb[1], n.dzb, n.grads + n.L[1].b_off, n.V);
    ++n.launches;
    // layer 2
    run_wgrad<C, C, TX>(n, n.h[0], n.dzb, n.grads + n.L[1].w_off);
    run_fwd<C, C, TX, 1>(n, n.dzb, n.L[1].frag_t, nullptr, nullptr, nullptr, n.dh);
    gelu_bwd_kernel<C><<<grid_blocks(n.V), 256, 0, n.stream>>>(n.dh, n.zb[0], n.dzb, n.grads + n.L[0].b_off, n.V);
    ++n.launches;
    // layer 1 (no input gradient)
    run_wgrad<2, C, TX>(n, n.x0, n.dzb, n.grads + n.L[0].w_off);
    if (loss_out) {
        double l = 0.0;
        LGD_CHECK_CUDA(cudaMemcpyAsync(&l, n.d_loss, sizeof(double), cudaMemcpyDeviceToHost, n.stream));
        LGD_CHECK_CUDA(cudaStreamSynchronize(n.stream));
        *loss_out = l / (double)n.V;
    }
}

// du = net(u, k); with add_to_u the fast path may add du to u itself
// (returns true when it did)
static bool forward(Net& n, const float *u, const float *k, float *du, bool add_to_u = false)
{
    if (n.fast && n.variant == 0) {
        return n.TX == 64 ? forward_fast_impl<64>(n, u, k, du, add_to_u) : forward_fast_impl<32>(n, u, k, du, add_to_u);
    }
    if (n.C == 24) {
        if (n.TX == 64) forward_impl<24, 64>(n, u, k, du); else forward_impl<24, 32>(n, u, k, du);
    } else {
        if (n.TX == 64) forward_impl<8, 64>(n, u, k, du); else forward_impl<8, 32>(n, u, k, du);
    }
    return false;
}

static void backward(Net& n, const float *target, double *loss)
{
    if (n.C == 24) {
        if (n.TX == 64) backward_impl<24, 64>(n, target, loss); else backward_impl<24, 32>(n, target, loss);
    } else {
        if (n.TX == 64) backward_impl<8, 64>(n, target, loss); else backward_impl<8, 32>(n, target, loss);
    }
}

static void net_free(Net& n)
{
    if (n.stream) cudaStreamSynchronize(n.stream);
    cudaFree(n.params);
    cudaFree(n.grads);
    cudaFree(n.m);
    cudaFree(n.v);
    for (int l = 0; l < 4; ++l) {
        cudaFree(n.L[l].frag);
        cudaFree(n.L[l].frag_t);
    }
    cudaFree(n.x0);
    for (int i = 0; i < 3; ++i) {
        cudaFree(n.h[i]);
        cudaFree(n.zb[i]);
    }
    cudaFree(n.du);
    cudaFree(n.dh);
    cudaFree(n.dzb);
    cudaFree(n.dz4);
    cudaFree(n.d_loss);
    cudaFree(n.hg[0]);
    cudaFree(n.hg[1]);
    cudaFree(n.wtc[0]);
    cudaFree(n.wtc[1]);
    cudaFree(n.d_err);
    if (n.stream) cudaStreamDestroy(n.stream);
}

static Net& net_of(lgd_net *h)
{
    LGD_REQUIRE(h != nullptr, LGD_ERR_INVALID, "null handle");
    return *reinterpret_cast<Net *>(h);
}

static long long param_count(int C)
{
    const int shapes[4][2] = {{2, C}, {C, C}, {C, C}, {C, 1}};
    long long p = 0;
    for (int l = 0; l < 4; ++l) p += 27LL * shapes[l][0] * shapes[l][1] + shapes[l][1];
    return p;
}

}  // namespace sur
}  // namespace lgd

using namespace lgd;
using namespace lgd::sur;

extern "C" {

int lgd_net_param_count(int channels, int64_t *count)
{
    return guard([&] {
        LGD_REQUIRE(channels == 24 || channels == 8, LGD_ERR_UNSUPPORTED, "the library is built for 24 or 8 channels");
        LGD_REQUIRE(count != nullptr, LGD_ERR_INVALID, "null output");
        *count = param_count(channels);
    });
}

int lgd_net_create(int nx, int ny, int nz, int batch, int channels, int training, lgd_net **out)
{
    return guard([&] {
        LGD_REQUIRE(out != nullptr, LGD_ERR_INVALID, "null output");
        *out = nullptr;
        LGD_REQUIRE(channels == 24 || channels == 8, LGD_ERR_UNSUPPORTED, "the library is built for 24 or 8 channels");
        LGD_REQUIRE(nx > 0 && ny > 0 && nz > 0 && batch > 0, LGD_ERR_INVALID, "sizes must be positive");
        LGD_REQUIRE(nx % 32 == 0, LGD_ERR_UNSUPPORTED, "nx must be a multiple of 32");
        LGD_REQUIRE(ny % TYT == 0, LGD_ERR_UNSUPPORTED, "ny must be a multiple of 4");
        Net *n = new Net();
        std::memset(n, 0, sizeof(Net));
        n->g.nx = nx;
        n->g.ny = ny;
        n->g.nz = nz;
        n->g.batch = batch;
        n->C = channels;
        n->TX = (nx % 64 == 0) ? 64 : 32;
        n->training = training != 0;
        n->V = (long long)nx * ny * nz * batch;
        n->P = param_count(channels);
        const int C = channels;
        const int shapes[4][2] = {{2, C}, {C, C}, {C, C}, {C, 1}};
        try {
            LGD_CHECK_CUDA(cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking));
            LGD_CHECK_CUDA(cudaMalloc(&n->params, sizeof(float) * n->P));
            LGD_CHECK_CUDA(cudaMemsetAsync(n->params, 0, sizeof(float) * n->P, n->stream));
            long long off = 0;
            for (int l = 0; l < 4; ++l) {
                Layer& L = n->L[l];
                L.cin = shapes[l][0];
                L.cout = shapes[l][1];
                L.w_off = off;
                off += 27LL * L.cin * L.cout;
                L.b_off = off;
                off += L.cout;
                L.frag_n = layer_frag_words(L.cin, L.cout);
                L.frag_t_n = layer_frag_words((L.cout + 1) & ~1, L.cin);
                LGD_CHECK_CUDA(cudaMalloc(&L.frag, sizeof(uint2) * L.frag_n));
                LGD_CHECK_CUDA(cudaMalloc(&L.frag_t, sizeof(uint2) * L.frag_t_n));
            }
            const long long V = n->V;
            LGD_CHECK_CUDA(cudaMalloc(&n->x0, sizeof(bf16) * 2 * V));
            const int nh = n->training ? 3 : 2;
            for (int i = 0; i < nh; ++i) LGD_CHECK_CUDA(cudaMalloc(&n->h[i], sizeof(bf16) * C * V));
            LGD_CHECK_CUDA(cudaMalloc(&n->du, sizeof(float) * V));
            if (n->training) {
                for (int i = 0; i < 3; ++i) LGD_CHECK_CUDA(cudaMalloc(&n->zb[i], sizeof(float) * C * V));
                LGD_CHECK_CUDA(cudaMalloc(&n->grads, sizeof(float) * n->P));
                LGD_CHECK_CUDA(cudaMalloc(&n->m, sizeof(float) * n->P));
                LGD_CHECK_CUDA(cudaMalloc(&n->v, sizeof(float) * n->P));
                LGD_CHECK_CUDA(cudaMemsetAsync(n->grads, 0, sizeof(float) * n->P, n->stream));
                LGD_CHECK_CUDA(cudaMemsetAsync(n->m, 0, sizeof(float) * n->P, n->stream));
                LGD_CHECK_CUDA(cudaMemsetAsync(n->v, 0, sizeof(float) * n->P, n->stream));
                LGD_CHECK_CUDA(cudaMalloc(&n->dh, sizeof(float) * C * V));
                LGD_CHECK_CUDA(cudaMalloc(&n->dzb, sizeof(bf16) * C * V));
                LGD_CHECK_CUDA(cudaMalloc(&n->dz4, sizeof(bf16) * 2 * V));
                LGD_CHECK_CUDA(cudaMalloc(&n->d_loss, sizeof(double)));
            }
            n->fast = !n->training && tc_applicable(nx, ny, C);
            if (n->fast) {
                const size_t gbytes = (size_t)batch * (nz + 2) * (ny + 2) * (nx + 2) * 32 * sizeof(bf16);
                for (int i = 0; i < 2; ++i) {
                    LGD_CHECK_CUDA(cudaMalloc(&n->hg[i], gbytes));
                    // channels 24..31 stay zero (layer 1 writes only 0..23)
                    LGD_CHECK_CUDA(cudaMemsetAsync(n->hg[i], 0, gbytes, n->stream));
                    LGD_CHECK_CUDA(cudaMalloc(&n->wtc[i], tc_weight_bytes()));
                }
                LGD_CHECK_CUDA(cudaMalloc(&n->d_err, sizeof(int)));
                LGD_CHECK_CUDA(cudaMemsetAsync(n->d_err, 0, sizeof(int), n->stream));
            }
            repack(*n);
            LGD_CHECK_CUDA(cudaStreamSynchronize(n->stream));
        } catch (...) {
            net_free(*n);
            delete n;
            throw;
        }
        *out = reinterpret_cast<lgd_net *>(n);
    });
}

int lgd_net_destroy(lgd_net *h)
{
    return guard([&] {
        if (!h) return;
        Net& n = net_of(h);
        net_free(n);
        delete &n;
    });
}

int lgd_net_set_params(lgd_net *h, const float *host, size_t count)
{
    return guard([&] {
        Net& n = net_of(h);
        LGD_REQUIRE(host != nullptr && (long long)count == n.P, LGD_ERR_INVALID, "parameter count mismatch");
        LGD_CHECK_CUDA(cudaMemcpyAsync(n.params, host, sizeof(float) * count, cudaMemcpyHostToDevice, n.stream));
        if (n.training) {
            LGD_CHECK_CUDA(cudaMemsetAsync(n.m, 0, sizeof(float) * n.P, n.stream));
            LGD_CHECK_CUDA(cudaMemsetAsync(n.v, 0, sizeof(float) * n.P, n.stream));
            n.t = 0;
        }
        repack(n);
        LGD_CHECK_CUDA(cudaStreamSynchronize(n.stream));
    });
}

int lgd_net_get_params(lgd_net *h, float *host, size_t count)
{
    return guard([&] {
        Net& n = net_of(h);
        LGD_REQUIRE(host != nullptr && (long long)count == n.P, LGD_ERR_INVALID, "parameter count mismatch");
        LGD_CHECK_CUDA(cudaMemcpyAsync(host, n.params, sizeof(float) * count, cudaMemcpyDeviceToHost, n.stream));
        LGD_CHECK_CUDA(cudaStreamSynchronize(n.stream));
    });
}

int lgd_net_get_grads(lgd_net *h, float *host, size_t count)
{
    return guard([&] {
        Net& n = net_of(h);
        LGD_REQUIRE(n.training, LGD_ERR_INVALID, "network was created without training buffers");
        LGD_REQUIRE(host != nullptr && (long long)count == n.P, LGD_ERR_INVALID, "parameter count mismatch");
        LGD_CHECK_CUDA(cudaMemcpyAsync(host, n.grads, sizeof(float) * count, cudaMemcpyDeviceToHost, n.stream));
        LGD_CHECK_CUDA(cudaStreamSynchronize(n.stream));
    });
}

int lgd_net_set_grads(lgd_net *h, const float *host, size_t count)
{
    return guard([&] {
        Net& n = net_of(h);
        LGD_REQUIRE(n.training, LGD_ERR_INVALID, "network was created without training buffers");
        LGD_REQUIRE(host != nullptr && (long long)count == n.P, LGD_ERR_INVALID, "parameter count mismatch");
        LGD_CHECK_CUDA(cudaMemcpyAsync(n.grads, host, sizeof(float) * count, cudaMemcpyHostToDevice, n.stream));
        LGD_CHECK_CUDA(cudaStreamSynchronize(n.stream));
    });
}

int lgd_net_forward(lgd_net *h, const float *d_u, const float *d_kappa, float *d_du)
{
    return guard([&] {
        Net& n = net_of(h);
        LGD_REQUIRE(d_u && d_kappa, LGD_ERR_INVALID, "null input");
        forward(n, d_u, d_kappa, d_du ? d_du : n.du);
        if (d_du && n.training) {
            LGD_CHECK_CUDA(cudaMemcpyAsync(n.du, d_du, sizeof(float) * n.V, cudaMemcpyDeviceToDevice, n.stream));
        }
    });
}

int lgd_net_backward(lgd_net *h, const float *d_target_du, double *loss)
{
    return guard([&] {
        Net& n = net_of(h);
        LGD_REQUIRE(n.training, LGD_ERR_INVALID, "network was created without training buffers");
        LGD_REQUIRE(d_target_du != nullptr, LGD_ERR_INVALID, "null target");
        backward(n, d_target_du, loss);
    });
}

int lgd_net_adam(lgd_net *h, float lr, float beta1, float beta2, float eps)
{
    return guard([&] {
        Net& n = net_of(h);
        LGD_REQUIRE(n.training, LGD_ERR_INVALID, "network was created without training buffers");
        ++n.t;
        const float c1 = 1.f - std::pow(beta1, (float)n.t);
        const float c2 = 1.f - std::pow(beta2, (float)n.t);
        adam_kernel<<<grid_blocks(n.P), 256, 0, n.stream>>>(n.params, n.grads, n.m, n.v, n.P, lr, beta1, beta2, eps, c1, c2);
        check_launch("adam");
        ++n.launches;
        repack(n);
    });
}

int lgd_net_advance(lgd_net *h, float *d_u, const float *d_kappa, int calls)
{
    return guard([&] {
        Net& n = net_of(h);
        LGD_REQUIRE(d_u && d_kappa, LGD_ERR_INVALID, "null input");
        LGD_REQUIRE(calls >= 0, LGD_ERR_INVALID, "negative call count");
        for (int c = 0; c < calls; ++c) {
            if (forward(n, d_u, d_kappa, n.du, true)) continue;
            add_inplace_kernel<<<grid_blocks(n.V), 256, 0, n.stream>>>(d_u, n.du, n.V);
            check_launch("residual update");
            ++n.launches;
        }
    });
}

int lgd_net_synchronize(lgd_net *h)
{
    return guard([&] {
        Net& n = net_of(h);
        LGD_CHECK_CUDA(cudaStreamSynchronize(n.stream));
        if (n.d_err) {
            int e = 0;
            LGD_CHECK_CUDA(cudaMemcpy(&e, n.d_err, sizeof(int), cudaMemcpyDeviceToHost));
            if (e) {
                LGD_CHECK_CUDA(cudaMemset(n.d_err, 0, sizeof(int)));
                throw Error(LGD_ERR_TIMEOUT, "tensor-core convolution gave up waiting for its copies or MMAs");
            }
        }
    });
}

int lgd_net_set_variant(lgd_net *h, int variant)
{
    return guard([&] {
        Net& n = net_of(h);
        LGD_REQUIRE(variant == 0 || variant == 1, LGD_ERR_INVALID, "network variant must be 0 or 1");
        n.variant = variant;
    });
}

int lgd_net_uses_tensor_core_path(lgd_net *h, int *yes)
{
    return guard([&] {
        LGD_REQUIRE(yes != nullptr, LGD_ERR_INVALID, "null output");
        Net& n = net_of(h);
        *yes = (n.fast && n.variant == 0) ? 1 : 0;
    });
}

int lgd_net_stream(lgd_net *h, void **stream)
{
    return guard([&] {
        LGD_REQUIRE(stream != nullptr, LGD_ERR_INVALID, "null output");
        *stream = (void *)net_of(h).stream;
    });
}

int lgd_net_launch_count(lgd_net *h, uint64_t *count)
{
    return guard([&] {
        LGD_REQUIRE(count != nullptr, LGD_ERR_INVALID, "null output");
        *count = net_of(h).launches;
    });
}

}  // extern "C"
