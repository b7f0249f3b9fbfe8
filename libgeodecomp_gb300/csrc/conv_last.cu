// The surrogate's last layer, C -> 1 (C = 24): du = conv3^3(h3) + bias, read
// from the ghosted BF16 activations [batch][nz+2][ny+2][nx+2][32].
//
// A 24 -> 1 convolution is 648 multiply-adds per voxel, too thin for an
// implicit GEMM with the voxels as M (N would be 1).  Instead the 27 taps
// become the N dimension: for every input voxel v of a plane the kernel
// computes the 27 tap products P[t][v] = sum_c W[t][c] h[v][c] with
// mma.sync m16n8k16 (M = voxels, N = 32 taps, K = 32 channels, FP32
// accumulation), parks P in shared memory, and every output voxel then sums
// its 27 entries P[t][v + offset(t)] - nine from each of three consecutive
// input planes, so a CTA marching in z keeps three partial sums in
// registers and finishes one output plane per input plane.
//
// CTA: a 64 x 4 tile of output voxels (one thread each), 256 threads.  Per
// input plane it stages the 66 x 6 halo voxels (64 B each, rows padded to
// 80 B so the ldmatrix row reads are conflict-free; cp.async into two
// buffers, the next plane in flight while this one is used), runs 25 M-tiles x 2
// K-steps x 4 N-tiles of MMAs over the eight warps, and writes P tap-major
// with a row stride of 404 floats (conflict-free stores of the accumulator
// fragments, consecutive voxels for the gather).  HBM traffic: the ghosted
// input once (64 B per voxel) plus the FP32 output (4 B per voxel); the
// halo rows and planes are re-read from L2.
#include <cuda_bf16.h>

#include <algorithm>

#include "lgd_internal.h"

namespace lgd {
namespace sur {
namespace last {

constexpr int TX = 64;                  // output tile
constexpr int TY = 4;
constexpr int HX = TX + 2;              // halo tile
constexpr int HY = TY + 2;
constexpr int HV = HX * HY;             // 396 staged voxels per plane
constexpr int MT = (HV + 15) / 16;      // 25 M-tiles
constexpr int MV = MT * 16;             // 400 rows
constexpr int CP = 32;                  // channels per ghosted voxel
constexpr int VS = 80;                  // staged voxel stride (bytes): 64 + 16 padding
constexpr int PS = 404;                 // P row stride (floats)
constexpr int THREADS = TX * TY;        // 256
constexpr int STAGE_BYTES = MV * VS;    // 32000
constexpr int P_BYTES = 27 * PS * 4;    // 43632
constexpr int SMEM = 2 * STAGE_BYTES + P_BYTES;

__device__ __forceinline__ uint32_t pack2(float lo, float hi)
{
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16(lo)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(hi)) << 16);
}

// du = conv(h) + bias (add_to_u: u += that instead)
__global__ void __launch_bounds__(THREADS, 2)
last_conv_kernel(const __nv_bfloat16 *__restrict__ h, const float *__restrict__ w, const float *__restrict__ bias,
                 float *__restrict__ out, int add_to_u, int nx, int ny, int nz, int zchunk)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float *P = reinterpret_cast<float *>(smem + 2 * STAGE_BYTES);

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const int x0 = blockIdx.x * TX;
    const int y0 = blockIdx.y * TY;
    const int zsplit = (nz + zchunk - 1) / zchunk;
    const int b = blockIdx.z / zsplit;
    const int z0 = (blockIdx.z % zsplit) * zchunk;
    const int z1 = min(z0 + zchunk, nz);
    const long long gnx = nx + 2, gny = ny + 2;

    // B fragments: B[k = channel][n = tap] = W[tap][channel] (zero beyond 24
    // channels and 27 taps); n-tile j, k-step s
    const int g = lane >> 2;
    const int t4 = lane & 3;
    uint32_t bf[4][2][2];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int tap = 8 * j + g;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
#pragma unroll
            for (int hlf = 0; hlf < 2; ++hlf) {
                const int c = 16 * s + 8 * hlf + 2 * t4;
                const float a = (tap < 27 && c < 24) ? __ldg(w + tap * 24 + c) : 0.f;
                const float bb = (tap < 27 && c + 1 < 24) ? __ldg(w + tap * 24 + c + 1) : 0.f;
                bf[j][s][hlf] = pack2(a, bb);
            }
        }
    }
    const float b4 = __ldg(bias);
    // padding rows of the last M-tile: zero once, in both buffers
    for (int i = tid; i < (MV - HV) * VS / 16; i += THREADS) {
        reinterpret_cast<uint4 *>(smem + HV * VS)[i] = make_uint4(0, 0, 0, 0);
        reinterpret_cast<uint4 *>(smem + STAGE_BYTES + HV * VS)[i] = make_uint4(0, 0, 0, 0);
    }
    // input plane zi (ghosted zg = zi + 1) into buffer buf, one cp.async group
    auto stage_plane = [&](int zi, int buf) {
        const long long plane = ((long long)b * (nz + 2) + (zi + 1)) * gny;
        unsigned char *dst = smem + buf * STAGE_BYTES;
        for (int c = tid; c < HV * 4; c += THREADS) {
            const int m = c >> 2;
            const int part = c & 3;
            const int yy = m / HX;
            const int xx = m - yy * HX;
            const __nv_bfloat16 *src = h + ((plane + y0 + yy) * gnx + x0 + xx) * CP + part * 8;
            const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst + m * VS + part * 16);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };

    const int tx = tid % TX;
    const int ty = tid / TX;
    const int mo = (ty + 1) * HX + (tx + 1);        // own voxel in the staged plane
    float acc_prev = 0.f, acc_cur = 0.f;            // outputs z = zi - 1 and z = zi

    // input planes zi = z0 - 1 .. z1 (ghosted zg = zi + 1)
    stage_plane(z0 - 1, 0);
    for (int zi = z0 - 1, it = 0; zi <= z1; ++zi, ++it) {
        const unsigned char *stage = smem + (it & 1) * STAGE_BYTES;
        // the other buffer was last read by the previous plane's MMAs (a
        // barrier ago): refill it with the next plane
        if (zi + 1 <= z1) {
            stage_plane(zi + 1, (it + 1) & 1);
        } else {
            asm volatile("cp.async.commit_group;" ::: "memory");
        }
        asm volatile("cp.async.wait_group 1;" ::: "memory");
        __syncthreads();                            // plane zi staged; the previous P consumed
        for (int mt = warp; mt < MT; mt += THREADS / 32) {
            float d[4][4];
#pragma unroll
            for (int j = 0; j < 4; ++j) d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.f;
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                const int row = mt * 16 + (lane & 7) + 8 * ((lane >> 3) & 1);
                const int col = 16 * s + 8 * (lane >> 4);
                const uint32_t addr = (uint32_t)__cvta_generic_to_shared(stage + row * VS + col * 2);
                uint32_t a0, a1, a2, a3;
                asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
                             : "=r"(a0), "=r"(a1), "=r"(a2), "=r"(a3)
                             : "r"(addr));
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                        "{%0,%1,%2,%3};\n"
                        : "+f"(d[j][0]), "+f"(d[j][1]), "+f"(d[j][2]), "+f"(d[j][3])
                        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(bf[j][s][0]), "r"(bf[j][s][1]));
                }
            }
            // accumulator fragment: rows g, g + 8; columns 2 t4, 2 t4 + 1
            const int m0 = mt * 16 + g;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int tap = 8 * j + 2 * t4;
                if (tap < 27) {
                    P[tap * PS + m0] = d[j][0];
                    P[tap * PS + m0 + 8] = d[j][2];
                }
                if (tap + 1 < 27) {
                    P[(tap + 1) * PS + m0] = d[j][1];
                    P[(tap + 1) * PS + m0 + 8] = d[j][3];
                }
            }
        }
        __syncthreads();
        // taps with dz = -1 reach output zi + 1, dz = 0 output zi, dz = +1
        // output zi - 1; each group of nine in (dy, dx) order
        float part[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            float s = 0.f;
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy) {
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx) {
                    const int tap = q * 9 + (dy + 1) * 3 + (dx + 1);
                    s += P[tap * PS + mo + dy * HX + dx];
                }
            }
            part[q] = s;
        }
        const float done = acc_prev + part[2];      // output zi - 1 is complete
        if (zi - 1 >= z0) {
            const int x = x0 + tx;
            const int y = y0 + ty;
            float *o = out + ((((long long)b * nz + (zi - 1)) * ny + y) * nx + x);
            if (add_to_u) {
                *o += done + b4;
            } else {
                *o = done + b4;
            }
        }
        acc_prev = acc_cur + part[1];
        acc_cur = part[0];
    }
}

}  // namespace last

bool last_conv_applicable(int nx, int ny, int channels)
{
    return channels == 24 && nx % last::TX == 0 && ny % last::TY == 0;
}

// h: ghosted [batch][nz+2][ny+2][nx+2][32] BF16; w: W4[27][24] FP32; out:
// [batch][nz][ny][nx] FP32, written (du) or added to (u += du)
void last_conv(const void *h, const float *w, const float *bias, float *out, bool add_to_u, int nx, int ny, int nz,
               int batch, cudaStream_t stream)
{
    // set up once per device
    static PerDevice<int> setup;
    const int sms = setup.get([] {
        LGD_CHECK_CUDA(cudaFuncSetAttribute(last::last_conv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            last::SMEM));
        int dev = 0, count = 0;
        LGD_CHECK_CUDA(cudaGetDevice(&dev));
        LGD_CHECK_CUDA(cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev));
        return count;
    });
    // z chunks: about four resident CTAs' worth of tiles per SM (two waves
    // of two), chunks of at least 8 planes (two extra input planes each)
    const long long xy = (long long)(nx / last::TX) * (ny / last::TY) * batch;
    const long long want = 4LL * sms;
    int zsplit = (int)std::max(1LL, std::min((long long)std::max(1, nz / 8), (want + xy - 1) / xy));
    const int zchunk = (nz + zsplit - 1) / zsplit;
    zsplit = (nz + zchunk - 1) / zchunk;
    dim3 grid(nx / last::TX, ny / last::TY, batch * zsplit);
    last::last_conv_kernel<<<grid, last::THREADS, last::SMEM, stream>>>(
        (const __nv_bfloat16 *)h, w, bias, out, add_to_u ? 1 : 0, nx, ny, nz, zchunk);
    check_launch("last convolution");
}

}  // namespace sur
}  // namespace lgd
