// Game of Life on uint8 cells (one byte per cell, 0 or 1), Moore radius 1.
//
// Fast path (torus, nx a multiple of 16): SWAR on 32-bit words.  A thread
// owns 16 consecutive cells of one row (one 16-byte load per row for the
// rows above, at and below) plus the 4-byte words left and right of them.
// Column sums of the three rows are formed per byte lane (values <= 3),
// shifted by one byte each way with funnel shifts for the horizontal
// neighbours, and the rule is applied with per-byte equality tests.  Every
// cell costs about five integer operations; traffic is 2 B/cell/step.
//
// Generic path (any size, cube or torus): one thread per cell.
#include "lgd_internal.h"
#include "k_cells.cuh"

namespace lgd {

// per-byte (x == 0) -> 1, else 0, for bytes below 0x80
__device__ __forceinline__ uint32_t bytes_zero(uint32_t x)
{
    return (~((x + 0x7F7F7F7Fu) | x) & 0x80808080u) >> 7;
}

__device__ __forceinline__ uint32_t gol_word(uint32_t vl_word, uint32_t v, uint32_t vr_word, uint32_t mid)
{
    // vl: byte k holds the column sum of cell k-1; vr: of cell k+1
    uint32_t vl = __funnelshift_l(vl_word, v, 8);
    uint32_t vr = __funnelshift_r(v, vr_word, 8);
    uint32_t tot = vl + v + vr;   // includes the cell itself
    uint32_t eq3 = bytes_zero(tot ^ 0x03030303u);
    uint32_t eq4 = bytes_zero(tot ^ 0x04040404u);
    return eq3 | (mid & eq4);
}

__global__ void __launch_bounds__(256)
gol_swar_torus_kernel(const uint8_t *__restrict__ in, uint8_t *__restrict__ out, int nx, int ny, long pitch)
{
    const int words16 = nx >> 4;
    const long long total = (long long)words16 * ny;
    for (long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x; gid < total;
         gid += (long long)gridDim.x * blockDim.x) {
        const int xi = (int)(gid % words16);
        const int y = (int)(gid / words16);
        const int x0 = xi << 4;
        const int yu = (y == 0) ? ny - 1 : y - 1;
        const int yd = (y == ny - 1) ? 0 : y + 1;
        const int xl = (x0 == 0) ? nx - 4 : x0 - 4;
        const int xr = (x0 + 16 == nx) ? 0 : x0 + 16;
        const uint8_t *ru = in + yu * pitch;
        const uint8_t *rm = in + y * pitch;
        const uint8_t *rd = in + yd * pitch;
        const uint4 a = *(const uint4 *)(ru + x0);
        const uint4 b = *(const uint4 *)(rm + x0);
        const uint4 c = *(const uint4 *)(rd + x0);
        const uint32_t vl = *(const uint32_t *)(ru + xl) + *(const uint32_t *)(rm + xl) + *(const uint32_t *)(rd + xl);
        const uint32_t vr = *(const uint32_t *)(ru + xr) + *(const uint32_t *)(rm + xr) + *(const uint32_t *)(rd + xr);
        const uint32_t v0 = a.x + b.x + c.x;
        const uint32_t v1 = a.y + b.y + c.y;
        const uint32_t v2 = a.z + b.z + c.z;
        const uint32_t v3 = a.w + b.w + c.w;
        uint4 o;
        o.x = gol_word(vl, v0, v1, b.x);
        o.y = gol_word(v0, v1, v2, b.y);
        o.z = gol_word(v1, v2, v3, b.z);
        o.w = gol_word(v2, v3, vr, b.w);
        *(uint4 *)(out + y * pitch + x0) = o;
    }
}

__global__ void gol_generic_kernel(View<const uint8_t> in, View<uint8_t> out, int periodic, uint8_t edge)
{
    const long long cells = (long long)in.nx * in.ny;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % in.nx);
        const int y = (int)(i / in.nx);
        int living = 0;
        for (int dy = -1; dy <= 1; ++dy) {
            for (int dx = -1; dx <= 1; ++dx) {
                living += load_bc(in, x + dx, y + dy, 0, periodic, edge);
            }
        }
        const uint8_t self = in.at(x, y, 0);
        out.at(x, y, 0) = gol_rule(self, living - self);
    }
}

void launch_gol(Grid& g, int steps)
{
    LGD_REQUIRE(g.desc.nz == 1, LGD_ERR_INVALID, "Game of Life grids are 2D (nz = 1)");
    const bool swar = ((g.desc.periodic & 3) == 3) && (g.desc.nx % 16 == 0) && (g.pitch_bytes[0] % 16 == 0);
    const long pitch = (long)g.pitch_bytes[0];
    for (int s = 0; s < steps; ++s) {
        const uint8_t *in = (const uint8_t *)g.m[0].buf[g.cur];
        uint8_t *out = (uint8_t *)g.m[0].buf[1 - g.cur];
        if (swar) {
            const long long work = (long long)(g.desc.nx / 16) * g.desc.ny;
            long long blocks = (work + 255) / 256;
            if (blocks > 152LL * 64) blocks = 152LL * 64;
            gol_swar_torus_kernel<<<(unsigned)blocks, 256, 0, g.stream>>>(in, out, g.desc.nx, g.desc.ny, pitch);
        } else {
            View<const uint8_t> vi;
            vi.p = in;
            vi.pitch = pitch;
            vi.nx = g.desc.nx;
            vi.ny = g.desc.ny;
            vi.nz = 1;
            View<uint8_t> vo;
            vo.p = out;
            vo.pitch = pitch;
            vo.nx = g.desc.nx;
            vo.ny = g.desc.ny;
            vo.nz = 1;
            const long long cells = (long long)g.desc.nx * g.desc.ny;
            long long blocks = (cells + 255) / 256;
            if (blocks > 152LL * 64) blocks = 152LL * 64;
            gol_generic_kernel<<<(unsigned)blocks, 256, 0, g.stream>>>(vi, vo, g.desc.periodic, (uint8_t)g.desc.edge[0]);
        }
        check_launch("game of life");
        ++g.launches;
        g.cur = 1 - g.cur;
    }
}

}  // namespace lgd
