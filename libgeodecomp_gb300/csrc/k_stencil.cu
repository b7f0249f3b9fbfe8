// Whole-grid 3D seven-point kernels (Jacobi-7 in FP64 / FP32 / 64-bit
// fixed point, variable-coefficient diffusion).
//
// 2.5D blocking: a CTA owns a BX x BY column of cells and marches along z.
// The plane being updated sits in shared memory with a one-cell halo (for
// the four in-plane neighbours); the planes below and above stay in
// registers, so every cell is read from memory once per plane sweep plus
// the halo re-reads, which hit L2.  Algorithmic traffic: one read and one
// write per cell and step (16 B/cell for FP64, 8 B for FP32; varcoef adds
// the coefficient read).
#include <algorithm>

#include "lgd_internal.h"
#include "k_cells.cuh"

namespace lgd {

static const int SBX = 32;
static const int SBY = 8;

// Value at arbitrary (x, y, z) within one grid extent outside the box:
// periodic axes wrap by modulo, the others return the edge value.
template<typename T>
__device__ __forceinline__ T load_any(const View<const T>& v, int x, int y, int z, int periodic, T edge)
{
    if ((unsigned)x >= (unsigned)v.nx) {
        if (!(periodic & 1)) return edge;
        x = ((x % v.nx) + v.nx) % v.nx;
    }
    if ((unsigned)y >= (unsigned)v.ny) {
        if (!(periodic & 2)) return edge;
        y = ((y % v.ny) + v.ny) % v.ny;
    }
    if ((unsigned)z >= (unsigned)v.nz) {
        if (!(periodic & 4)) return edge;
        z = ((z % v.nz) + v.nz) % v.nz;
    }
    return v.at(x, y, z);
}

template<typename CELL>
__global__ void __launch_bounds__(SBX * SBY)
jacobi7_zmarch_kernel(View<const typename CELL::T> in, View<typename CELL::T> out, int periodic,
                      typename CELL::T edge, int zchunk)
{
    typedef typename CELL::T T;
    __shared__ T tile[SBY + 2][SBX + 2];
    const int tx = threadIdx.x;
    const int ty = threadIdx.y;
    const int x = blockIdx.x * SBX + tx;
    const int y = blockIdx.y * SBY + ty;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, in.nz);
    const bool inside = (x < in.nx) && (y < in.ny);

    T below = load_any(in, x, y, z0 - 1, periodic, edge);
    T cur = load_any(in, x, y, z0, periodic, edge);
    for (int z = z0; z < z1; ++z) {
        T above = (inside && z + 1 < in.nz) ? in.at(x, y, z + 1) : load_any(in, x, y, z + 1, periodic, edge);
        tile[ty + 1][tx + 1] = cur;
        if (tx == 0) tile[ty + 1][0] = load_any(in, x - 1, y, z, periodic, edge);
        if (tx == SBX - 1) tile[ty + 1][SBX + 1] = load_any(in, x + 1, y, z, periodic, edge);
        if (ty == 0) tile[0][tx + 1] = load_any(in, x, y - 1, z, periodic, edge);
        if (ty == SBY - 1) tile[SBY + 1][tx + 1] = load_any(in, x, y + 1, z, periodic, edge);
        __syncthreads();
        if (inside) {
            out.at(x, y, z) = CELL::apply(cur, tile[ty][tx + 1], tile[ty + 2][tx + 1], tile[ty + 1][tx + 2],
                                          tile[ty + 1][tx], above, below);
        }
        __syncthreads();
        below = cur;
        cur = above;
    }
}

// Register-column variant: a warp owns 32 consecutive x and TY consecutive
// rows and marches along z.  x-neighbours come from the neighbouring lanes
// (shuffles; lanes 0 and 31 load the one cell beyond the warp), y-neighbours
// from the thread's own column except the two rows just outside it, z
// neighbours from the registers of the previous and next plane.  No shared
// memory and no barriers; per plane a thread issues TY coalesced loads of
// the next plane plus two rows of halo (L2 hits).
template<typename T>
__device__ __forceinline__ T shfl_down1(T v)
{
    return __shfl_down_sync(0xffffffffu, v, 1);
}

template<typename T>
__device__ __forceinline__ T shfl_up1(T v)
{
    return __shfl_up_sync(0xffffffffu, v, 1);
}

template<typename CELL, int TY>
__global__ void __launch_bounds__(128)
jacobi7_zcol_kernel(View<const typename CELL::T> in, View<typename CELL::T> out, int periodic,
                    typename CELL::T edge, int zchunk)
{
    typedef typename CELL::T T;
    const int lane = threadIdx.x;
    const int x = blockIdx.x * 32 + lane;
    const int y0 = (blockIdx.y * blockDim.y + threadIdx.y) * TY;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, in.nz);
    if (y0 >= in.ny) return;   // whole warp leaves together (y0 is warp-uniform)
    const bool xin = x < in.nx;

    T bel[TY], cur[TY], abv[TY];
#pragma unroll
    for (int j = 0; j < TY; ++j) {
        bel[j] = load_any(in, x, y0 + j, z0 - 1, periodic, edge);
        cur[j] = load_any(in, x, y0 + j, z0, periodic, edge);
    }
    for (int z = z0; z < z1; ++z) {
#pragma unroll
        for (int j = 0; j < TY; ++j) {
            const int y = y0 + j;
            abv[j] = (xin && y < in.ny && z + 1 < in.nz) ? in.at(x, y, z + 1) : load_any(in, x, y, z + 1, periodic, edge);
        }
        const T hn = load_any(in, x, y0 - 1, z, periodic, edge);
        const T hs = load_any(in, x, y0 + TY, z, periodic, edge);
#pragma unroll
        for (int j = 0; j < TY; ++j) {
            const int y = y0 + j;
            T e = shfl_down1(cur[j]);
            T w = shfl_up1(cur[j]);
            if (lane == 31) e = load_any(in, x + 1, y, z, periodic, edge);
            if (lane == 0) w = load_any(in, x - 1, y, z, periodic, edge);
            const T n = (j == 0) ? hn : cur[j - 1];
            const T s = (j == TY - 1) ? hs : cur[j + 1];
            if (xin && y < in.ny) {
                out.at(x, y, z) = CELL::apply(cur[j], n, s, e, w, abv[j], bel[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < TY; ++j) {
            bel[j] = cur[j];
            cur[j] = abv[j];
        }
    }
}

// Pair variant (default): like the register-column kernel, but every lane
// owns two neighbouring x cells (one 16-byte load or store per row and
// plane for 8-byte cells), so half of the x-neighbours are in the thread's
// own registers; warps whose 64 x 4 footprint plus its one-cell rim lies
// inside the grid take a path without any boundary test, and the z loop is
// unrolled three times so the below / centre / above planes rotate through
// register names instead of being copied.
template<typename T>
struct Pair {
    T a, b;
};

template<typename T>
__device__ __forceinline__ Pair<T> ld_pair(const T *p)
{
    Pair<T> r;
    if (sizeof(T) == 8) {
        const longlong2 v = *reinterpret_cast<const longlong2 *>(p);
        r.a = *reinterpret_cast<const T *>(&v.x);
        r.b = *reinterpret_cast<const T *>(&v.y);
    } else {
        const int2 v = *reinterpret_cast<const int2 *>(p);
        r.a = *reinterpret_cast<const T *>(&v.x);
        r.b = *reinterpret_cast<const T *>(&v.y);
    }
    return r;
}

template<typename T>
__device__ __forceinline__ void st_pair(T *p, T a, T b)
{
    if (sizeof(T) == 8) {
        longlong2 v;
        v.x = *reinterpret_cast<const long long *>(&a);
        v.y = *reinterpret_cast<const long long *>(&b);
        *reinterpret_cast<longlong2 *>(p) = v;
    } else {
        int2 v;
        v.x = *reinterpret_cast<const int *>(&a);
        v.y = *reinterpret_cast<const int *>(&b);
        *reinterpret_cast<int2 *>(p) = v;
    }
}

// Everything a warp of the pair kernel needs to address its footprint: the
// warp owns x in [x0 - 2 lane, + 64), rows [y0, y0 + TY) and all of them
// exist.  Rows and planes outside the grid are either wrapped (periodic
// axis) or replaced by the edge value; those decisions are uniform across
// the warp.  Only lanes 0 and 31 look one cell beyond the warp in x.
template<typename T, int TY>
struct PairFrame {
    const T *in;
    T *out;
    long pitch;
    long plane;
    int nx, ny, nz;
    int periodic;
    int x0, y0, lane;
    T edge;

    // row y of plane z of the input at column x0, or null for "edge"
    __device__ __forceinline__ const T *row(int y, int z) const
    {
        if (y < 0 || y >= ny) {
            if (!(periodic & 2)) return nullptr;
            y = (y < 0) ? y + ny : y - ny;
        }
        if (z < 0 || z >= nz) {
            if (!(periodic & 4)) return nullptr;
            z = (z < 0) ? z + nz : z - nz;
        }
        return in + (long)z * plane + (long)y * pitch + x0;
    }

    __device__ __forceinline__ Pair<T> pair_at(const T *r) const
    {
        if (r) return ld_pair(r);
        Pair<T> e;
        e.a = edge;
        e.b = edge;
        return e;
    }

    __device__ __forceinline__ void load_plane(int z, Pair<T> (&P)[TY]) const
    {
        const T *r = row(y0, z);   // the TY rows are all inside in y
#pragma unroll
        for (int j = 0; j < TY; ++j) P[j] = pair_at(r ? r + j * pitch : nullptr);
    }

    // cell x0 - 1 (lane 0) or x0 + 2 (lane 31) of row r (r points at x0)
    __device__ __forceinline__ T west(const T *r) const
    {
        if (x0 >= 1) return r[-1];
        return (periodic & 1) ? r[nx - 1 - x0] : edge;
    }

    __device__ __forceinline__ T east(const T *r) const
    {
        if (x0 + 2 < nx) return r[2];
        return (periodic & 1) ? r[-x0] : edge;
    }
};

// Plane z: B / C / A hold planes z - 1, z, z + 1; N receives plane z + 2
// when load_next is set.
template<typename CELL, int TY>
__device__ __forceinline__ void pair_plane(const PairFrame<typename CELL::T, TY>& f, int z, bool load_next,
                                           const Pair<typename CELL::T> (&B)[TY], const Pair<typename CELL::T> (&C)[TY],
                                           const Pair<typename CELL::T> (&A)[TY], Pair<typename CELL::T> (&N)[TY])
{
    typedef typename CELL::T T;
    if (load_next) f.load_plane(z + 2, N);
    const T *r = f.in + (long)z * f.plane + (long)f.y0 * f.pitch + f.x0;
    const Pair<T> hn = f.pair_at(f.row(f.y0 - 1, z));
    const Pair<T> hs = f.pair_at(f.row(f.y0 + TY, z));
    T *o = f.out + (long)z * f.plane + (long)f.y0 * f.pitch + f.x0;
#pragma unroll
    for (int j = 0; j < TY; ++j) {
        T w0 = shfl_up1(C[j].b);
        T e1 = shfl_down1(C[j].a);
        if (f.lane == 0) w0 = f.west(r + j * f.pitch);
        if (f.lane == 31) e1 = f.east(r + j * f.pitch);
        const Pair<T> n = (j == 0) ? hn : C[j - 1];
        const Pair<T> s = (j == TY - 1) ? hs : C[j + 1];
        const T o0 = CELL::apply(C[j].a, n.a, s.a, C[j].b, w0, A[j].a, B[j].a);
        const T o1 = CELL::apply(C[j].b, n.b, s.b, e1, C[j].a, A[j].b, B[j].b);
        st_pair(o + j * f.pitch, o0, o1);
    }
}

template<typename CELL, int TY>
__global__ void __launch_bounds__(64)
jacobi7_pair_kernel(View<const typename CELL::T> in, View<typename CELL::T> out, int periodic,
                    typename CELL::T edge, int zchunk)
{
    typedef typename CELL::T T;
    const int lane = threadIdx.x;
    const int xb = blockIdx.x * 64;
    const int x0 = xb + 2 * lane;
    const int y0 = (blockIdx.y * blockDim.y + threadIdx.y) * TY;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, in.nz);
    if (y0 >= in.ny) return;   // warp-uniform

    if (xb + 64 <= in.nx && y0 + TY <= in.ny) {
        // full warp footprint: vector path
        PairFrame<T, TY> f;
        f.in = in.p;
        f.out = out.p;
        f.pitch = in.pitch;
        f.plane = in.pitch * in.ny;
        f.nx = in.nx;
        f.ny = in.ny;
        f.nz = in.nz;
        f.periodic = periodic;
        f.x0 = x0;
        f.y0 = y0;
        f.lane = lane;
        f.edge = edge;
        Pair<T> P0[TY], P1[TY], P2[TY], P3[TY];
        f.load_plane(z0 - 1, P0);
        f.load_plane(z0, P1);
        f.load_plane(z0 + 1, P2);
        // four register sets rotate: plane z uses (below, centre, above) and
        // fills the fourth with plane z + 2, which plane z + 1 needs
        for (int z = z0; z < z1; z += 4) {
            pair_plane<CELL, TY>(f, z, z + 1 < z1, P0, P1, P2, P3);
            if (z + 1 >= z1) break;
            pair_plane<CELL, TY>(f, z + 1, z + 2 < z1, P1, P2, P3, P0);
            if (z + 2 >= z1) break;
            pair_plane<CELL, TY>(f, z + 2, z + 3 < z1, P2, P3, P0, P1);
            if (z + 3 >= z1) break;
            pair_plane<CELL, TY>(f, z + 3, z + 4 < z1, P3, P0, P1, P2);
        }
        return;
    }

    // partial footprint (grid edge in x or y): per-cell loads
    const bool xin0 = x0 < in.nx;
    const bool xin1 = x0 + 1 < in.nx;
    for (int z = z0; z < z1; ++z) {
#pragma unroll
        for (int j = 0; j < TY; ++j) {
            const int y = y0 + j;
            const T c0 = load_any(in, x0, y, z, periodic, edge);
            const T c1 = load_any(in, x0 + 1, y, z, periodic, edge);
            T w0 = shfl_up1(c1);
            T e1 = shfl_down1(c0);
            if (lane == 0) w0 = load_any(in, x0 - 1, y, z, periodic, edge);
            if (lane == 31) e1 = load_any(in, x0 + 2, y, z, periodic, edge);
            if (xin0 && y < in.ny) {
                out.at(x0, y, z) = CELL::apply(c0, load_any(in, x0, y - 1, z, periodic, edge),
                                               load_any(in, x0, y + 1, z, periodic, edge), c1, w0,
                                               load_any(in, x0, y, z + 1, periodic, edge),
                                               load_any(in, x0, y, z - 1, periodic, edge));
            }
            if (xin1 && y < in.ny) {
                out.at(x0 + 1, y, z) = CELL::apply(c1, load_any(in, x0 + 1, y - 1, z, periodic, edge),
                                                   load_any(in, x0 + 1, y + 1, z, periodic, edge), e1, c0,
                                                   load_any(in, x0 + 1, y, z + 1, periodic, edge),
                                                   load_any(in, x0 + 1, y, z - 1, periodic, edge));
            }
        }
    }
}

template<typename R>
__global__ void __launch_bounds__(SBX * SBY)
varcoef_zmarch_kernel(View<const R> u, View<const R> k, View<R> out, int periodic, R edgeU, R edgeK, int zchunk)
{
    __shared__ R tu[SBY + 2][SBX + 2];
    __shared__ R tk[SBY + 2][SBX + 2];
    const int tx = threadIdx.x;
    const int ty = threadIdx.y;
    const int x = blockIdx.x * SBX + tx;
    const int y = blockIdx.y * SBY + ty;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, u.nz);
    const bool inside = (x < u.nx) && (y < u.ny);

    R ub = load_any(u, x, y, z0 - 1, periodic, edgeU);
    R kb = load_any(k, x, y, z0 - 1, periodic, edgeK);
    R uc = load_any(u, x, y, z0, periodic, edgeU);
    R kc = load_any(k, x, y, z0, periodic, edgeK);
    for (int z = z0; z < z1; ++z) {
        R ut = load_any(u, x, y, z + 1, periodic, edgeU);
        R kt = load_any(k, x, y, z + 1, periodic, edgeK);
        tu[ty + 1][tx + 1] = uc;
        tk[ty + 1][tx + 1] = kc;
        if (tx == 0) {
            tu[ty + 1][0] = load_any(u, x - 1, y, z, periodic, edgeU);
            tk[ty + 1][0] = load_any(k, x - 1, y, z, periodic, edgeK);
        }
        if (tx == SBX - 1) {
            tu[ty + 1][SBX + 1] = load_any(u, x + 1, y, z, periodic, edgeU);
            tk[ty + 1][SBX + 1] = load_any(k, x + 1, y, z, periodic, edgeK);
        }
        if (ty == 0) {
            tu[0][tx + 1] = load_any(u, x, y - 1, z, periodic, edgeU);
            tk[0][tx + 1] = load_any(k, x, y - 1, z, periodic, edgeK);
        }
        if (ty == SBY - 1) {
            tu[SBY + 1][tx + 1] = load_any(u, x, y + 1, z, periodic, edgeU);
            tk[SBY + 1][tx + 1] = load_any(k, x, y + 1, z, periodic, edgeK);
        }
        __syncthreads();
        if (inside) {
            out.at(x, y, z) = VarCoef<R>::apply(
                uc, kc,
                tu[ty + 1][tx], tk[ty + 1][tx],            // -x
                tu[ty + 1][tx + 2], tk[ty + 1][tx + 2],    // +x
                tu[ty][tx + 1], tk[ty][tx + 1],            // -y
                tu[ty + 2][tx + 1], tk[ty + 2][tx + 1],    // +y
                ub, kb,                                    // -z
                ut, kt);                                   // +z
        }
        __syncthreads();
        ub = uc;
        kb = kc;
        uc = ut;
        kc = kt;
    }
}

template<typename T>
static View<T> mview(Grid& g, int member, int which)
{
    View<T> v;
    v.p = (T *)g.m[member].buf[g.m[member].is_static ? 0 : (which ? 1 - g.cur : g.cur)];
    v.pitch = (long)(g.pitch_bytes[member] / sizeof(T));
    v.nx = g.desc.nx;
    v.ny = g.desc.ny;
    v.nz = g.desc.nz;
    return v;
}

template<typename T>
static View<const T> cmview(Grid& g, int member, int which)
{
    View<T> v = mview<T>(g, member, which);
    View<const T> c;
    c.p = v.p;
    c.pitch = v.pitch;
    c.nx = v.nx;
    c.ny = v.ny;
    c.nz = v.nz;
    return c;
}

static dim3 zmarch_grid(const Grid& g, int *zchunk)
{
    const int bx = (g.desc.nx + SBX - 1) / SBX;
    const int by = (g.desc.ny + SBY - 1) / SBY;
    const long long xy = (long long)bx * by;
    // enough CTAs to fill 152 SMs several times over, z chunks of >= 8 planes
    int zsplit = (int)((152LL * 8 + xy - 1) / xy);
    zsplit = max(1, min(zsplit, (g.desc.nz + 7) / 8));
    *zchunk = (g.desc.nz + zsplit - 1) / zsplit;
    zsplit = (g.desc.nz + *zchunk - 1) / *zchunk;
    return dim3(bx, by, zsplit);
}

long long fix_edge(const Grid& g);

static const int ZCOL_TY = 4;   // rows per warp
static const int ZCOL_WY = 4;   // warps per CTA

static dim3 zcol_grid(const Grid& g, int *zchunk)
{
    const int bx = (g.desc.nx + 31) / 32;
    const int by = (g.desc.ny + ZCOL_TY * ZCOL_WY - 1) / (ZCOL_TY * ZCOL_WY);
    const long long xy = (long long)bx * by;
    // about 16 resident CTAs of 128 threads per SM, several waves deep
    int zsplit = (int)((152LL * 16 * 2 + xy - 1) / xy);
    zsplit = max(1, min(zsplit, (g.desc.nz + 15) / 16));
    *zchunk = (g.desc.nz + zsplit - 1) / zsplit;
    zsplit = (g.desc.nz + *zchunk - 1) / *zchunk;
    return dim3(bx, by, zsplit);
}

static const int PAIR_TY = 4;   // rows per warp
static const int PAIR_WY = 2;   // warps per CTA

static dim3 pair_grid(const Grid& g, int ty, int *zchunk)
{
    const int bx = (g.desc.nx + 63) / 64;
    const int by = (g.desc.ny + ty * PAIR_WY - 1) / (ty * PAIR_WY);
    const long long xy = (long long)bx * by;
    // about 24 resident CTAs of 64 threads per SM, two waves
    int zsplit = (int)((152LL * 24 * 2 + xy - 1) / xy);
    zsplit = max(1, min(zsplit, (g.desc.nz + 15) / 16));
    *zchunk = (g.desc.nz + zsplit - 1) / zsplit;
    zsplit = (g.desc.nz + *zchunk - 1) / *zchunk;
    return dim3(bx, by, zsplit);
}

template<typename CELL>
static void launch_zcol(Grid& g, View<const typename CELL::T> in, View<typename CELL::T> out, typename CELL::T edge)
{
    int zchunk = 1;
    if (g.variant == 2) {
        const dim3 grid = zcol_grid(g, &zchunk);
        jacobi7_zcol_kernel<CELL, ZCOL_TY><<<grid, dim3(32, ZCOL_WY), 0, g.stream>>>(in, out, g.desc.periodic, edge,
                                                                                    zchunk);
    } else if (g.variant == 3) {
        const dim3 grid = pair_grid(g, 8, &zchunk);
        jacobi7_pair_kernel<CELL, 8><<<grid, dim3(32, PAIR_WY), 0, g.stream>>>(in, out, g.desc.periodic, edge, zchunk);
    } else if (g.variant == 4) {
        const dim3 grid = pair_grid(g, 2, &zchunk);
        jacobi7_pair_kernel<CELL, 2><<<grid, dim3(32, PAIR_WY), 0, g.stream>>>(in, out, g.desc.periodic, edge, zchunk);
    } else {
        const dim3 grid = pair_grid(g, PAIR_TY, &zchunk);
        jacobi7_pair_kernel<CELL, PAIR_TY><<<grid, dim3(32, PAIR_WY), 0, g.stream>>>(in, out, g.desc.periodic, edge,
                                                                                    zchunk);
    }
}

void launch_jacobi7(Grid& g, int steps)
{
    if ((g.variant == 0 || g.variant == 6) && tma_applicable(g)) {
        // temporal blocking: passes of `depth` steps, then one shorter pass
        // for the remainder (single steps go through the one-step kernel)
        int depth = (g.time_block == 0) ? (tb_applicable(g) ? tb_default_depth(g) : 1) : g.time_block;
        if (tb_applicable(g)) depth = std::min(depth, tb_max_depth(g));
        if (depth > 1 && tb_applicable(g)) {
            while (steps >= 2) {
                const int d = steps >= depth ? depth : steps;
                launch_jacobi7_tb(g, d, g.tb_shape);
                steps -= d;
            }
        }
        for (int s = 0; s < steps; ++s) launch_jacobi7_tma(g);
        return;
    }
    if (g.variant != 1) {
        for (int s = 0; s < steps; ++s) {
            switch (g.desc.cell) {
            case LGD_CELL_JACOBI7_F64:
                launch_zcol<Jacobi7F64>(g, cmview<double>(g, 0, 0), mview<double>(g, 0, 1), g.desc.edge[0]);
                break;
            case LGD_CELL_JACOBI7_F32:
                launch_zcol<Jacobi7F32>(g, cmview<float>(g, 0, 0), mview<float>(g, 0, 1), (float)g.desc.edge[0]);
                break;
            case LGD_CELL_JACOBI7_F64_FIX:
                launch_zcol<Jacobi7Fix>(g, cmview<long long>(g, 0, 0), mview<long long>(g, 0, 1), fix_edge(g));
                break;
            default:
                throw Error(LGD_ERR_UNSUPPORTED, "not a Jacobi cell");
            }
            check_launch("jacobi7");
            ++g.launches;
            g.cur = 1 - g.cur;
        }
        return;
    }
    int zchunk = 1;
    dim3 grid = zmarch_grid(g, &zchunk);
    dim3 block(SBX, SBY);
    for (int s = 0; s < steps; ++s) {
        switch (g.desc.cell) {
        case LGD_CELL_JACOBI7_F64:
            jacobi7_zmarch_kernel<Jacobi7F64><<<grid, block, 0, g.stream>>>(
                cmview<double>(g, 0, 0), mview<double>(g, 0, 1), g.desc.periodic, g.desc.edge[0], zchunk);
            break;
        case LGD_CELL_JACOBI7_F32:
            jacobi7_zmarch_kernel<Jacobi7F32><<<grid, block, 0, g.stream>>>(
                cmview<float>(g, 0, 0), mview<float>(g, 0, 1), g.desc.periodic, (float)g.desc.edge[0], zchunk);
            break;
        case LGD_CELL_JACOBI7_F64_FIX:
            jacobi7_zmarch_kernel<Jacobi7Fix><<<grid, block, 0, g.stream>>>(
                cmview<long long>(g, 0, 0), mview<long long>(g, 0, 1), g.desc.periodic, fix_edge(g), zchunk);
            break;
        default:
            throw Error(LGD_ERR_UNSUPPORTED, "not a Jacobi cell");
        }
        check_launch("jacobi7");
        ++g.launches;
        g.cur = 1 - g.cur;
    }
}

// Variable-coefficient diffusion with the pair kernel's scheme (two x cells
// per lane, TY rows per warp, z rotation through four register sets,
// warp-uniform wrap / edge decisions), carrying u and k.  Traffic: u read,
// k read, u written: 12 B per cell for FP32.
template<typename R, int TY>
__device__ __forceinline__ void varcoef_pair_plane(const PairFrame<R, TY>& fu, const PairFrame<R, TY>& fk, int z,
                                                   bool load_next, const Pair<R> (&UB)[TY], const Pair<R> (&UC)[TY],
                                                   const Pair<R> (&UA)[TY], Pair<R> (&UN)[TY], const Pair<R> (&KB)[TY],
                                                   const Pair<R> (&KC)[TY], const Pair<R> (&KA)[TY], Pair<R> (&KN)[TY])
{
    if (load_next) {
        fu.load_plane(z + 2, UN);
        fk.load_plane(z + 2, KN);
    }
    const long roff = (long)z * fu.plane + (long)fu.y0 * fu.pitch + fu.x0;
    const R *ru = fu.in + roff;
    const R *rk = fk.in + roff;
    const Pair<R> hnu = fu.pair_at(fu.row(fu.y0 - 1, z));
    const Pair<R> hsu = fu.pair_at(fu.row(fu.y0 + TY, z));
    const Pair<R> hnk = fk.pair_at(fk.row(fk.y0 - 1, z));
    const Pair<R> hsk = fk.pair_at(fk.row(fk.y0 + TY, z));
    R *o = fu.out + roff;
#pragma unroll
    for (int j = 0; j < TY; ++j) {
        R wu = shfl_up1(UC[j].b);
        R eu = shfl_down1(UC[j].a);
        R wk = shfl_up1(KC[j].b);
        R ek = shfl_down1(KC[j].a);
        if (fu.lane == 0) {
            wu = fu.west(ru + j * fu.pitch);
            wk = fk.west(rk + j * fk.pitch);
        }
        if (fu.lane == 31) {
            eu = fu.east(ru + j * fu.pitch);
            ek = fk.east(rk + j * fk.pitch);
        }
        const Pair<R> nu = (j == 0) ? hnu : UC[j - 1];
        const Pair<R> su = (j == TY - 1) ? hsu : UC[j + 1];
        const Pair<R> nk = (j == 0) ? hnk : KC[j - 1];
        const Pair<R> sk = (j == TY - 1) ? hsk : KC[j + 1];
        const R o0 = VarCoef<R>::apply(UC[j].a, KC[j].a, wu, wk, UC[j].b, KC[j].b, nu.a, nk.a, su.a, sk.a, UB[j].a, KB[j].a,
                                       UA[j].a, KA[j].a);
        const R o1 = VarCoef<R>::apply(UC[j].b, KC[j].b, UC[j].a, KC[j].a, eu, ek, nu.b, nk.b, su.b, sk.b, UB[j].b, KB[j].b,
                                       UA[j].b, KA[j].b);
        st_pair(o + j * fu.pitch, o0, o1);
    }
}

template<typename R, int TY>
__global__ void __launch_bounds__(64)
varcoef_pair_kernel(View<const R> u, View<const R> k, View<R> out, int periodic, R edgeU, R edgeK, int zchunk)
{
    const int lane = threadIdx.x;
    const int xb = blockIdx.x * 64;
    const int x0 = xb + 2 * lane;
    const int y0 = (blockIdx.y * blockDim.y + threadIdx.y) * TY;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, u.nz);
    if (y0 >= u.ny) return;   // warp-uniform

    if (xb + 64 <= u.nx && y0 + TY <= u.ny) {
        PairFrame<R, TY> fu, fk;
        fu.in = u.p;
        fu.out = out.p;
        fu.pitch = u.pitch;
        fu.plane = u.pitch * u.ny;
        fu.nx = u.nx;
        fu.ny = u.ny;
        fu.nz = u.nz;
        fu.periodic = periodic;
        fu.x0 = x0;
        fu.y0 = y0;
        fu.lane = lane;
        fu.edge = edgeU;
        fk = fu;
        fk.in = k.p;
        fk.edge = edgeK;
        Pair<R> U0[TY], U1[TY], U2[TY], U3[TY], K0[TY], K1[TY], K2[TY], K3[TY];
        fu.load_plane(z0 - 1, U0);
        fu.load_plane(z0, U1);
        fu.load_plane(z0 + 1, U2);
        fk.load_plane(z0 - 1, K0);
        fk.load_plane(z0, K1);
        fk.load_plane(z0 + 1, K2);
        for (int z = z0; z < z1; z += 4) {
            varcoef_pair_plane<R, TY>(fu, fk, z, z + 1 < z1, U0, U1, U2, U3, K0, K1, K2, K3);
            if (z + 1 >= z1) break;
            varcoef_pair_plane<R, TY>(fu, fk, z + 1, z + 2 < z1, U1, U2, U3, U0, K1, K2, K3, K0);
            if (z + 2 >= z1) break;
            varcoef_pair_plane<R, TY>(fu, fk, z + 2, z + 3 < z1, U2, U3, U0, U1, K2, K3, K0, K1);
            if (z + 3 >= z1) break;
            varcoef_pair_plane<R, TY>(fu, fk, z + 3, z + 4 < z1, U3, U0, U1, U2, K3, K0, K1, K2);
        }
        return;
    }

    // partial footprint: per-cell loads
    for (int z = z0; z < z1; ++z) {
#pragma unroll
        for (int j = 0; j < TY; ++j) {
            const int y = y0 + j;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int x = x0 + h;
                if (x < u.nx && y < u.ny) {
                    out.at(x, y, z) = VarCoef<R>::apply(
                        u.at(x, y, z), k.at(x, y, z),
                        load_any(u, x - 1, y, z, periodic, edgeU), load_any(k, x - 1, y, z, periodic, edgeK),
                        load_any(u, x + 1, y, z, periodic, edgeU), load_any(k, x + 1, y, z, periodic, edgeK),
                        load_any(u, x, y - 1, z, periodic, edgeU), load_any(k, x, y - 1, z, periodic, edgeK),
                        load_any(u, x, y + 1, z, periodic, edgeU), load_any(k, x, y + 1, z, periodic, edgeK),
                        load_any(u, x, y, z - 1, periodic, edgeU), load_any(k, x, y, z - 1, periodic, edgeK),
                        load_any(u, x, y, z + 1, periodic, edgeU), load_any(k, x, y, z + 1, periodic, edgeK));
                }
            }
        }
    }
}

void launch_varcoef(Grid& g, int steps)
{
    // default: the TMA kernel for FP32 cells (HBM-bound); FP64 cells are
    // bound by the FP64 rate, where the register kernel measured faster
    const bool tma = (g.variant == 6) || (g.variant == 0 && g.desc.cell == LGD_CELL_VARCOEF_F32);
    if (tma && varcoef_tma_applicable(g)) {
        for (int s = 0; s < steps; ++s) launch_varcoef_tma(g);
        return;
    }
    if (g.variant != 1) {
        // two rows per warp: u and k both rotate through four planes
        const int VC_TY = 2;
        int zchunk = 1;
        const dim3 grid = pair_grid(g, VC_TY, &zchunk);
        for (int s = 0; s < steps; ++s) {
            if (g.desc.cell == LGD_CELL_VARCOEF_F32) {
                varcoef_pair_kernel<float, VC_TY><<<grid, dim3(32, PAIR_WY), 0, g.stream>>>(
                    cmview<float>(g, 0, 0), cmview<float>(g, 1, 0), mview<float>(g, 0, 1), g.desc.periodic,
                    (float)g.desc.edge[0], (float)g.desc.edge[1], zchunk);
            } else {
                varcoef_pair_kernel<double, VC_TY><<<grid, dim3(32, PAIR_WY), 0, g.stream>>>(
                    cmview<double>(g, 0, 0), cmview<double>(g, 1, 0), mview<double>(g, 0, 1), g.desc.periodic,
                    g.desc.edge[0], g.desc.edge[1], zchunk);
            }
            check_launch("varcoef");
            ++g.launches;
            g.cur = 1 - g.cur;
        }
        return;
    }
    int zchunk = 1;
    dim3 grid = zmarch_grid(g, &zchunk);
    dim3 block(SBX, SBY);
    for (int s = 0; s < steps; ++s) {
        if (g.desc.cell == LGD_CELL_VARCOEF_F32) {
            varcoef_zmarch_kernel<float><<<grid, block, 0, g.stream>>>(
                cmview<float>(g, 0, 0), cmview<float>(g, 1, 0), mview<float>(g, 0, 1), g.desc.periodic,
                (float)g.desc.edge[0], (float)g.desc.edge[1], zchunk);
        } else {
            varcoef_zmarch_kernel<double><<<grid, block, 0, g.stream>>>(
                cmview<double>(g, 0, 0), cmview<double>(g, 1, 0), mview<double>(g, 0, 1), g.desc.periodic,
                g.desc.edge[0], g.desc.edge[1], zchunk);
        }
        check_launch("varcoef");
        ++g.launches;
        g.cur = 1 - g.cur;
    }
}

}  // namespace lgd
