// Generic per-cell kernels: region (streak list) updates, streak copies
// between the grid and packed host-side buffers, the seeded fill and the
// deterministic checksum.
//
// A region update is the device form of UpdateFunctor<CELL>()(region, ...,
// gridOld, &gridNew, nanoStep) (storage/updatefunctor.h:403-428): only the
// cells of the streaks are written into the next grid.  One thread per
// cell; a thread finds its streak by binary search over the streaks'
// exclusive prefix sums of lengths.
#include "lgd_internal.h"
#include "k_cells.cuh"

namespace lgd {

__device__ __forceinline__ void locate_cell(const int *streaks, const long long *prefix, int n_streaks,
                                            long long i, int *x, int *y, int *z)
{
    int lo = 0;
    int hi = n_streaks - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= i) {
            lo = mid;
        } else {
            hi = mid - 1;
        }
    }
    *x = streaks[4 * lo] + (int)(i - prefix[lo]);
    *y = streaks[4 * lo + 1];
    *z = streaks[4 * lo + 2];
}

template<typename T>
struct Stencil7Loads {
    T c, n, s, e, w, t, b;
    __device__ __forceinline__ Stencil7Loads(const View<const T>& v, int x, int y, int z, int periodic, T edge)
    {
        c = v.at(x, y, z);
        n = load_bc(v, x, y - 1, z, periodic, edge);
        s = load_bc(v, x, y + 1, z, periodic, edge);
        e = load_bc(v, x + 1, y, z, periodic, edge);
        w = load_bc(v, x - 1, y, z, periodic, edge);
        t = load_bc(v, x, y, z + 1, periodic, edge);
        b = load_bc(v, x, y, z - 1, periodic, edge);
    }
};

template<typename CELL>
__global__ void region_jacobi_kernel(View<const typename CELL::T> in, View<typename CELL::T> out, int periodic,
                                     typename CELL::T edge, const int *streaks, const long long *prefix,
                                     int n_streaks, long long cells)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= cells) return;
    int x, y, z;
    locate_cell(streaks, prefix, n_streaks, i, &x, &y, &z);
    Stencil7Loads<typename CELL::T> l(in, x, y, z, periodic, edge);
    out.at(x, y, z) = CELL::apply(l.c, l.n, l.s, l.e, l.w, l.t, l.b);
}

// valB' = valA(0,0,-1) + valA(0,-1,0) + valA(-1,0,0) + valA(1,0,0) +
// valA(0,1,0) + valA(0,0,1)
// (storage/test/unit/fixedneighborhoodupdatefunctortest.h:30-46).
__global__ void region_sum6_kernel(View<const double> a, View<double> outB, int periodic, double edgeA,
                                   const int *streaks, const long long *prefix, int n_streaks, long long cells)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= cells) return;
    int x, y, z;
    locate_cell(streaks, prefix, n_streaks, i, &x, &y, &z);
    double acc = load_bc(a, x, y, z - 1, periodic, edgeA);
    acc = __dadd_rn(acc, load_bc(a, x, y - 1, z, periodic, edgeA));
    acc = __dadd_rn(acc, load_bc(a, x - 1, y, z, periodic, edgeA));
    acc = __dadd_rn(acc, load_bc(a, x + 1, y, z, periodic, edgeA));
    acc = __dadd_rn(acc, load_bc(a, x, y + 1, z, periodic, edgeA));
    acc = __dadd_rn(acc, load_bc(a, x, y, z + 1, periodic, edgeA));
    outB.at(x, y, z) = acc;
}

__global__ void region_gol_kernel(View<const uint8_t> in, View<uint8_t> out, int periodic, uint8_t edge,
                                  const int *streaks, const long long *prefix, int n_streaks, long long cells)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= cells) return;
    int x, y, z;
    locate_cell(streaks, prefix, n_streaks, i, &x, &y, &z);
    int living = 0;
    for (int dy = -1; dy <= 1; ++dy) {
        for (int dx = -1; dx <= 1; ++dx) {
            living += load_bc(in, x + dx, y + dy, z, periodic, edge);
        }
    }
    uint8_t self = in.at(x, y, z);
    out.at(x, y, z) = gol_rule(self, living - self);
}

// The self-validating test cell (LGD_CELL_TEST; the reference's TestCell,
// misc/testcell.h:205-372): a cell copies itself, checks every neighbour of
// its stencil as the simulator delivers it - the neighbour's position,
// dimensions and cycle counter, and whether it is the edge cell, against
// what the cell's own position and the topology imply - and the nano step
// against its cycle counter, then counts the cycle.  A failed check clears
// the valid flag (the cycle counter stays where it was when the nano step
// is wrong, as in the reference).
__device__ __forceinline__ bool test_check_neighbor(const TestRec& c, const TestRec& o, const int rel[3], int dim,
                                                    int periodic)
{
    if (!o.valid) return false;
    bool should_edge = false;
    int expect[3] = {0, 0, 0};
    for (int a = 0; a < dim; ++a) {
        const int p = c.pos[a] + rel[a];
        if ((periodic >> a) & 1) {
            expect[a] = ((p % c.dim[a]) + c.dim[a]) % c.dim[a];
        } else {
            should_edge |= p < 0 || p >= c.dim[a];
            expect[a] = p;
        }
    }
    if ((o.edge != 0) != should_edge) return false;
    if (!should_edge) {
        if (o.cycle != c.cycle) return false;
        for (int a = 0; a < dim; ++a) {
            if (o.dim[a] != c.dim[a] || o.pos[a] != expect[a]) return false;
        }
    }
    return true;
}

__global__ void region_test_kernel(View<const TestRec> in, View<TestRec> out, int dim, int periodic, int von_neumann,
                                   unsigned nano_steps, unsigned nano, int edge_code, const int *streaks,
                                   const long long *prefix, int n_streaks, long long cells)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= cells) return;
    int x, y, z;
    locate_cell(streaks, prefix, n_streaks, i, &x, &y, &z);
    const TestRec c = in.at(x, y, z);
    TestRec r = c;
    if (c.edge) {
        r.valid = 0;
        out.at(x, y, z) = r;
        return;
    }
    const int n[3] = {in.nx, in.ny, in.nz};
    bool ok = c.valid != 0;
    for (int dz = (dim > 2 ? -1 : 0); dz <= (dim > 2 ? 1 : 0); ++dz) {
        for (int dy = (dim > 1 ? -1 : 0); dy <= (dim > 1 ? 1 : 0); ++dy) {
            for (int dx = -1; dx <= 1; ++dx) {
                if (von_neumann && abs(dx) + abs(dy) + abs(dz) > 1) continue;
                const int rel[3] = {dx, dy, dz};
                // the neighbour as delivered: wrapped on periodic axes, the
                // edge cell beyond the others
                int g[3] = {x + dx, y + dy, z + dz};
                bool outside = false;
                for (int a = 0; a < dim; ++a) {
                    if (g[a] < 0 || g[a] >= n[a]) {
                        if ((periodic >> a) & 1) {
                            g[a] = (g[a] + n[a]) % n[a];
                        } else {
                            outside = true;
                        }
                    }
                }
                TestRec o;
                if (outside) {
                    o = TestRec();
                    o.valid = (unsigned char)(edge_code & 1);
                    o.edge = (unsigned char)((edge_code >> 1) & 1);
                } else {
                    o = in.at(g[0], g[1], g[2]);
                }
                ok &= test_check_neighbor(c, o, rel, dim, periodic);
            }
        }
    }
    if (nano >= nano_steps || nano != c.cycle % nano_steps) {
        r.valid = 0;
        out.at(x, y, z) = r;
        return;
    }
    r.valid = ok ? 1 : 0;
    r.cycle = c.cycle + 1;
    out.at(x, y, z) = r;
}

template<typename R>
__global__ void region_varcoef_kernel(View<const R> u, View<const R> k, View<R> out, int periodic, R edgeU, R edgeK,
                                      const int *streaks, const long long *prefix, int n_streaks, long long cells)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= cells) return;
    int x, y, z;
    locate_cell(streaks, prefix, n_streaks, i, &x, &y, &z);
    out.at(x, y, z) = VarCoef<R>::apply(
        u.at(x, y, z), k.at(x, y, z),
        load_bc(u, x - 1, y, z, periodic, edgeU), load_bc(k, x - 1, y, z, periodic, edgeK),
        load_bc(u, x + 1, y, z, periodic, edgeU), load_bc(k, x + 1, y, z, periodic, edgeK),
        load_bc(u, x, y - 1, z, periodic, edgeU), load_bc(k, x, y - 1, z, periodic, edgeK),
        load_bc(u, x, y + 1, z, periodic, edgeU), load_bc(k, x, y + 1, z, periodic, edgeK),
        load_bc(u, x, y, z - 1, periodic, edgeU), load_bc(k, x, y, z - 1, periodic, edgeK),
        load_bc(u, x, y, z + 1, periodic, edgeU), load_bc(k, x, y, z + 1, periodic, edgeK));
}

template<typename T>
static View<T> view_of(Grid& g, int member, int which)
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
static View<const T> cview_of(Grid& g, int member, int which)
{
    View<T> v = view_of<T>(g, member, which);
    View<const T> c;
    c.p = v.p;
    c.pitch = v.pitch;
    c.nx = v.nx;
    c.ny = v.ny;
    c.nz = v.nz;
    return c;
}

long long fix_edge(const Grid& g);

void launch_region(Grid& g, const int *d_streaks, const long long *d_prefix, int n_streaks, long long cells,
                   unsigned nano_step)
{
    if (cells == 0) return;
    const int threads = 256;
    long long blocks = (cells + threads - 1) / threads;
    LGD_REQUIRE(blocks < (1ll << 31), LGD_ERR_RANGE, "region too large");
    const int per = g.desc.periodic;
    switch (g.desc.cell) {
    case LGD_CELL_JACOBI7_F64:
        region_jacobi_kernel<Jacobi7F64><<<(unsigned)blocks, threads, 0, g.stream>>>(
            cview_of<double>(g, 0, 0), view_of<double>(g, 0, 1), per, g.desc.edge[0], d_streaks, d_prefix, n_streaks, cells);
        break;
    case LGD_CELL_JACOBI7_F64_FIX:
        region_jacobi_kernel<Jacobi7Fix><<<(unsigned)blocks, threads, 0, g.stream>>>(
            cview_of<long long>(g, 0, 0), view_of<long long>(g, 0, 1), per, fix_edge(g), d_streaks, d_prefix, n_streaks, cells);
        break;
    case LGD_CELL_JACOBI7_F32:
        region_jacobi_kernel<Jacobi7F32><<<(unsigned)blocks, threads, 0, g.stream>>>(
            cview_of<float>(g, 0, 0), view_of<float>(g, 0, 1), per, (float)g.desc.edge[0], d_streaks, d_prefix, n_streaks, cells);
        break;
    case LGD_CELL_SUM6_F64:
        region_sum6_kernel<<<(unsigned)blocks, threads, 0, g.stream>>>(
            cview_of<double>(g, 0, 0), view_of<double>(g, 1, 1), per, g.desc.edge[0], d_streaks, d_prefix, n_streaks, cells);
        break;
    case LGD_CELL_GOL_U8:
        region_gol_kernel<<<(unsigned)blocks, threads, 0, g.stream>>>(
            cview_of<uint8_t>(g, 0, 0), view_of<uint8_t>(g, 0, 1), per, (uint8_t)g.desc.edge[0], d_streaks, d_prefix, n_streaks, cells);
        break;
    case LGD_CELL_VARCOEF_F32:
        region_varcoef_kernel<float><<<(unsigned)blocks, threads, 0, g.stream>>>(
            cview_of<float>(g, 0, 0), cview_of<float>(g, 1, 0), view_of<float>(g, 0, 1), per,
            (float)g.desc.edge[0], (float)g.desc.edge[1], d_streaks, d_prefix, n_streaks, cells);
        break;
    case LGD_CELL_VARCOEF_F64:
        region_varcoef_kernel<double><<<(unsigned)blocks, threads, 0, g.stream>>>(
            cview_of<double>(g, 0, 0), cview_of<double>(g, 1, 0), view_of<double>(g, 0, 1), per,
            g.desc.edge[0], g.desc.edge[1], d_streaks, d_prefix, n_streaks, cells);
        break;
    case LGD_CELL_TEST:
        region_test_kernel<<<(unsigned)blocks, threads, 0, g.stream>>>(
            cview_of<TestRec>(g, 0, 0), view_of<TestRec>(g, 0, 1), g.desc.dim, per, g.desc.flags & LGD_TEST_VON_NEUMANN,
            test_nano_steps(g), nano_step % test_nano_steps(g), (int)g.desc.edge[0], d_streaks, d_prefix, n_streaks,
            cells);
        break;
    default:
        throw Error(LGD_ERR_UNSUPPORTED, "cell kind has no region kernel");
    }
    check_launch("region update");
    ++g.launches;
}

// ------------------------------------------------------------ streak copy
// records of any size (record grids): one thread per record, 4-byte words
// where the record size allows, else bytes
template<typename W>
__global__ void streak_copy_records_kernel(unsigned char *base, long pitch_bytes, int ny, int rec_words,
                                           const int *streaks, const long long *prefix, int n_streaks,
                                           long long cells, W *packed, bool to_grid)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= cells) return;
    int x, y, z;
    locate_cell(streaks, prefix, n_streaks, i, &x, &y, &z);
    W *cell = (W *)(base + ((long)z * ny + y) * pitch_bytes) + (long)x * rec_words;
    W *pk = packed + i * rec_words;
    for (int k = 0; k < rec_words; ++k) {
        if (to_grid) {
            cell[k] = pk[k];
        } else {
            pk[k] = cell[k];
        }
    }
}

// streaks of a fixed-point grid as FP64 values (k * 2^(scale_exp - 57))
__global__ void streak_copy_fix_kernel(View<long long> v, const int *streaks, const long long *prefix, int n_streaks,
                                       long long cells, double *packed, bool to_grid, int scale_exp)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= cells) return;
    int x, y, z;
    locate_cell(streaks, prefix, n_streaks, i, &x, &y, &z);
    if (to_grid) {
        v.at(x, y, z) = __double2ll_rn(ldexp(packed[i], LGD_FIX_BITS - scale_exp));
    } else {
        packed[i] = ldexp((double)v.at(x, y, z), scale_exp - LGD_FIX_BITS);
    }
}

int fix_scale_exp(const Grid& g);

void launch_streak_copy_fix(Grid& g, const int *d_streaks, const long long *d_prefix, int n_streaks, long long cells,
                            double *d_packed, bool to_grid)
{
    if (cells == 0) return;
    const int threads = 256;
    const long long blocks = (cells + threads - 1) / threads;
    streak_copy_fix_kernel<<<(unsigned)blocks, threads, 0, g.stream>>>(view_of<long long>(g, 0, 0), d_streaks,
                                                                      d_prefix, n_streaks, cells, d_packed, to_grid,
                                                                      fix_scale_exp(g));
    check_launch("fixed-point streak copy");
    ++g.launches;
}

template<typename T>
__global__ void streak_copy_kernel(View<T> v, const int *streaks, const long long *prefix, int n_streaks,
                                   long long cells, T *packed, bool to_grid)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= cells) return;
    int x, y, z;
    locate_cell(streaks, prefix, n_streaks, i, &x, &y, &z);
    if (to_grid) {
        v.at(x, y, z) = packed[i];
    } else {
        packed[i] = v.at(x, y, z);
    }
}

void launch_streak_copy(Grid& g, int member, int which, const int *d_streaks, const long long *d_prefix,
                        int n_streaks, long long cells, void *d_packed, bool to_grid)
{
    if (cells == 0) return;
    const int threads = 256;
    long long blocks = (cells + threads - 1) / threads;
    switch (g.m[member].elem) {
    case 1:
        streak_copy_kernel<uint8_t><<<(unsigned)blocks, threads, 0, g.stream>>>(
            view_of<uint8_t>(g, member, which), d_streaks, d_prefix, n_streaks, cells, (uint8_t *)d_packed, to_grid);
        break;
    case 4:
        streak_copy_kernel<float><<<(unsigned)blocks, threads, 0, g.stream>>>(
            view_of<float>(g, member, which), d_streaks, d_prefix, n_streaks, cells, (float *)d_packed, to_grid);
        break;
    case 8:
        streak_copy_kernel<double><<<(unsigned)blocks, threads, 0, g.stream>>>(
            view_of<double>(g, member, which), d_streaks, d_prefix, n_streaks, cells, (double *)d_packed, to_grid);
        break;
    case 64:
        streak_copy_kernel<TestRec><<<(unsigned)blocks, threads, 0, g.stream>>>(
            view_of<TestRec>(g, member, which), d_streaks, d_prefix, n_streaks, cells, (TestRec *)d_packed, to_grid);
        break;
    default: {
        const int elem = g.m[member].elem;
        unsigned char *base = (unsigned char *)g.m[member].buf[g.m[member].is_static ? 0 : (which ? 1 - g.cur : g.cur)];
        const long pitch = (long)g.pitch_bytes[member];
        if (elem % 4 == 0) {
            streak_copy_records_kernel<uint32_t><<<(unsigned)blocks, threads, 0, g.stream>>>(
                base, pitch, g.desc.ny, elem / 4, d_streaks, d_prefix, n_streaks, cells, (uint32_t *)d_packed, to_grid);
        } else {
            streak_copy_records_kernel<uint8_t><<<(unsigned)blocks, threads, 0, g.stream>>>(
                base, pitch, g.desc.ny, elem, d_streaks, d_prefix, n_streaks, cells, (uint8_t *)d_packed, to_grid);
        }
    }
    }
    check_launch("streak copy");
    ++g.launches;
}

// ------------------------------------------------------------------- fill
template<typename T, int MODE>
__global__ void fill_kernel(View<T> v, uint64_t key, double p, int scale_exp)
{
    long long cells = (long long)v.nx * v.ny * v.nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
         i += (long long)gridDim.x * blockDim.x) {
        int x = (int)(i % v.nx);
        long long r = i / v.nx;
        int y = (int)(r % v.ny);
        int z = (int)(r / v.ny);
        double u = splitmix_uniform(key, (uint64_t)i);
        if (MODE == 0) {
            v.at(x, y, z) = (T)u;
        } else if (MODE == 1) {
            v.at(x, y, z) = (T)(u < p ? 1 : 0);
        } else {
            v.at(x, y, z) = (T)__double2ll_rn(ldexp(u, LGD_FIX_BITS - scale_exp));
        }
    }
}

uint64_t stream_key(uint64_t seed, int stream)
{
    return splitmix_mix(seed * 256ull + (uint64_t)stream);
}

void launch_fill(Grid& g, int member, int which, uint64_t seed, int stream, int mode, double p, int scale_exp)
{
    const uint64_t key = stream_key(seed, stream);
    const int threads = 256;
    const int blocks = 152 * 8;
    switch (g.m[member].elem) {
    case 1:
        fill_kernel<uint8_t, 1><<<blocks, threads, 0, g.stream>>>(view_of<uint8_t>(g, member, which), key, p, 0);
        break;
    case 4:
        fill_kernel<float, 0><<<blocks, threads, 0, g.stream>>>(view_of<float>(g, member, which), key, p, 0);
        break;
    case 8:
        if (mode == 2) {
            fill_kernel<long long, 2><<<blocks, threads, 0, g.stream>>>(view_of<long long>(g, member, which), key, p, scale_exp);
        } else {
            fill_kernel<double, 0><<<blocks, threads, 0, g.stream>>>(view_of<double>(g, member, which), key, p, 0);
        }
        break;
    default:
        throw Error(LGD_ERR_INVALID, "unsupported member size");
    }
    check_launch("fill");
    ++g.launches;
}

// --------------------------------------------------------------- checksum
// Block b sums its rows (fixed order, fixed tree); the host adds the
// per-block partials in order.  Deterministic for a given grid shape.
template<typename T, bool FIX>
__global__ void checksum_kernel(View<const T> v, double *partials, int scale_exp)
{
    __shared__ double red[256];
    long long rows = (long long)v.ny * v.nz;
    double acc = 0.0;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const T *row = v.p + r * v.pitch;
        for (int x = threadIdx.x; x < v.nx; x += blockDim.x) {
            acc += FIX ? ldexp((double)row[x], scale_exp - LGD_FIX_BITS) : (double)row[x];
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

int fix_scale_exp(const Grid& g);

void launch_checksum(Grid& g, int member, int which, double *out)
{
    const int blocks = 1024;
    if (g.partial_capacity < blocks) {
        if (g.d_partials) cudaFree(g.d_partials);
        g.d_partials = nullptr;
        LGD_CHECK_CUDA(cudaMalloc(&g.d_partials, sizeof(double) * blocks));
        g.partial_capacity = blocks;
    }
    const bool fix = g.desc.cell == LGD_CELL_JACOBI7_F64_FIX && member == 0;
    switch (g.m[member].elem) {
    case 1:
        checksum_kernel<uint8_t, false><<<blocks, 256, 0, g.stream>>>(cview_of<uint8_t>(g, member, which), g.d_partials, 0);
        break;
    case 4:
        checksum_kernel<float, false><<<blocks, 256, 0, g.stream>>>(cview_of<float>(g, member, which), g.d_partials, 0);
        break;
    case 8:
        if (fix) {
            checksum_kernel<long long, true><<<blocks, 256, 0, g.stream>>>(cview_of<long long>(g, member, which), g.d_partials,
                                                                         fix_scale_exp(g));
        } else {
            checksum_kernel<double, false><<<blocks, 256, 0, g.stream>>>(cview_of<double>(g, member, which), g.d_partials, 0);
        }
        break;
    default:
        throw Error(LGD_ERR_INVALID, "unsupported member size");
    }
    check_launch("checksum");
    ++g.launches;
    double host[1024];
    LGD_CHECK_CUDA(cudaMemcpyAsync(host, g.d_partials, sizeof(double) * blocks, cudaMemcpyDeviceToHost, g.stream));
    LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
    double s = 0.0;
    for (int i = 0; i < blocks; ++i) s += host[i];
    *out = s;
}

}  // namespace lgd
