// C ABI of the structured-grid part: handle lifetime, host <-> device
// copies, stepping, region updates.  See include/lgd_gpu.h for the
// contract and the reference entry points each function replaces.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lgd_internal.h"
#include "k_common.cuh"

namespace lgd {

static thread_local int t_last_code = LGD_OK;
static thread_local std::string t_last_msg;

void set_error(int code, const std::string& msg)
{
    t_last_code = code;
    t_last_msg = msg;
}

void clear_error()
{
    t_last_code = LGD_OK;
    t_last_msg.clear();
}

struct CellInfo {
    int n_members;
    int elem[2];        // device element size per member
    int host_elem[2];   // element size at the ABI
    bool is_static[2];
    int dim_min, dim_max;
};

static CellInfo cell_info(int cell)
{
    switch (cell) {
    case LGD_CELL_JACOBI7_F64:     return {1, {8, 0}, {8, 0}, {false, false}, 3, 3};
    case LGD_CELL_JACOBI7_F64_FIX: return {1, {8, 0}, {8, 0}, {false, false}, 3, 3};
    case LGD_CELL_JACOBI7_F32:     return {1, {4, 0}, {4, 0}, {false, false}, 3, 3};
    case LGD_CELL_SUM6_F64:        return {2, {8, 8}, {8, 8}, {false, false}, 3, 3};
    case LGD_CELL_GOL_U8:          return {1, {1, 0}, {1, 0}, {false, false}, 2, 2};
    case LGD_CELL_VARCOEF_F32:     return {2, {4, 4}, {4, 4}, {false, true}, 3, 3};
    case LGD_CELL_VARCOEF_F64:     return {2, {8, 8}, {8, 8}, {false, true}, 3, 3};
    case LGD_CELL_TEST:            return {1, {64, 0}, {64, 0}, {false, false}, 1, 3};
    case LGD_CELL_RECORD:          return {1, {0, 0}, {0, 0}, {false, false}, 1, 3};   // size per grid
    default:
        throw Error(LGD_ERR_INVALID, "unknown cell kind " + std::to_string(cell));
    }
}

// ---------------------------------------------------------- fixed point
// The FP64 Jacobi grid in fixed-point form: value = k * 2^(fix_exp - LGD_FIX_BITS).
// fix_exp is chosen at upload so that every value and the edge cell fit
// (|value| <= 2^fix_exp); averaging never leaves that range.
static int exp_bound(double m)
{
    if (!(m > 0.0)) return 0;
    int e = 0;
    double f = std::frexp(m, &e);   // m = f * 2^e, f in [0.5, 1)
    (void)f;
    return e;                        // 2^e > m
}

long long fix_edge(const Grid& g)
{
    return std::llrint(std::ldexp(g.desc.edge[0], LGD_FIX_BITS - g.fix_exp));
}

int fix_scale_exp(const Grid& g)
{
    return g.fix_exp;
}

// dense (x-fastest, rows of nx) doubles -> pitched fixed point
// (warps take whole rows, lanes walk a row: no division per cell)
__global__ void to_fix_pitched_kernel(const double *src, long long *dst, int nx, long long rows, long long pitch, int exp)
{
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long r = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
        for (int x = lane; x < nx; x += 32) {
            dst[r * pitch + x] = __double2ll_rn(ldexp(src[r * nx + x], LGD_FIX_BITS - exp));
        }
    }
}

__global__ void from_fix_pitched_kernel(const long long *src, double *dst, int nx, long long rows, long long pitch, int exp)
{
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long r = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
        for (int x = lane; x < nx; x += 32) {
            dst[r * nx + x] = ldexp((double)src[r * pitch + x], exp - LGD_FIX_BITS);
        }
    }
}

// per-block max |v| (NaN propagates as NaN through fmax's operand order
// being irrelevant: a NaN block result is turned into +inf so the host sees
// a non-finite maximum)
__global__ void absmax_kernel(const double *v, long long n, double *partial, unsigned long long *negative)
{
    __shared__ double red[256];
    double m = 0.0;
    bool bad = false;
    bool neg = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double a = fabs(v[i]);
        bad |= !(a <= 1.7976931348623157e308);
        neg |= v[i] < 0.0;
        m = fmax(m, a);
    }
    if (__any_sync(0xffffffffu, neg) && (threadIdx.x & 31) == 0) atomicOr(negative, 1ull);
    red[threadIdx.x] = bad ? __longlong_as_double(0x7ff0000000000000ll) : m;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void rescale_fix_kernel(long long *buf, long long n, int shift)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long v = buf[i];
        buf[i] = (v + (1ll << (shift - 1))) >> shift;
    }
}

static size_t buffer_elems(const Grid& g, int member)
{
    return g.pitch_bytes[member] / g.m[member].elem * (size_t)g.desc.ny * g.desc.nz;
}

// Raises fix_exp to at least e, rescaling both buffers.
static void raise_fix_exp(Grid& g, int e)
{
    if (e <= g.fix_exp) return;
    const int shift = e - g.fix_exp;
    const long long n = (long long)buffer_elems(g, 0);
    for (int b = 0; b < 2; ++b) {
        if (shift >= 62) {
            LGD_CHECK_CUDA(cudaMemsetAsync(g.m[0].buf[b], 0, n * 8, g.stream));
        } else {
            rescale_fix_kernel<<<152 * 4, 256, 0, g.stream>>>((long long *)g.m[0].buf[b], n, shift);
            check_launch("rescale");
            ++g.launches;
        }
    }
    g.fix_exp = e;
}

// max |k| over the cells of one fixed-point buffer (rows of nx cells, pitch
// elements apart) into *out with atomicMax
__global__ void fix_absmax_kernel(const long long *buf, int nx, long long rows, long long pitch,
                                  unsigned long long *out)
{
    unsigned long long m = 0;
    // warps take whole rows (no division per cell), lanes walk a row
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long r = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
        const long long *row = buf + r * pitch;
        for (int x = lane; x < nx; x += 32) {
            const long long v = row[x];
            m = max(m, (unsigned long long)(v < 0 ? -v : v));
        }
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

__global__ void shift_fix_kernel(long long *buf, long long n, int shift)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        buf[i] = (long long)((unsigned long long)buf[i] << shift);
    }
}

// Lowers fix_exp as far as both buffers and the edge cell allow (the
// largest |k| just below 2^57 afterwards), shifting both buffers left: no
// rounding, only unused high bits are traded for fraction bits.  With a
// zero edge cell a decaying grid keeps 57 significant bits at its maximum
// instead of losing one per halving.  Synchronises the grid's stream.
static void lower_fix_exp(Grid& g)
{
    if (g.fix_pinned) {
        g.fix_steps_unchecked = 0;
        return;
    }
    const long long rows = (long long)g.desc.ny * g.desc.nz;
    const long long pitch = (long long)(g.pitch_bytes[0] / 8);
    LGD_CHECK_CUDA(cudaMemsetAsync(g.d_fixmax, 0, sizeof(unsigned long long), g.stream));
    for (int b = 0; b < 2; ++b) {
        fix_absmax_kernel<<<152 * 4, 256, 0, g.stream>>>((const long long *)g.m[0].buf[b], g.desc.nx, rows, pitch,
                                                         g.d_fixmax);
        check_launch("fixed-point maximum");
        ++g.launches;
    }
    unsigned long long m = 0;
    LGD_CHECK_CUDA(cudaMemcpyAsync(&m, g.d_fixmax, sizeof(m), cudaMemcpyDeviceToHost, g.stream));
    LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
    g.fix_steps_unchecked = 0;
    if (m == 0) return;                                         // an all-zero grid keeps its exponent
    int shift = __builtin_clzll(m) - (64 - LGD_FIX_BITS);      // m << shift < 2^57 <= m << (shift + 1)
    if (g.desc.edge[0] != 0.0) shift = std::min(shift, g.fix_exp - exp_bound(std::fabs(g.desc.edge[0])));
    shift = std::min(shift, g.fix_exp + 960);                  // stays far inside the double range
    if (shift <= 0) return;
    const long long n = (long long)buffer_elems(g, 0);
    for (int b = 0; b < 2; ++b) {
        shift_fix_kernel<<<152 * 4, 256, 0, g.stream>>>((long long *)g.m[0].buf[b], n, shift);
        check_launch("fixed-point rescale");
        ++g.launches;
    }
    g.fix_exp -= shift;
    LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
}

// --------------------------------------------------------------- helpers
// Reads (and clears) the device error word that kernels with bounded waits
// set when a wait gave up; call after the stream is synchronised.
static void check_device_error(Grid& g)
{
    int e = 0;
    LGD_CHECK_CUDA(cudaMemcpy(&e, g.d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        LGD_CHECK_CUDA(cudaMemset(g.d_err, 0, sizeof(int)));
        throw Error(LGD_ERR_TIMEOUT, "a device-side wait gave up; the last step's results are incomplete");
    }
}

// Device staging buffer of the handle for conversions at the boundary,
// allocated on first use and grown when needed (kept until destroy, so
// repeated uploads and downloads do not allocate).
static double *staging(Grid& g, size_t bytes)
{
    if (bytes > g.stage_bytes) {
        if (g.d_stage) {
            LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
            cudaFree(g.d_stage);
            g.d_stage = nullptr;
            g.stage_bytes = 0;
        }
        LGD_CHECK_CUDA(cudaMalloc(&g.d_stage, bytes));
        g.stage_bytes = bytes;
    }
    return (double *)g.d_stage;
}

// Row chunks of a fixed-point transfer: the copy of chunk k overlaps the
// conversion of its neighbour (16 chunks: 64 MiB each at 512^3 FP64).
constexpr int XFER_CHUNKS = 16;
// steps of a fixed-point grid between two checks of its exponent
constexpr int FIX_CHECK_STEPS = 256;
constexpr int ABSMAX_BLOCKS = 152;

static void xfer_init(Grid& g)
{
    if (g.xfer_ready) return;
    static_assert(XFER_CHUNKS + 1 <= (int)(sizeof(g.xfer_ev) / sizeof(g.xfer_ev[0])), "event array too small");
    LGD_CHECK_CUDA(cudaStreamCreateWithFlags(&g.xfer_stream, cudaStreamNonBlocking));
    for (int k = 0; k <= XFER_CHUNKS; ++k) {
        LGD_CHECK_CUDA(cudaEventCreateWithFlags(&g.xfer_ev[k], cudaEventDisableTiming));
    }
    g.xfer_ready = true;
}

static Grid& grid_of(lgd_handle *h)
{
    LGD_REQUIRE(h != nullptr, LGD_ERR_INVALID, "null handle");
    return h->g;
}

static void check_member(const Grid& g, int member, int which)
{
    LGD_REQUIRE(member >= 0 && member < g.n_members, LGD_ERR_INVALID, "member index out of range");
    LGD_REQUIRE(which == 0 || which == 1, LGD_ERR_INVALID, "which must be 0 (current) or 1 (next)");
}

static void *member_buf(Grid& g, int member, int which)
{
    if (g.m[member].is_static) return g.m[member].buf[0];
    return g.m[member].buf[which ? 1 - g.cur : g.cur];
}

static size_t cells_of(const Grid& g)
{
    return (size_t)g.desc.nx * g.desc.ny * g.desc.nz;
}

// Validates streaks (x, y, z, endX) and stages them plus their prefix sums
// on the device; returns the number of cells.
static long long stage_streaks(Grid& g, const int *streaks, int n)
{
    LGD_REQUIRE(n >= 0, LGD_ERR_INVALID, "negative streak count");
    LGD_REQUIRE(n == 0 || streaks != nullptr, LGD_ERR_INVALID, "null streak list");
    std::vector<long long> prefix(n > 0 ? n : 1);
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        const int x = streaks[4 * i];
        const int y = streaks[4 * i + 1];
        const int z = streaks[4 * i + 2];
        const int end = streaks[4 * i + 3];
        LGD_REQUIRE(x >= 0 && end <= g.desc.nx && x <= end, LGD_ERR_RANGE, "streak outside the grid in x");
        LGD_REQUIRE(y >= 0 && y < g.desc.ny, LGD_ERR_RANGE, "streak outside the grid in y");
        LGD_REQUIRE(z >= 0 && z < g.desc.nz, LGD_ERR_RANGE, "streak outside the grid in z");
        prefix[i] = total;
        total += end - x;
    }
    if (n > g.streak_capacity) {
        if (g.d_streaks) cudaFree(g.d_streaks);
        if (g.d_streak_prefix) cudaFree(g.d_streak_prefix);
        g.d_streaks = nullptr;
        g.d_streak_prefix = nullptr;
        g.streak_capacity = 0;
        LGD_CHECK_CUDA(cudaMalloc(&g.d_streaks, sizeof(int) * 4 * n));
        LGD_CHECK_CUDA(cudaMalloc(&g.d_streak_prefix, sizeof(long long) * n));
        g.streak_capacity = n;
    }
    if (n > 0) {
        LGD_CHECK_CUDA(cudaMemcpyAsync(g.d_streaks, streaks, sizeof(int) * 4 * n, cudaMemcpyHostToDevice, g.stream));
        LGD_CHECK_CUDA(cudaMemcpyAsync(g.d_streak_prefix, prefix.data(), sizeof(long long) * n, cudaMemcpyHostToDevice, g.stream));
        // the staging arrays are host stack/heap memory: finish before they go
        LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
    }
    return total;
}

void launch_fill(Grid& g, int member, int which, uint64_t seed, int stream, int mode, double p, int scale_exp);

}  // namespace lgd

using namespace lgd;

extern "C" {

int lgd_gpu_last_error(char *buf, size_t len)
{
    if (buf && len > 0) {
        std::strncpy(buf, t_last_msg.c_str(), len - 1);
        buf[len - 1] = '\0';
    }
    return t_last_code;
}

int lgd_gpu_version(void)
{
    return 10000;
}

int lgd_gpu_device_count(int *count)
{
    return guard([&] {
        LGD_REQUIRE(count != nullptr, LGD_ERR_INVALID, "null count");
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            n = 0;
        }
        *count = n;
    });
}

// Allocates a grid; record grids (LGD_CELL_RECORD) take their element size
// and edge record from the arguments.
static void create_grid(const lgd_grid_desc *desc, size_t record_bytes, const void *edge_record, lgd_handle **out)
{
    {
        LGD_REQUIRE(desc != nullptr && out != nullptr, LGD_ERR_INVALID, "null argument");
        *out = nullptr;
        CellInfo ci = cell_info(desc->cell);
        if (desc->cell == LGD_CELL_RECORD) {
            LGD_REQUIRE(record_bytes >= 1 && record_bytes <= LGD_RECORD_MAX_BYTES, LGD_ERR_INVALID,
                        "record size out of range (1 .. LGD_RECORD_MAX_BYTES)");
            LGD_REQUIRE(edge_record != nullptr, LGD_ERR_INVALID, "null edge record");
            ci.elem[0] = ci.host_elem[0] = (int)record_bytes;
        }
        LGD_REQUIRE(desc->dim >= ci.dim_min && desc->dim <= ci.dim_max, LGD_ERR_INVALID, "dimension does not match the cell");
        LGD_REQUIRE(desc->nx > 0 && desc->ny > 0 && desc->nz > 0, LGD_ERR_INVALID, "grid dimensions must be positive");
        LGD_REQUIRE(desc->dim == 3 || desc->nz == 1, LGD_ERR_INVALID, "2D grids have nz = 1");
        LGD_REQUIRE(desc->dim >= 2 || desc->ny == 1, LGD_ERR_INVALID, "1D grids have ny = nz = 1");
        LGD_REQUIRE(desc->cell == LGD_CELL_TEST ? (desc->flags & ~(LGD_TEST_VON_NEUMANN | 0xff00)) == 0
                                                : desc->flags == 0,
                    LGD_ERR_INVALID, "flags not defined for this cell kind");
        LGD_REQUIRE((desc->periodic & ~7) == 0, LGD_ERR_INVALID, "periodic mask has bits beyond z");
        int ndev = 0;
        LGD_CHECK_CUDA(cudaGetDeviceCount(&ndev));
        LGD_REQUIRE(ndev > 0, LGD_ERR_CUDA, "no CUDA device");

        lgd_handle *h = new lgd_handle();
        Grid& g = h->g;
        std::memset(&g, 0, sizeof(Grid));
        g.desc = *desc;
        g.n_members = ci.n_members;
        LGD_CHECK_CUDA(cudaGetDevice(&g.device));
        try {
            LGD_CHECK_CUDA(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
            LGD_CHECK_CUDA(cudaMalloc(&g.d_err, sizeof(int)));
            LGD_CHECK_CUDA(cudaMemsetAsync(g.d_err, 0, sizeof(int), g.stream));
            for (int m = 0; m < ci.n_members; ++m) {
                g.m[m].elem = ci.elem[m];
                g.m[m].is_static = ci.is_static[m];
                g.pitch_bytes[m] = (size_t)round_up(desc->nx * ci.elem[m], 128);
                const size_t bytes = g.pitch_bytes[m] * (size_t)desc->ny * desc->nz;
                for (int b = 0; b < (ci.is_static[m] ? 1 : 2); ++b) {
                    LGD_CHECK_CUDA(cudaMalloc(&g.m[m].buf[b], bytes));
                    LGD_CHECK_CUDA(cudaMemsetAsync(g.m[m].buf[b], 0, bytes, g.stream));
                }
            }
            g.pitch_elems = g.pitch_bytes[0] / ci.elem[0];
            g.plane_elems = g.pitch_elems * desc->ny;
            if (desc->cell == LGD_CELL_RECORD) {
                g.edge_record = (unsigned char *)std::malloc(record_bytes);
                LGD_REQUIRE(g.edge_record != nullptr, LGD_ERR_NOMEM, "host allocation failed");
                std::memcpy(g.edge_record, edge_record, record_bytes);
                LGD_CHECK_CUDA(cudaMalloc(&g.d_edge_record, record_bytes));
                LGD_CHECK_CUDA(cudaMemcpyAsync(g.d_edge_record, edge_record, record_bytes, cudaMemcpyHostToDevice,
                                               g.stream));
            }
            if (desc->cell == LGD_CELL_JACOBI7_F64_FIX) {
                g.fix_exp = exp_bound(std::fabs(desc->edge[0]));
                g.fix_nonneg = desc->edge[0] >= 0.0;
                LGD_CHECK_CUDA(cudaMalloc(&g.d_fixmax, 2 * sizeof(unsigned long long)));
                LGD_CHECK_CUDA(cudaMemsetAsync(g.d_fixmax, 0, 2 * sizeof(unsigned long long), g.stream));
            }
            LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
        } catch (...) {
            for (int m = 0; m < 2; ++m) {
                for (int b = 0; b < 2; ++b) {
                    if (g.m[m].buf[b]) cudaFree(g.m[m].buf[b]);
                }
            }
            if (g.d_err) cudaFree(g.d_err);
            if (g.d_fixmax) cudaFree(g.d_fixmax);
            if (g.d_edge_record) cudaFree(g.d_edge_record);
            std::free(g.edge_record);
            if (g.stream) cudaStreamDestroy(g.stream);
            delete h;
            throw;
        }
        *out = h;
    }
}

int lgd_gpu_create(const lgd_grid_desc *desc, lgd_handle **out)
{
    return guard([&] {
        LGD_REQUIRE(desc == nullptr || desc->cell != LGD_CELL_RECORD, LGD_ERR_INVALID,
                    "record grids are created by lgd_gpu_create_records");
        create_grid(desc, 0, nullptr, out);
    });
}

int lgd_gpu_create_records(const lgd_grid_desc *desc, size_t record_bytes, const void *edge_record,
                           lgd_handle **out)
{
    return guard([&] {
        LGD_REQUIRE(desc == nullptr || desc->cell == LGD_CELL_RECORD, LGD_ERR_INVALID,
                    "desc->cell must be LGD_CELL_RECORD");
        create_grid(desc, record_bytes, edge_record, out);
    });
}

int lgd_gpu_set_edge_record(lgd_handle *h, const void *edge_record, size_t bytes)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(g.desc.cell == LGD_CELL_RECORD, LGD_ERR_INVALID, "not a record grid");
        LGD_REQUIRE(edge_record != nullptr && bytes == (size_t)g.m[0].elem, LGD_ERR_INVALID,
                    "edge record size does not match the grid's records");
        std::memcpy(g.edge_record, edge_record, bytes);
        LGD_CHECK_CUDA(cudaMemcpyAsync(g.d_edge_record, g.edge_record, bytes, cudaMemcpyHostToDevice, g.stream));
        LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
    });
}

int lgd_gpu_edge_record_device(lgd_handle *h, const void **device_edge)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(g.desc.cell == LGD_CELL_RECORD, LGD_ERR_INVALID, "not a record grid");
        LGD_REQUIRE(device_edge != nullptr, LGD_ERR_INVALID, "null output");
        *device_edge = g.d_edge_record;
    });
}

int lgd_gpu_set_fixed_point_exponent(lgd_handle *h, int e, int pin)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(g.desc.cell == LGD_CELL_JACOBI7_F64_FIX, LGD_ERR_INVALID, "not a fixed-point grid");
        LGD_REQUIRE(e >= exp_bound(std::fabs(g.desc.edge[0])) && e <= 1000 && e >= -960, LGD_ERR_RANGE,
                    "exponent out of range for the grid's edge cell");
        if (e > g.fix_exp) {
            raise_fix_exp(g, e);
        } else if (e < g.fix_exp) {
            const long long rows = (long long)g.desc.ny * g.desc.nz;
            const long long pitch = (long long)(g.pitch_bytes[0] / 8);
            LGD_CHECK_CUDA(cudaMemsetAsync(g.d_fixmax, 0, sizeof(unsigned long long), g.stream));
            for (int b = 0; b < 2; ++b) {
                fix_absmax_kernel<<<152 * 4, 256, 0, g.stream>>>((const long long *)g.m[0].buf[b], g.desc.nx, rows,
                                                                 pitch, g.d_fixmax);
                check_launch("fixed-point maximum");
                ++g.launches;
            }
            unsigned long long m = 0;
            LGD_CHECK_CUDA(cudaMemcpyAsync(&m, g.d_fixmax, sizeof(m), cudaMemcpyDeviceToHost, g.stream));
            LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
            const int shift = g.fix_exp - e;
            LGD_REQUIRE(m == 0 || (shift < 64 && (m >> (LGD_FIX_BITS - shift)) == 0), LGD_ERR_RANGE,
                        "the grid's values do not fit the lower exponent");
            const long long n = (long long)buffer_elems(g, 0);
            for (int b = 0; b < 2; ++b) {
                shift_fix_kernel<<<152 * 4, 256, 0, g.stream>>>((long long *)g.m[0].buf[b], n, shift);
                check_launch("fixed-point rescale");
                ++g.launches;
            }
            g.fix_exp = e;
        }
        g.fix_pinned = pin != 0;
        LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
    });
}

int lgd_gpu_plane_bytes(lgd_handle *h, int member, size_t *bytes)
{
    return guard([&] {
        Grid& g = grid_of(h);
        check_member(g, member, 0);
        LGD_REQUIRE(bytes != nullptr, LGD_ERR_INVALID, "null output");
        *bytes = g.pitch_bytes[member] * (g.desc.dim == 3 ? (size_t)g.desc.ny : 1);
    });
}

int lgd_gpu_copy_planes(lgd_handle *h, int member, int which, int p0, int np, void *buf, size_t bytes, int to_grid)
{
    return guard([&] {
        Grid& g = grid_of(h);
        check_member(g, member, which);
        const int planes = g.desc.dim == 3 ? g.desc.nz : g.desc.ny;
        LGD_REQUIRE(p0 >= 0 && np >= 0 && p0 + np <= planes, LGD_ERR_RANGE, "planes outside the grid");
        const size_t plane = g.pitch_bytes[member] * (g.desc.dim == 3 ? (size_t)g.desc.ny : 1);
        LGD_REQUIRE(bytes == plane * (size_t)np, LGD_ERR_INVALID, "byte count does not match the planes");
        LGD_REQUIRE(buf != nullptr || np == 0, LGD_ERR_INVALID, "null buffer");
        char *base = (char *)member_buf(g, member, which) + plane * (size_t)p0;
        if (np > 0) {
            if (to_grid) {
                LGD_CHECK_CUDA(cudaMemcpyAsync(base, buf, bytes, cudaMemcpyDefault, g.stream));
            } else {
                LGD_CHECK_CUDA(cudaMemcpyAsync(buf, base, bytes, cudaMemcpyDefault, g.stream));
            }
        }
        LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
    });
}

int lgd_gpu_get_desc(lgd_handle *h, lgd_grid_desc *out)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(out != nullptr, LGD_ERR_INVALID, "null output");
        *out = g.desc;
    });
}

int lgd_gpu_count_launches(lgd_handle *h, uint64_t n)
{
    return guard([&] { grid_of(h).launches += n; });
}

int lgd_gpu_destroy(lgd_handle *h)
{
    return guard([&] {
        if (!h) return;
        Grid& g = h->g;
        cudaStreamSynchronize(g.stream);
        for (int m = 0; m < 2; ++m) {
            for (int b = 0; b < 2; ++b) {
                if (g.m[m].buf[b]) cudaFree(g.m[m].buf[b]);
            }
        }
        if (g.d_streaks) cudaFree(g.d_streaks);
        if (g.d_streak_prefix) cudaFree(g.d_streak_prefix);
        if (g.d_partials) cudaFree(g.d_partials);
        if (g.d_err) cudaFree(g.d_err);
        if (g.d_fixmax) cudaFree(g.d_fixmax);
        if (g.d_edge_record) cudaFree(g.d_edge_record);
        std::free(g.edge_record);
        if (g.d_stage) cudaFree(g.d_stage);
        if (g.xfer_ready) {
            cudaStreamSynchronize(g.xfer_stream);
            for (int k = 0; k <= XFER_CHUNKS; ++k) cudaEventDestroy(g.xfer_ev[k]);
            cudaStreamDestroy(g.xfer_stream);
        }
        cudaStreamDestroy(g.stream);
        delete h;
    });
}

int lgd_gpu_upload(lgd_handle *h, int member, int which, const void *host, size_t bytes)
{
    return guard([&] {
        Grid& g = grid_of(h);
        check_member(g, member, which);
        const size_t n = cells_of(g);
        const int helem = g.m[member].elem;
        LGD_REQUIRE(host != nullptr, LGD_ERR_INVALID, "null host buffer");
        LGD_REQUIRE(bytes == n * helem, LGD_ERR_INVALID, "byte count does not match the grid");
        const size_t rows = (size_t)g.desc.ny * g.desc.nz;
        if (g.desc.cell == LGD_CELL_JACOBI7_F64_FIX) {
            // Stage the doubles on the device in row chunks.  Each chunk is
            // converted with the grid's current exponent as soon as it has
            // landed, while the next one is copied, and its max |value| is
            // kept per block.  If the maximum needs a larger exponent, the
            // whole staging buffer is converted again after raising it.
            const int K = (int)std::min<size_t>(XFER_CHUNKS, rows);
            double *tmp = staging(g, n * 8 + 8 * (size_t)XFER_CHUNKS * ABSMAX_BLOCKS);
            double *partial = tmp + n;
            long long *dst = (long long *)member_buf(g, member, which);
            const size_t pitch = g.pitch_bytes[0] / 8;
            const size_t nx = (size_t)g.desc.nx;
            const int e0 = g.fix_exp;
            xfer_init(g);
            // the copies wait for earlier work of the grid (the staging buffer)
            LGD_CHECK_CUDA(cudaMemsetAsync(g.d_fixmax + 1, 0, sizeof(unsigned long long), g.stream));
            LGD_CHECK_CUDA(cudaEventRecord(g.xfer_ev[XFER_CHUNKS], g.stream));
            LGD_CHECK_CUDA(cudaStreamWaitEvent(g.xfer_stream, g.xfer_ev[XFER_CHUNKS], 0));
            for (int k = 0; k < K; ++k) {
                const size_t r0 = rows * k / K, r1 = rows * (k + 1) / K;
                LGD_CHECK_CUDA(cudaMemcpyAsync(tmp + r0 * nx, (const double *)host + r0 * nx, (r1 - r0) * nx * 8,
                                               cudaMemcpyHostToDevice, g.xfer_stream));
                LGD_CHECK_CUDA(cudaEventRecord(g.xfer_ev[k], g.xfer_stream));
                LGD_CHECK_CUDA(cudaStreamWaitEvent(g.stream, g.xfer_ev[k], 0));
                absmax_kernel<<<ABSMAX_BLOCKS, 256, 0, g.stream>>>(tmp + r0 * nx, (long long)((r1 - r0) * nx),
                                                                   partial + (size_t)k * ABSMAX_BLOCKS, g.d_fixmax + 1);
                check_launch("max |value|");
                to_fix_pitched_kernel<<<152 * 2, 256, 0, g.stream>>>(tmp + r0 * nx, dst + r0 * pitch, g.desc.nx,
                                                                    (long long)(r1 - r0), (long long)pitch, e0);
                check_launch("to fixed point");
                g.launches += 2;
            }
            std::vector<double> hpart((size_t)K * ABSMAX_BLOCKS);
            unsigned long long negative = 0;
            LGD_CHECK_CUDA(cudaMemcpyAsync(hpart.data(), partial, sizeof(double) * hpart.size(), cudaMemcpyDeviceToHost,
                                           g.stream));
            LGD_CHECK_CUDA(cudaMemcpyAsync(&negative, g.d_fixmax + 1, sizeof(negative), cudaMemcpyDeviceToHost,
                                           g.stream));
            LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
            // sticky: once a grid has held a negative value its steps keep
            // the sign handling (the results do not depend on it)
            if (negative) g.fix_nonneg = false;
            double m = std::fabs(g.desc.edge[0]);
            for (double v : hpart) m = std::fmax(m, v);
            LGD_REQUIRE(std::isfinite(m), LGD_ERR_INVALID, "grid holds a non-finite value");
            if (exp_bound(m) > g.fix_exp) {
                raise_fix_exp(g, exp_bound(m));
                to_fix_pitched_kernel<<<152 * 8, 256, 0, g.stream>>>(tmp, dst, g.desc.nx, (long long)rows,
                                                                    (long long)pitch, g.fix_exp);
                check_launch("to fixed point");
                ++g.launches;
                LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
            }
            // values well below the exponent's range: lower it (both
            // buffers), then convert the doubles again at the new scale so
            // that no fraction bit is lost at the boundary.  An upload whose
            // maximum needs the current exponent (m in [2^(e-1), 2^e))
            // keeps it: the buffers' maximum then has its top fraction bit
            // set, and a scan of both buffers would find nothing to lower.
            if (m > 0.0 && exp_bound(m) >= g.fix_exp) return;
            const int e_before = g.fix_exp;
            lower_fix_exp(g);
            if (g.fix_exp < e_before) {
                to_fix_pitched_kernel<<<152 * 8, 256, 0, g.stream>>>(tmp, dst, g.desc.nx, (long long)rows,
                                                                    (long long)pitch, g.fix_exp);
                check_launch("to fixed point");
                ++g.launches;
                LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
            }
            return;
        }
        LGD_CHECK_CUDA(cudaMemcpy2DAsync(member_buf(g, member, which), g.pitch_bytes[member], host,
                                         (size_t)g.desc.nx * helem, (size_t)g.desc.nx * helem, rows,
                                         cudaMemcpyHostToDevice, g.stream));
        LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
    });
}

int lgd_gpu_download(lgd_handle *h, int member, int which, void *host, size_t bytes)
{
    return guard([&] {
        Grid& g = grid_of(h);
        check_member(g, member, which);
        const size_t n = cells_of(g);
        const int helem = g.m[member].elem;
        LGD_REQUIRE(host != nullptr, LGD_ERR_INVALID, "null host buffer");
        LGD_REQUIRE(bytes == n * helem, LGD_ERR_INVALID, "byte count does not match the grid");
        const size_t rows = (size_t)g.desc.ny * g.desc.nz;
        if (g.desc.cell == LGD_CELL_JACOBI7_F64_FIX) {
            // convert row chunks on the grid's stream, copy each out on the
            // transfer stream as soon as it is converted
            const int K = (int)std::min<size_t>(XFER_CHUNKS, rows);
            double *tmp = staging(g, n * 8);
            const long long *src = (const long long *)member_buf(g, member, which);
            const size_t pitch = g.pitch_bytes[0] / 8;
            const size_t nx = (size_t)g.desc.nx;
            xfer_init(g);
            for (int k = 0; k < K; ++k) {
                const size_t r0 = rows * k / K, r1 = rows * (k + 1) / K;
                from_fix_pitched_kernel<<<152 * 2, 256, 0, g.stream>>>(src + r0 * pitch, tmp + r0 * nx, g.desc.nx,
                                                                      (long long)(r1 - r0), (long long)pitch, g.fix_exp);
                check_launch("from fixed point");
                ++g.launches;
                LGD_CHECK_CUDA(cudaEventRecord(g.xfer_ev[k], g.stream));
                LGD_CHECK_CUDA(cudaStreamWaitEvent(g.xfer_stream, g.xfer_ev[k], 0));
                LGD_CHECK_CUDA(cudaMemcpyAsync((double *)host + r0 * nx, tmp + r0 * nx, (r1 - r0) * nx * 8,
                                               cudaMemcpyDeviceToHost, g.xfer_stream));
            }
            // later work of the grid (which may reuse the staging buffer)
            // waits for the copies
            LGD_CHECK_CUDA(cudaEventRecord(g.xfer_ev[XFER_CHUNKS], g.xfer_stream));
            LGD_CHECK_CUDA(cudaStreamWaitEvent(g.stream, g.xfer_ev[XFER_CHUNKS], 0));
            LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
            check_device_error(g);
            return;
        }
        LGD_CHECK_CUDA(cudaMemcpy2DAsync(host, (size_t)g.desc.nx * helem, member_buf(g, member, which),
                                         g.pitch_bytes[member], (size_t)g.desc.nx * helem, rows,
                                         cudaMemcpyDeviceToHost, g.stream));
        LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
        check_device_error(g);
    });
}

int lgd_gpu_write_bov(lgd_handle *h, int member, const char *prefix, unsigned step, const char *variable)
{
    return guard([&] {
        Grid& g = grid_of(h);
        check_member(g, member, 0);
        LGD_REQUIRE(prefix != nullptr && variable != nullptr, LGD_ERR_INVALID, "null file prefix or variable name");
        const size_t n = cells_of(g);
        const int elem = g.m[member].elem;
        LGD_REQUIRE(g.desc.cell != LGD_CELL_RECORD && (elem == 1 || elem == 4 || elem == 8), LGD_ERR_UNSUPPORTED,
                    "BOV holds scalar members only");
        std::vector<unsigned char> data(n * elem);
        const int rc = lgd_gpu_download(h, member, 0, data.data(), data.size());
        LGD_REQUIRE(rc == LGD_OK, rc, "download for the BOV snapshot failed");
        const char *format = (elem == 8) ? "DOUBLE" : (elem == 4) ? "FLOAT" : "BYTE";
        char stepbuf[32];
        std::snprintf(stepbuf, sizeof(stepbuf), "%05u", step);
        const std::string stem = std::string(prefix) + "." + stepbuf;
        const std::string header_name = stem + ".bov";
        const std::string data_name = stem + ".data";
        char dims[96];
        std::snprintf(dims, sizeof(dims), "%d %d %d", g.desc.nx, g.desc.ny, g.desc.nz);
        const std::string header = std::string("TIME: ") + std::to_string(step) + "\n" + "DATA_FILE: " + data_name + "\n" +
                                   "DATA_SIZE: " + dims + "\n" + "DATA_FORMAT: " + format + "\n" + "VARIABLE: " +
                                   variable + "\n" + "DATA_ENDIAN: LITTLE\n" + "BRICK_ORIGIN: 0 0 0\n" +
                                   "BRICK_SIZE: " + dims + "\n" + "DIVIDE_BRICK: true\n" + "DATA_BRICKLETS: " + dims +
                                   "\n" + "DATA_COMPONENTS: 1\n";
        FILE *f = std::fopen(header_name.c_str(), "wb");
        LGD_REQUIRE(f != nullptr, LGD_ERR_INVALID, "cannot open " + header_name);
        const bool ok1 = std::fwrite(header.data(), 1, header.size(), f) == header.size();
        const bool ok2 = std::fclose(f) == 0;
        LGD_REQUIRE(ok1 && ok2, LGD_ERR_INVALID, "cannot write " + header_name);
        f = std::fopen(data_name.c_str(), "wb");
        LGD_REQUIRE(f != nullptr, LGD_ERR_INVALID, "cannot open " + data_name);
        const bool ok3 = std::fwrite(data.data(), 1, data.size(), f) == data.size();
        const bool ok4 = std::fclose(f) == 0;
        LGD_REQUIRE(ok3 && ok4, LGD_ERR_INVALID, "cannot write " + data_name);
    });
}

// Snapshot (checkpoint) files in the layout of the reference's MPIIO
// (io/mpiio.h:85-125 writeRegion, :180-200 offset and getLengths): the
// dimensions as DIM 32-bit ints (x, y[, z]), the step and the maximum step
// count as 32-bit unsigned, the edge cell, then every cell at header +
// index * cell bytes, index x fastest.  A cell record is the grid's members
// in order, each in its host type (the reference writes sizeof(CELL)
// bytes: the same for cells without padding).
static size_t cell_record_bytes(const Grid& g)
{
    size_t b = 0;
    for (int m = 0; m < g.n_members; ++m) b += (size_t)g.m[m].elem;
    return b;
}

static void member_edge_bytes(const Grid& g, int m, unsigned char *out)
{
    const double e = g.desc.edge[m];
    const int elem = g.m[m].elem;
    if (g.desc.cell == LGD_CELL_RECORD) {
        std::memcpy(out, g.edge_record, (size_t)elem);
    } else if (g.desc.cell == LGD_CELL_TEST) {
        // the reference TestInitializer's edge cell: position -1 on every
        // axis, the grid's dimensions, cycle 0, test value 666
        TestRec r;
        std::memset(&r, 0, sizeof(r));
        const int dims[3] = {g.desc.nx, g.desc.ny, g.desc.nz};
        for (int a = 0; a < 3; ++a) {
            r.pos[a] = a < g.desc.dim ? -1 : 0;
            r.dim[a] = a < g.desc.dim ? dims[a] : 1;
        }
        r.valid = (unsigned char)((int)e & 1);
        r.edge = (unsigned char)(((int)e >> 1) & 1);
        r.test_value = 666.0f;
        std::memcpy(out, &r, sizeof(r));
    } else if (elem == 8) {
        std::memcpy(out, &e, 8);
    } else if (elem == 4) {
        const float f = (float)e;
        std::memcpy(out, &f, 4);
    } else {
        out[0] = (unsigned char)(e != 0.0);
    }
}

static std::vector<unsigned char> snapshot_header(const Grid& g, unsigned step, unsigned max_steps)
{
    const int dims[3] = {g.desc.nx, g.desc.ny, g.desc.nz};
    std::vector<unsigned char> h(4 * (size_t)g.desc.dim + 8 + cell_record_bytes(g));
    std::memcpy(h.data(), dims, 4 * (size_t)g.desc.dim);
    std::memcpy(h.data() + 4 * g.desc.dim, &step, 4);
    std::memcpy(h.data() + 4 * g.desc.dim + 4, &max_steps, 4);
    size_t off = 4 * (size_t)g.desc.dim + 8;
    for (int m = 0; m < g.n_members; ++m) {
        member_edge_bytes(g, m, h.data() + off);
        off += (size_t)g.m[m].elem;
    }
    return h;
}

int lgd_gpu_write_snapshot(lgd_handle *h, const char *path, unsigned step, unsigned max_steps)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(path != nullptr, LGD_ERR_INVALID, "null file name");
        const size_t n = cells_of(g);
        const size_t rec = cell_record_bytes(g);
        std::vector<unsigned char> cells(n * rec);
        size_t moff = 0;
        for (int m = 0; m < g.n_members; ++m) {
            const size_t elem = (size_t)g.m[m].elem;
            std::vector<unsigned char> data(n * elem);
            const int rc = lgd_gpu_download(h, m, 0, data.data(), data.size());
            LGD_REQUIRE(rc == LGD_OK, rc, "download for the snapshot failed");
            for (size_t i = 0; i < n; ++i) std::memcpy(&cells[i * rec + moff], &data[i * elem], elem);
            moff += elem;
        }
        const std::vector<unsigned char> header = snapshot_header(g, step, max_steps);
        FILE *f = std::fopen(path, "wb");
        LGD_REQUIRE(f != nullptr, LGD_ERR_INVALID, std::string("cannot open ") + path);
        const bool ok1 = std::fwrite(header.data(), 1, header.size(), f) == header.size();
        const bool ok2 = std::fwrite(cells.data(), 1, cells.size(), f) == cells.size();
        const bool ok3 = std::fclose(f) == 0;
        LGD_REQUIRE(ok1 && ok2 && ok3, LGD_ERR_INVALID, std::string("cannot write ") + path);
    });
}

int lgd_snapshot_info(const char *path, int dim, int *dims, unsigned *step, unsigned *max_steps)
{
    return guard([&] {
        LGD_REQUIRE(path != nullptr && dims != nullptr && step != nullptr && max_steps != nullptr, LGD_ERR_INVALID,
                    "null argument");
        LGD_REQUIRE(dim == 2 || dim == 3, LGD_ERR_INVALID, "dim must be 2 or 3");
        FILE *f = std::fopen(path, "rb");
        LGD_REQUIRE(f != nullptr, LGD_ERR_INVALID, std::string("cannot open ") + path);
        int d[3] = {0, 0, 1};
        unsigned meta[2] = {0, 0};
        const bool ok = std::fread(d, 4, (size_t)dim, f) == (size_t)dim && std::fread(meta, 4, 2, f) == 2;
        std::fclose(f);
        LGD_REQUIRE(ok, LGD_ERR_INVALID, std::string("snapshot header too short: ") + path);
        for (int i = 0; i < dim; ++i) dims[i] = d[i];
        *step = meta[0];
        *max_steps = meta[1];
    });
}

int lgd_gpu_read_snapshot(lgd_handle *h, const char *path, unsigned *step, unsigned *max_steps)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(path != nullptr, LGD_ERR_INVALID, "null file name");
        const size_t n = cells_of(g);
        const size_t rec = cell_record_bytes(g);
        const std::vector<unsigned char> expect = snapshot_header(g, 0, 0);
        std::vector<unsigned char> header(expect.size());
        FILE *f = std::fopen(path, "rb");
        LGD_REQUIRE(f != nullptr, LGD_ERR_INVALID, std::string("cannot open ") + path);
        std::vector<unsigned char> cells(n * rec);
        const bool ok1 = std::fread(header.data(), 1, header.size(), f) == header.size();
        const bool ok2 = ok1 && std::fread(cells.data(), 1, cells.size(), f) == cells.size();
        std::fclose(f);
        LGD_REQUIRE(ok1, LGD_ERR_INVALID, std::string("snapshot header too short: ") + path);
        const size_t dbytes = 4 * (size_t)g.desc.dim;
        LGD_REQUIRE(std::memcmp(header.data(), expect.data(), dbytes) == 0, LGD_ERR_INVALID,
                    "snapshot dimensions differ from the grid's");
        LGD_REQUIRE(std::memcmp(header.data() + dbytes + 8, expect.data() + dbytes + 8, rec) == 0, LGD_ERR_INVALID,
                    "snapshot edge cell differs from the grid's");
        LGD_REQUIRE(ok2, LGD_ERR_INVALID, std::string("snapshot holds fewer cells than the grid: ") + path);
        size_t moff = 0;
        for (int m = 0; m < g.n_members; ++m) {
            const size_t elem = (size_t)g.m[m].elem;
            std::vector<unsigned char> data(n * elem);
            for (size_t i = 0; i < n; ++i) std::memcpy(&data[i * elem], &cells[i * rec + moff], elem);
            const int rc = lgd_gpu_upload(h, m, 0, data.data(), data.size());
            LGD_REQUIRE(rc == LGD_OK, rc, "upload of the snapshot failed");
            moff += elem;
        }
        if (step) std::memcpy(step, header.data() + dbytes, 4);
        if (max_steps) std::memcpy(max_steps, header.data() + dbytes + 4, 4);
    });
}

static void device_copy(lgd_handle *h, int member, int which, void *dev, size_t bytes, bool to_grid)
{
    Grid& g = grid_of(h);
    check_member(g, member, which);
    LGD_REQUIRE(g.desc.cell != LGD_CELL_JACOBI7_F64_FIX, LGD_ERR_UNSUPPORTED,
                "device copies of the fixed-point grid are not supported");
    const size_t n = cells_of(g);
    const size_t elem = (size_t)g.m[member].elem;
    LGD_REQUIRE(dev != nullptr, LGD_ERR_INVALID, "null device buffer");
    LGD_REQUIRE(bytes == n * elem, LGD_ERR_INVALID, "byte count does not match the grid");
    const size_t rows = (size_t)g.desc.ny * g.desc.nz;
    const size_t row_bytes = (size_t)g.desc.nx * elem;
    if (to_grid) {
        LGD_CHECK_CUDA(cudaMemcpy2DAsync(member_buf(g, member, which), g.pitch_bytes[member], dev, row_bytes, row_bytes,
                                         rows, cudaMemcpyDeviceToDevice, g.stream));
    } else {
        LGD_CHECK_CUDA(cudaMemcpy2DAsync(dev, row_bytes, member_buf(g, member, which), g.pitch_bytes[member], row_bytes,
                                         rows, cudaMemcpyDeviceToDevice, g.stream));
    }
    LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
}

static void region_copy(lgd_handle *h, int member, const int *streaks, int n_streaks, void *host,
                        size_t bytes, bool to_grid)
{
    Grid& g = grid_of(h);
    check_member(g, member, 0);
    const long long cells = stage_streaks(g, streaks, n_streaks);
    const int elem = g.m[member].elem;
    LGD_REQUIRE(bytes == (size_t)cells * elem, LGD_ERR_INVALID, "byte count does not match the streaks");
    if (cells == 0) return;
    LGD_REQUIRE(host != nullptr, LGD_ERR_INVALID, "null host buffer");
    const bool fix = g.desc.cell == LGD_CELL_JACOBI7_F64_FIX;
    if (fix && to_grid) {
        // values the exponent cannot hold raise it first; negative ones end
        // the sign-free fast path
        const double *v = static_cast<const double *>(host);
        double m = 0.0;
        bool neg = false;
        for (long long i = 0; i < cells; ++i) {
            LGD_REQUIRE(std::isfinite(v[i]), LGD_ERR_INVALID, "grid holds a non-finite value");
            m = std::fmax(m, std::fabs(v[i]));
            neg |= v[i] < 0.0;
        }
        if (neg) g.fix_nonneg = false;
        if (exp_bound(m) > g.fix_exp) raise_fix_exp(g, exp_bound(m));
    }
    void *d = nullptr;
    LGD_CHECK_CUDA(cudaMallocAsync(&d, bytes, g.stream));
    if (to_grid) {
        LGD_CHECK_CUDA(cudaMemcpyAsync(d, host, bytes, cudaMemcpyHostToDevice, g.stream));
    }
    if (fix) {
        // FP64 values at the boundary, fixed point on the device
        launch_streak_copy_fix(g, g.d_streaks, g.d_streak_prefix, n_streaks, cells, (double *)d, to_grid);
    } else {
        launch_streak_copy(g, member, 0, g.d_streaks, g.d_streak_prefix, n_streaks, cells, d, to_grid);
    }
    if (!to_grid) {
        LGD_CHECK_CUDA(cudaMemcpyAsync(host, d, bytes, cudaMemcpyDeviceToHost, g.stream));
    }
    LGD_CHECK_CUDA(cudaFreeAsync(d, g.stream));
    LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
}

int lgd_gpu_upload_device(lgd_handle *h, int member, int which, const void *dev, size_t bytes)
{
    return guard([&] { device_copy(h, member, which, const_cast<void *>(dev), bytes, true); });
}

int lgd_gpu_download_device(lgd_handle *h, int member, int which, void *dev, size_t bytes)
{
    return guard([&] { device_copy(h, member, which, dev, bytes, false); });
}

int lgd_gpu_save_region(lgd_handle *h, int member, const int *streaks, int n_streaks, void *host, size_t bytes)
{
    return guard([&] { region_copy(h, member, streaks, n_streaks, host, bytes, false); });
}

int lgd_gpu_load_region(lgd_handle *h, int member, const int *streaks, int n_streaks, const void *host, size_t bytes)
{
    return guard([&] { region_copy(h, member, streaks, n_streaks, const_cast<void *>(host), bytes, true); });
}

int lgd_gpu_step(lgd_handle *h, unsigned nano_step, int count)
{
    // the compiled cells have one nano step, except the test cell, whose
    // updates run nano steps nano_step, nano_step + 1, ...
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(count >= 0, LGD_ERR_INVALID, "negative step count");
        LGD_REQUIRE(g.desc.cell != LGD_CELL_RECORD, LGD_ERR_UNSUPPORTED,
                    "record grids run the cell's own update() through gb300cell.cuh");
        if (count == 0) return;
        switch (g.desc.cell) {
        case LGD_CELL_JACOBI7_F64:
        case LGD_CELL_JACOBI7_F32:
            launch_jacobi7(g, count);
            break;
        case LGD_CELL_JACOBI7_F64_FIX:
            // the exponent follows a decaying grid down: checked after every
            // FIX_CHECK_STEPS steps (one read of both buffers and a wait),
            // also inside a long call
            while (count > 0) {
                const int k = std::min(count, std::max(1, FIX_CHECK_STEPS - g.fix_steps_unchecked));
                launch_jacobi7(g, k);
                g.fix_steps_unchecked += k;
                count -= k;
                if (g.fix_steps_unchecked >= FIX_CHECK_STEPS) lower_fix_exp(g);
            }
            break;
        case LGD_CELL_GOL_U8:
            launch_gol(g, count);
            break;
        case LGD_CELL_VARCOEF_F32:
        case LGD_CELL_VARCOEF_F64:
            launch_varcoef(g, count);
            break;
        default: {
            // cells without a whole-grid kernel: region update over all rows
            std::vector<int> streaks;
            streaks.reserve((size_t)g.desc.ny * g.desc.nz * 4);
            for (int z = 0; z < g.desc.nz; ++z) {
                for (int y = 0; y < g.desc.ny; ++y) {
                    streaks.push_back(0);
                    streaks.push_back(y);
                    streaks.push_back(z);
                    streaks.push_back(g.desc.nx);
                }
            }
            const int n = (int)(streaks.size() / 4);
            const long long cells = stage_streaks(g, streaks.data(), n);
            for (int s = 0; s < count; ++s) {
                launch_region(g, g.d_streaks, g.d_streak_prefix, n, cells, nano_step + (unsigned)s);
                g.cur = 1 - g.cur;
            }
        }
        }
    });
}

int lgd_gpu_update_region(lgd_handle *h, const int *streaks, int n_streaks, unsigned nano_step)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(g.desc.cell != LGD_CELL_RECORD, LGD_ERR_UNSUPPORTED,
                    "record grids run the cell's own update() through gb300cell.cuh");
        const long long cells = stage_streaks(g, streaks, n_streaks);
        launch_region(g, g.d_streaks, g.d_streak_prefix, n_streaks, cells, nano_step);
    });
}

int lgd_gpu_swap(lgd_handle *h)
{
    return guard([&] {
        Grid& g = grid_of(h);
        g.cur = 1 - g.cur;
    });
}

int lgd_gpu_fill_uniform(lgd_handle *h, int member, int which, uint64_t seed, int stream)
{
    return guard([&] {
        Grid& g = grid_of(h);
        check_member(g, member, which);
        LGD_REQUIRE(g.desc.cell != LGD_CELL_RECORD && g.m[member].elem != 1, LGD_ERR_INVALID,
                    "uniform fill needs a floating-point member");
        if (g.desc.cell == LGD_CELL_JACOBI7_F64_FIX) {
            raise_fix_exp(g, 0);   // uniform values lie in [0, 1)
            launch_fill(g, member, which, seed, stream, 2, 0.0, g.fix_exp);
            const int e_before = g.fix_exp;
            lower_fix_exp(g);
            if (g.fix_exp < e_before) launch_fill(g, member, which, seed, stream, 2, 0.0, g.fix_exp);
        } else {
            launch_fill(g, member, which, seed, stream, 0, 0.0, 0);
        }
        LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
    });
}

int lgd_gpu_fill_bernoulli(lgd_handle *h, int member, int which, uint64_t seed, int stream, double p)
{
    return guard([&] {
        Grid& g = grid_of(h);
        check_member(g, member, which);
        LGD_REQUIRE(g.desc.cell != LGD_CELL_RECORD && g.m[member].elem == 1, LGD_ERR_INVALID,
                    "Bernoulli fill needs a uint8 member");
        launch_fill(g, member, which, seed, stream, 1, p, 0);
        LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
    });
}

int lgd_gpu_checksum(lgd_handle *h, int member, int which, double *sum)
{
    return guard([&] {
        Grid& g = grid_of(h);
        check_member(g, member, which);
        LGD_REQUIRE(sum != nullptr, LGD_ERR_INVALID, "null output");
        LGD_REQUIRE(g.desc.cell != LGD_CELL_RECORD, LGD_ERR_UNSUPPORTED, "records have no numeric sum");
        // the checksum kernel reads through the current/next view
        const int saved = g.cur;
        if (which == 1 && !g.m[member].is_static) g.cur = 1 - g.cur;
        try {
            launch_checksum(g, member, 0, sum);
        } catch (...) {
            g.cur = saved;
            throw;
        }
        g.cur = saved;
    });
}

int lgd_gpu_test_bounded_waits(lgd_handle *h, long long wait_cycles, int skip_plane)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(wait_cycles >= 0 && skip_plane >= -1, LGD_ERR_INVALID, "negative wait bound or plane");
        g.test_wait_cycles = wait_cycles;
        g.test_skip_plane = skip_plane + 1;
    });
}

int lgd_gpu_synchronize(lgd_handle *h)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_CHECK_CUDA(cudaStreamSynchronize(g.stream));
        check_device_error(g);
    });
}

int lgd_gpu_device_ptr(lgd_handle *h, int member, int which, void **ptr, size_t *pitch_bytes)
{
    return guard([&] {
        Grid& g = grid_of(h);
        check_member(g, member, which);
        LGD_REQUIRE(ptr != nullptr, LGD_ERR_INVALID, "null output");
        *ptr = member_buf(g, member, which);
        if (pitch_bytes) *pitch_bytes = g.pitch_bytes[member];
    });
}

int lgd_gpu_launch_count(lgd_handle *h, uint64_t *count)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(count != nullptr, LGD_ERR_INVALID, "null output");
        *count = g.launches;
    });
}

int lgd_gpu_set_time_block(lgd_handle *h, int depth)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(depth >= 0 && depth <= LGD_TB_MAX_DEPTH, LGD_ERR_INVALID, "time block depth out of range");
        g.time_block = depth;
    });
}

int lgd_gpu_set_time_block_shape(lgd_handle *h, int shape)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(shape >= 0 && shape <= 2, LGD_ERR_INVALID, "time block shape must lie in [0, 2]");
        g.tb_shape = shape;
    });
}

int lgd_gpu_set_variant(lgd_handle *h, int variant)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(variant >= 0 && variant <= 6, LGD_ERR_INVALID, "variant must lie in [0, 6]");
        g.variant = variant;
    });
}

int lgd_gpu_stream(lgd_handle *h, void **stream)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(stream != nullptr, LGD_ERR_INVALID, "null output");
        *stream = (void *)g.stream;
    });
}

int lgd_gpu_fixed_point_exponent(lgd_handle *h, int *exp)
{
    return guard([&] {
        Grid& g = grid_of(h);
        LGD_REQUIRE(exp != nullptr, LGD_ERR_INVALID, "null output");
        LGD_REQUIRE(g.desc.cell == LGD_CELL_JACOBI7_F64_FIX, LGD_ERR_INVALID, "not a fixed-point grid");
        *exp = g.fix_exp;
    });
}

}  // extern "C"
