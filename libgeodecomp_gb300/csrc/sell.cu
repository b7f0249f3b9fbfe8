// Unstructured grids in SELL-C-sigma form: the host-side builder and the
// device diffusion step x' = 0.1 x + W x.
//
// Builder.  The layout is the reference's, byte for byte, so that grids
// built by either side can be exchanged:
//   - ReorderingUnstructuredGrid::setWeights (storage/
//     reorderingunstructuredgrid.h:195-284): inside windows of sigma rows
//     the rows are stably sorted by decreasing length; physical row p holds
//     logical row perm[p]; column ids are remapped to physical ids;
//   - SellCSigmaSparseMatrixContainer / InitFromMatrix (storage/
//     sellcsigmasparsematrixcontainer.h:49-161): chunks of C rows,
//     chunkLength = longest row of the chunk, chunkOffset[c+1] =
//     chunkOffset[c] + C * chunkLength[c], entry k of row r at
//     chunkOffset[r / C] + k * C + r % C, a row's entries in ascending
//     (physical) column order, padding value 0 / column 0.
// The window sort here is a counting sort on the row length (stable by
// construction), the per-row column sort an insertion sort (rows are short).
//
// Kernel.  C = 32 puts one chunk on one warp: lane l owns row
// chunk * 32 + l, entry k of all 32 rows is one coalesced 256-byte load of
// values and a 128-byte load of columns, and the x[column] gathers hit L2
// (the FP64 vector of 4M nodes is 32 MiB).  Other C values use one thread
// per row with the same indexing.  Each lane stops at its own row length,
// as the reference's neighbourhood iterator does
// (storage/unstructuredneighborhood.h:154-170), so padding costs no traffic.
#include <algorithm>
#include <cstring>
#include <vector>

#include "lgd_internal.h"
#include "../../include/lgd_sell.h"

namespace lgd {

struct Sell {
    int n;                  // rows (nodes)
    int C;
    int n_chunks;
    int rows_padded;
    long long total;        // value slots
    int precision;          // 8 (FP64) or 4 (FP32)
    int flags;
    int *d_chunk_offset;    // n_chunks + 1
    int *d_row_length;      // rows_padded
    void *d_values;         // total, FP64 or FP32
    int *d_column;          // total
    void *d_x[2];           // rows_padded each
    int *d_perm;            // physical -> logical (n), or null
    int cur;
    int variant;            // kernel variant, see lgd_sell_set_variant
    cudaStream_t stream;
    uint64_t launches;
};

// -------------------------------------------------------------- kernels
template<typename R, bool EXACT>
__device__ __forceinline__ R madd(R acc, R a, R b);

template<>
__device__ __forceinline__ double madd<double, true>(double acc, double a, double b)
{
    return __dadd_rn(acc, __dmul_rn(a, b));
}

template<>
__device__ __forceinline__ double madd<double, false>(double acc, double a, double b)
{
    return fma(a, b, acc);
}

template<>
__device__ __forceinline__ float madd<float, false>(float acc, float a, float b)
{
    return fmaf(a, b, acc);
}

template<>
__device__ __forceinline__ float madd<float, true>(float acc, float a, float b)
{
    return __fadd_rn(acc, __fmul_rn(a, b));
}

// one thread per row; row = blockIdx * blockDim + thread, so a warp of 32
// consecutive rows is one chunk when C = 32
template<typename R, bool EXACT>
__global__ void __launch_bounds__(256)
sell_diffusion_kernel(const int *__restrict__ chunk_offset, const int *__restrict__ row_length,
                      const R *__restrict__ values, const int *__restrict__ column,
                      const R *__restrict__ x, R *__restrict__ xn, int n, int C, int row_begin, int row_end)
{
    const int row = row_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= row_end) return;
    const int chunk = row / C;
    const long long base = (long long)chunk_offset[chunk] + (row - chunk * C);
    const int len = row_length[row];
    R acc = (R)0;
    const R *v = values + base;
    const int *c = column + base;
    int k = 0;
    // two independent gathers in flight per iteration (measured faster on
    // GB300 than four with evict-first matrix loads: 0.25 vs 0.30 ms/step)
    for (; k + 1 < len; k += 2) {
        const R w0 = __ldg(v + (long long)k * C);
        const int c0 = __ldg(c + (long long)k * C);
        const R w1 = __ldg(v + (long long)(k + 1) * C);
        const int c1 = __ldg(c + (long long)(k + 1) * C);
        const R x0 = __ldg(x + c0);
        const R x1 = __ldg(x + c1);
        acc = madd<R, EXACT>(acc, x0, w0);
        acc = madd<R, EXACT>(acc, x1, w1);
    }
    if (k < len) {
        const R w0 = __ldg(v + (long long)k * C);
        const int c0 = __ldg(c + (long long)k * C);
        acc = madd<R, EXACT>(acc, __ldg(x + c0), w0);
    }
    // x' = 0.1 * x + acc
    if (EXACT) {
        xn[row] = (sizeof(R) == 8) ? (R)__dadd_rn(__dmul_rn(0.1, (double)x[row]), (double)acc)
                                   : (R)__fadd_rn(__fmul_rn(0.1f, (float)x[row]), (float)acc);
    } else {
        xn[row] = (R)0.1 * x[row] + acc;
    }
}

// Software-pipelined form: the matrix entries of slots k+D .. k+2D-1 are
// loaded while the x gathers of slots k .. k+D-1 are in flight, so a
// row's iterations cost one memory round trip each instead of a DRAM trip
// followed by a dependent L2 trip.  Slots below the chunk length exist for
// every lane of the chunk, lanes load only their own row's entries; the
// sum runs in slot order, as in the kernel above.
template<typename R, bool EXACT, int D>
__device__ __forceinline__ void sell_pipe_row(const int *__restrict__ chunk_offset, const int *__restrict__ row_length,
                                              const R *__restrict__ values, const int *__restrict__ column,
                                              const R *__restrict__ x, R *__restrict__ xn, int C, int row, int chunk)
{
    const long long cbase = chunk_offset[chunk];
    const long long base = cbase + (row - chunk * C);
    const int len = row_length[row];
    const R xr = x[row];
    const R *v = values + base;
    const int *c = column + base;
    R w[D];
    int cc[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
        w[j] = (R)0;
        cc[j] = 0;
        if (j < len) {
            w[j] = __ldg(v + (long long)j * C);
            cc[j] = __ldg(c + (long long)j * C);
        }
    }
    R acc = (R)0;
    for (int k = 0; k < len; k += D) {
        R g[D];
#pragma unroll
        for (int j = 0; j < D; ++j) g[j] = (k + j < len) ? __ldg(x + cc[j]) : (R)0;
        R nw[D];
        int nc[D];
#pragma unroll
        for (int j = 0; j < D; ++j) {
            nw[j] = (R)0;
            nc[j] = 0;
            if (k + D + j < len) {
                nw[j] = __ldg(v + (long long)(k + D + j) * C);
                nc[j] = __ldg(c + (long long)(k + D + j) * C);
            }
        }
#pragma unroll
        for (int j = 0; j < D; ++j) {
            if (k + j < len) acc = madd<R, EXACT>(acc, g[j], w[j]);
            w[j] = nw[j];
            cc[j] = nc[j];
        }
    }
    if (EXACT) {
        xn[row] = (sizeof(R) == 8) ? (R)__dadd_rn(__dmul_rn(0.1, (double)xr), (double)acc)
                                   : (R)__fadd_rn(__fmul_rn(0.1f, (float)xr), (float)acc);
    } else {
        xn[row] = (R)0.1 * xr + acc;
    }
}

// One thread per row.  The sigma-window sort puts a window's longest rows
// into its first chunk, so the chunks (warps) of one CTA finish at very
// different times and the CTA holds its slot until the longest is done;
// CTAs of 128 threads (four chunks) measured 0.207 ms per step on the
// 4M-node power-law matrix against 0.219 for 64 and 0.233 for 256 threads.
// Loads stay on the read-only path: hints that skip L1 on the gathers,
// keep x in L2 with evict_last or stream the matrix with evict_first, and
// an L2 bulk prefetch of each chunk, all measured slower.
template<typename R, bool EXACT, int D, int THREADS>
__global__ void __launch_bounds__(THREADS)
sell_diffusion_pipe_kernel(const int *__restrict__ chunk_offset, const int *__restrict__ row_length,
                           const R *__restrict__ values, const int *__restrict__ column,
                           const R *__restrict__ x, R *__restrict__ xn, int n, int C, int row_begin, int row_end)
{
    const int row = row_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= row_end) return;
    sell_pipe_row<R, EXACT, D>(chunk_offset, row_length, values, column, x, xn, C, row, row / C);
}

template<typename R>
__global__ void permute_in_kernel(const double *logical, const int *perm, R *phys, int n)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        phys[p] = (R)logical[perm ? perm[p] : p];
    }
}

template<typename R>
__global__ void permute_out_kernel(const R *phys, const int *perm, double *logical, int n)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        logical[perm ? perm[p] : p] = (double)phys[p];
    }
}

static Sell& sell_of(lgd_sell *h)
{
    LGD_REQUIRE(h != nullptr, LGD_ERR_INVALID, "null handle");
    return *reinterpret_cast<Sell *>(h);
}

static void sell_free(Sell& s)
{
    if (s.stream) cudaStreamSynchronize(s.stream);
    cudaFree(s.d_chunk_offset);
    cudaFree(s.d_row_length);
    cudaFree(s.d_values);
    cudaFree(s.d_column);
    cudaFree(s.d_x[0]);
    cudaFree(s.d_x[1]);
    cudaFree(s.d_perm);
    if (s.stream) cudaStreamDestroy(s.stream);
}

template<typename R, bool EXACT, int D, int THREADS>
static void launch_pipe(Sell& s, int row_begin, int row_end, const R *x, R *xn, const R *vals)
{
    const int blocks = (row_end - row_begin + THREADS - 1) / THREADS;
    sell_diffusion_pipe_kernel<R, EXACT, D, THREADS><<<blocks, THREADS, 0, s.stream>>>(
        s.d_chunk_offset, s.d_row_length, vals, s.d_column, x, xn, s.n, s.C, row_begin, row_end);
}

template<typename R, bool EXACT>
static void launch_sell_typed(Sell& s, int row_begin, int row_end)
{
    const R *x = (const R *)s.d_x[s.cur];
    R *xn = (R *)s.d_x[1 - s.cur];
    const R *vals = (const R *)s.d_values;
    switch (s.variant) {
    case 1: {
        const int threads = 256;
        const int blocks = (row_end - row_begin + threads - 1) / threads;
        sell_diffusion_kernel<R, EXACT><<<blocks, threads, 0, s.stream>>>(
            s.d_chunk_offset, s.d_row_length, vals, s.d_column, x, xn, s.n, s.C, row_begin, row_end);
        break;
    }
    case 2: launch_pipe<R, EXACT, 2, 256>(s, row_begin, row_end, x, xn, vals); break;
    case 3: launch_pipe<R, EXACT, 4, 64>(s, row_begin, row_end, x, xn, vals); break;
    case 4: launch_pipe<R, EXACT, 4, 256>(s, row_begin, row_end, x, xn, vals); break;
    case 5: launch_pipe<R, EXACT, 8, 64>(s, row_begin, row_end, x, xn, vals); break;
    default: launch_pipe<R, EXACT, 4, 128>(s, row_begin, row_end, x, xn, vals); break;
    }
}

static void launch_sell(Sell& s, int row_begin, int row_end)
{
    if (row_end <= row_begin) return;
    const bool exact = (s.flags & LGD_SELL_EXACT) != 0;
    if (s.precision == 8) {
        if (exact) {
            launch_sell_typed<double, true>(s, row_begin, row_end);
        } else {
            launch_sell_typed<double, false>(s, row_begin, row_end);
        }
    } else {
        if (exact) {
            launch_sell_typed<float, true>(s, row_begin, row_end);
        } else {
            launch_sell_typed<float, false>(s, row_begin, row_end);
        }
    }
    check_launch("sell diffusion");
    ++s.launches;
}


// ------------------------------------------------------- builder on the GPU
// The same layout as lgd_sell_plan + lgd_sell_fill, built by kernels:
//   1. row lengths from row_ptr (checked: non-decreasing, at most
//      LGD_SELL_GPU_MAX_ROW);
//   2. per sigma-window a stable sort by decreasing length: one CTA sorts
//      the keys ((MAX_ROW - length) << 12 | index in window) with a bitonic
//      network in shared memory - unique keys, so the order is the stable
//      one of the host's counting sort;
//   3. row_length[p] = length of perm[p], the inverse permutation;
//   4. chunk lengths, then one CTA scans C * chunk length into chunk_offset;
//   5. one warp per physical row ranks the row's entries by (physical
//      column, position) - the host's stable insertion sort - and writes
//      value and column to chunk_offset[p / C] + rank * C + p % C.
// Errors (bad row_ptr, a column outside the node set, a row too long, more
// than 2^31-1 slots) set bits of a device word that the host checks.
namespace sbuild {

constexpr int SORT_THREADS = 512;
constexpr int KEY_BITS = 12;                 // index inside a window: sigma <= 4096

enum { E_ROWPTR = 1, E_LONGROW = 2, E_COLUMN = 4, E_TOTAL = 8 };

__global__ void lengths_kernel(const int64_t *__restrict__ row_ptr, int n, int *__restrict__ len, int *err)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const long long d = row_ptr[r + 1] - row_ptr[r];
        if (d < 0 || (r == 0 && row_ptr[0] != 0)) {
            atomicOr(err, E_ROWPTR);
            len[r] = 0;
        } else if (d > LGD_SELL_GPU_MAX_ROW) {
            atomicOr(err, E_LONGROW);
            len[r] = 0;
        } else {
            len[r] = (int)d;
        }
    }
}

// one CTA per window [w0, w0 + cnt); P = the window padded to a power of two
__global__ void __launch_bounds__(SORT_THREADS)
window_sort_kernel(const int *__restrict__ len, int n, int sigma, int P, int *__restrict__ perm)
{
    extern __shared__ uint32_t keys[];
    const int w0 = blockIdx.x * sigma;
    const int cnt = min(sigma, n - w0);
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        keys[i] = (i < cnt) ? ((uint32_t)(LGD_SELL_GPU_MAX_ROW - len[w0 + i]) << KEY_BITS) | (uint32_t)i : 0xffffffffu;
    }
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const uint32_t a = keys[i], b = keys[l];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        perm[w0 + i] = w0 + (int)(keys[i] & ((1u << KEY_BITS) - 1));
    }
}

__global__ void row_length_kernel(const int *__restrict__ len, const int *__restrict__ perm, int n, int rows_padded,
                                  int *__restrict__ row_length, int *__restrict__ inv)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < rows_padded; p += gridDim.x * blockDim.x) {
        if (p < n) {
            const int r = perm[p];
            row_length[p] = len[r];
            inv[r] = p;
        } else {
            row_length[p] = 0;
        }
    }
}

// chunk_offset[c] = sum of C * max row length over the chunks before c, one
// CTA of 1024 threads, each scanning a contiguous run of chunks
__global__ void __launch_bounds__(1024)
chunk_scan_kernel(const int *__restrict__ row_length, int C, int n_chunks, int *__restrict__ chunk_offset,
                  long long *total, int *err)
{
    __shared__ long long part[1024];
    const int t = threadIdx.x;
    const int per = (n_chunks + 1023) / 1024;
    const int c0 = min(n_chunks, t * per);
    const int c1 = min(n_chunks, c0 + per);
    long long sum = 0;
    for (int c = c0; c < c1; ++c) {
        int m = 0;
        for (int l = 0; l < C; ++l) m = max(m, row_length[c * C + l]);
        sum += (long long)m * C;
    }
    part[t] = sum;
    __syncthreads();
    if (t == 0) {
        long long acc = 0;
        for (int i = 0; i < 1024; ++i) {
            const long long v = part[i];
            part[i] = acc;
            acc += v;
        }
        *total = acc;
        if (acc > 0x7fffffffLL) atomicOr(err, E_TOTAL);
        chunk_offset[n_chunks] = (int)min(acc, 0x7fffffffLL);
    }
    __syncthreads();
    long long acc = part[t];
    for (int c = c0; c < c1; ++c) {
        chunk_offset[c] = (int)min(acc, 0x7fffffffLL);
        int m = 0;
        for (int l = 0; l < C; ++l) m = max(m, row_length[c * C + l]);
        acc += (long long)m * C;
    }
}

// one warp per physical row: rank the row's entries by (physical column,
// position) and place them
template<typename R>
__global__ void __launch_bounds__(256)
fill_kernel(const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ col, const double *__restrict__ w,
            const int *__restrict__ perm, const int *__restrict__ inv, const int *__restrict__ chunk_offset, int n,
            int C, long long total, R *__restrict__ values, int *__restrict__ column, int *err)
{
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long p = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); p < n; p += warps) {
        const int r = perm[p];
        const long long b = row_ptr[r];
        const long long dl = row_ptr[r + 1] - b;
        const int d = (int)(dl < LGD_SELL_GPU_MAX_ROW ? dl : LGD_SELL_GPU_MAX_ROW);
        const long long base = (long long)chunk_offset[p / C] + p % C;
        const int tiles = (d + 31) / 32;
        // key of entry e: physical column in the high word, position low
        auto key_of = [&](int e) -> unsigned long long {
            if (e >= d) return ~0ull;
            const int c = col[b + e];
            const int pc = (c >= 0 && c < n) ? inv[c] : 0;
            return ((unsigned long long)(unsigned)pc << 32) | (unsigned)e;
        };
        for (int a = 0; a < tiles; ++a) {
            const int e = a * 32 + lane;
            const unsigned long long ke = key_of(e);
            int rank = 0;
            for (int t = 0; t < tiles; ++t) {
                const unsigned long long kt = key_of(t * 32 + lane);
#pragma unroll 8
                for (int sft = 0; sft < 32; ++sft) {
                    rank += (__shfl_sync(0xffffffffu, kt, sft) < ke) ? 1 : 0;
                }
            }
            if (e < d) {
                const int c = col[b + e];
                if (c < 0 || c >= n) atomicOr(err, E_COLUMN);
                const long long slot = base + (long long)rank * C;
                if (slot < total) {
                    values[slot] = (R)w[b + e];
                    column[slot] = (int)(ke >> 32);
                }
            }
        }
    }
}

}  // namespace sbuild
}  // namespace lgd

using namespace lgd;

extern "C" {

int lgd_sell_plan(int n, const int64_t *row_ptr, int C, int sigma, int32_t *perm, int32_t *row_length,
                  int32_t *chunk_length, int32_t *chunk_offset, int64_t *total)
{
    return guard([&] {
        LGD_REQUIRE(n > 0, LGD_ERR_INVALID, "node count must be positive");
        LGD_REQUIRE(C >= 1 && sigma >= 1, LGD_ERR_INVALID, "C and sigma must be at least 1");
        LGD_REQUIRE(row_ptr && perm && row_length && chunk_length && chunk_offset && total, LGD_ERR_INVALID,
                    "null argument");
        LGD_REQUIRE(row_ptr[0] == 0, LGD_ERR_INVALID, "row_ptr[0] must be 0");
        int max_len = 0;
        for (int r = 0; r < n; ++r) {
            const long long d = row_ptr[r + 1] - row_ptr[r];
            LGD_REQUIRE(d >= 0 && d <= (1 << 30), LGD_ERR_INVALID, "row_ptr must be non-decreasing");
            max_len = std::max(max_len, (int)d);
        }
        // stable counting sort by decreasing length inside each window
        std::vector<int> count(max_len + 2);
        for (int w0 = 0; w0 < n; w0 += sigma) {
            const int cnt = std::min(sigma, n - w0);
            std::fill(count.begin(), count.end(), 0);
            for (int i = 0; i < cnt; ++i) {
                const int d = (int)(row_ptr[w0 + i + 1] - row_ptr[w0 + i]);
                ++count[max_len - d + 1];
            }
            for (int b = 1; b < (int)count.size(); ++b) count[b] += count[b - 1];
            for (int i = 0; i < cnt; ++i) {
                const int d = (int)(row_ptr[w0 + i + 1] - row_ptr[w0 + i]);
                perm[w0 + count[max_len - d]++] = w0 + i;
            }
        }
        const int n_chunks = (n - 1) / C + 1;
        const int rows_padded = n_chunks * C;
        for (int p = 0; p < rows_padded; ++p) {
            row_length[p] = (p < n) ? (int)(row_ptr[perm[p] + 1] - row_ptr[perm[p]]) : 0;
        }
        long long acc = 0;
        for (int c = 0; c < n_chunks; ++c) {
            int m = 0;
            for (int l = 0; l < C; ++l) m = std::max(m, row_length[c * C + l]);
            chunk_length[c] = m;
            LGD_REQUIRE(acc <= 0x7fffffffLL, LGD_ERR_RANGE, "more than 2^31-1 SELL value slots");
            chunk_offset[c] = (int)acc;
            acc += (long long)m * C;
        }
        LGD_REQUIRE(acc <= 0x7fffffffLL, LGD_ERR_RANGE, "more than 2^31-1 SELL value slots");
        chunk_offset[n_chunks] = (int)acc;
        *total = acc;
    });
}

int lgd_sell_fill(int n, const int64_t *row_ptr, const int32_t *col, const double *w, int C, const int32_t *perm,
                  const int32_t *chunk_offset, int64_t total, int remap_columns, double *values, int32_t *column)
{
    return guard([&] {
        LGD_REQUIRE(n > 0 && C >= 1, LGD_ERR_INVALID, "bad sizes");
        LGD_REQUIRE(row_ptr && perm && chunk_offset && (total == 0 || (values && column)), LGD_ERR_INVALID,
                    "null argument");
        LGD_REQUIRE(row_ptr[n] == 0 || (col && w), LGD_ERR_INVALID, "null matrix arrays");
        std::vector<int> log_to_phys(n, -1);
        for (int p = 0; p < n; ++p) {
            LGD_REQUIRE(perm[p] >= 0 && perm[p] < n && log_to_phys[perm[p]] < 0, LGD_ERR_INVALID,
                        "perm is not a permutation");
            log_to_phys[perm[p]] = p;
        }
        std::memset(values, 0, sizeof(double) * (size_t)total);
        std::memset(column, 0, sizeof(int32_t) * (size_t)total);
        std::vector<std::pair<int, long long> > row;
        for (int p = 0; p < n; ++p) {
            const int r = perm[p];
            const long long b = row_ptr[r];
            const int d = (int)(row_ptr[r + 1] - b);
            row.resize(d);
            for (int k = 0; k < d; ++k) {
                const int c = col[b + k];
                LGD_REQUIRE(c >= 0 && c < n, LGD_ERR_RANGE, "column id outside the node set");
                row[k] = std::make_pair(remap_columns ? log_to_phys[c] : c, b + k);
            }
            // insertion sort by column (ties keep input order)
            for (int i = 1; i < d; ++i) {
                std::pair<int, long long> t = row[i];
                int j = i - 1;
                while (j >= 0 && row[j].first > t.first) {
                    row[j + 1] = row[j];
                    --j;
                }
                row[j + 1] = t;
            }
            const long long base = (long long)chunk_offset[p / C] + p % C;
            for (int k = 0; k < d; ++k) {
                LGD_REQUIRE(base + (long long)k * C < total, LGD_ERR_INVALID, "chunk_offset does not fit the rows");
                values[base + (long long)k * C] = w[row[k].second];
                column[base + (long long)k * C] = row[k].first;
            }
        }
    });
}

int lgd_sell_create(int n, int C, int64_t total, const int32_t *chunk_offset, const int32_t *row_length,
                    const double *values, const int32_t *column, const int32_t *perm, int precision, int flags,
                    lgd_sell **out)
{
    return guard([&] {
        LGD_REQUIRE(out != nullptr, LGD_ERR_INVALID, "null output");
        *out = nullptr;
        LGD_REQUIRE(n > 0 && C >= 1 && total >= 0, LGD_ERR_INVALID, "bad sizes");
        LGD_REQUIRE(precision == 8 || precision == 4, LGD_ERR_INVALID, "precision must be 8 (FP64) or 4 (FP32)");
        LGD_REQUIRE(chunk_offset && row_length && (total == 0 || (values && column)), LGD_ERR_INVALID, "null argument");
        const int n_chunks = (n - 1) / C + 1;
        const int rows_padded = n_chunks * C;
        LGD_REQUIRE(chunk_offset[0] == 0 && chunk_offset[n_chunks] == total, LGD_ERR_INVALID,
                    "chunk_offset does not span the values");
        for (int p = 0; p < rows_padded; ++p) {
            const int c = p / C;
            LGD_REQUIRE(row_length[p] >= 0 && (long long)row_length[p] * C <= chunk_offset[c + 1] - chunk_offset[c],
                        LGD_ERR_INVALID, "row length exceeds its chunk");
        }
        for (long long i = 0; i < total; ++i) {
            LGD_REQUIRE(column[i] >= 0 && column[i] < n, LGD_ERR_RANGE, "column id outside the node set");
        }
        Sell *s = new Sell();
        std::memset(s, 0, sizeof(Sell));
        s->n = n;
        s->C = C;
        s->n_chunks = n_chunks;
        s->rows_padded = rows_padded;
        s->total = total;
        s->precision = precision;
        s->flags = flags;
        try {
            LGD_CHECK_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
            LGD_CHECK_CUDA(cudaMalloc(&s->d_chunk_offset, sizeof(int) * (n_chunks + 1)));
            LGD_CHECK_CUDA(cudaMalloc(&s->d_row_length, sizeof(int) * rows_padded));
            LGD_CHECK_CUDA(cudaMalloc(&s->d_values, (size_t)precision * std::max<long long>(total, 1)));
            LGD_CHECK_CUDA(cudaMalloc(&s->d_column, sizeof(int) * std::max<long long>(total, 1)));
            for (int b = 0; b < 2; ++b) {
                LGD_CHECK_CUDA(cudaMalloc(&s->d_x[b], (size_t)precision * rows_padded));
                LGD_CHECK_CUDA(cudaMemsetAsync(s->d_x[b], 0, (size_t)precision * rows_padded, s->stream));
            }
            LGD_CHECK_CUDA(cudaMemcpyAsync(s->d_chunk_offset, chunk_offset, sizeof(int) * (n_chunks + 1),
                                           cudaMemcpyHostToDevice, s->stream));
            LGD_CHECK_CUDA(cudaMemcpyAsync(s->d_row_length, row_length, sizeof(int) * rows_padded,
                                           cudaMemcpyHostToDevice, s->stream));
            if (total > 0) {
                LGD_CHECK_CUDA(cudaMemcpyAsync(s->d_column, column, sizeof(int) * total, cudaMemcpyHostToDevice, s->stream));
                if (precision == 8) {
                    LGD_CHECK_CUDA(cudaMemcpyAsync(s->d_values, values, sizeof(double) * total, cudaMemcpyHostToDevice,
                                                   s->stream));
                } else {
                    std::vector<float> vf(values, values + total);
                    LGD_CHECK_CUDA(cudaMemcpyAsync(s->d_values, vf.data(), sizeof(float) * total, cudaMemcpyHostToDevice,
                                                   s->stream));
                    LGD_CHECK_CUDA(cudaStreamSynchronize(s->stream));
                }
            }
            if (perm) {
                LGD_CHECK_CUDA(cudaMalloc(&s->d_perm, sizeof(int) * n));
                LGD_CHECK_CUDA(cudaMemcpyAsync(s->d_perm, perm, sizeof(int) * n, cudaMemcpyHostToDevice, s->stream));
            }
            LGD_CHECK_CUDA(cudaStreamSynchronize(s->stream));
        } catch (...) {
            sell_free(*s);
            delete s;
            throw;
        }
        *out = reinterpret_cast<lgd_sell *>(s);
    });
}

namespace {

// order[k] = the node numbered k: reverse Cuthill-McKee over the graph's
// edges in both directions
std::vector<int32_t> rcm_order(int n, const int64_t *rp, const int32_t *col)
{
    const int64_t nnz = rp[n];
    std::vector<int64_t> deg(n, 0);
    std::vector<int64_t> trp((size_t)n + 1, 0);
    for (int r = 0; r < n; ++r) {
        deg[r] += rp[r + 1] - rp[r];
        for (int64_t e = rp[r]; e < rp[r + 1]; ++e) {
            const int32_t c = col[e];
            if (c < 0 || c >= n) throw Error(LGD_ERR_RANGE, "column id outside the node set");
            ++trp[(size_t)c + 1];
            ++deg[c];
        }
    }
    for (int r = 0; r < n; ++r) trp[(size_t)r + 1] += trp[r];
    std::vector<int32_t> tcol((size_t)nnz);
    {
        std::vector<int64_t> fill(trp.begin(), trp.end() - 1);
        for (int r = 0; r < n; ++r) {
            for (int64_t e = rp[r]; e < rp[r + 1]; ++e) tcol[(size_t)fill[col[e]]++] = r;
        }
    }
    std::vector<int32_t> by_degree(n);
    for (int i = 0; i < n; ++i) by_degree[i] = i;
    std::stable_sort(by_degree.begin(), by_degree.end(), [&](int32_t a, int32_t b) { return deg[a] < deg[b]; });
    std::vector<char> seen(n, 0);
    std::vector<int32_t> order;
    order.reserve(n);
    std::vector<int32_t> nb;
    size_t head = 0;
    for (int32_t start : by_degree) {
        if (seen[start]) continue;
        seen[start] = 1;
        order.push_back(start);
        for (; head < order.size(); ++head) {
            const int32_t u = order[head];
            nb.clear();
            for (int64_t e = rp[u]; e < rp[u + 1]; ++e) {
                if (!seen[col[e]]) {
                    seen[col[e]] = 1;
                    nb.push_back(col[e]);
                }
            }
            for (int64_t e = trp[u]; e < trp[(size_t)u + 1]; ++e) {
                if (!seen[tcol[e]]) {
                    seen[tcol[e]] = 1;
                    nb.push_back(tcol[e]);
                }
            }
            std::stable_sort(nb.begin(), nb.end(), [&](int32_t a, int32_t b) { return deg[a] < deg[b]; });
            order.insert(order.end(), nb.begin(), nb.end());
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

__global__ void compose_perm_kernel(int *perm, const int32_t *order, int n)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) perm[p] = order[perm[p]];
}

}  // namespace

int lgd_graph_rcm(int n, const int64_t *row_ptr, const int32_t *col, int32_t *order)
{
    return guard([&] {
        LGD_REQUIRE(n > 0 && row_ptr != nullptr && order != nullptr, LGD_ERR_INVALID, "empty graph or null array");
        LGD_REQUIRE(row_ptr[n] == 0 || col != nullptr, LGD_ERR_INVALID, "null column array");
        const std::vector<int32_t> o = rcm_order(n, row_ptr, col);
        std::copy(o.begin(), o.end(), order);
    });
}

int lgd_sell_create_from_csr(int n, const int64_t *row_ptr, const int32_t *col, const double *w, int C, int sigma,
                             int device_input, int precision, int flags, lgd_sell **out)
{
    if (flags & LGD_SELL_RENUMBER) {
        // number the nodes in reverse Cuthill-McKee order, build from the
        // renumbered CSR, then compose the permutation so that logical
        // order stays the caller's
        return guard([&] {
            LGD_REQUIRE(out != nullptr, LGD_ERR_INVALID, "null output");
            *out = nullptr;
            LGD_REQUIRE(!device_input, LGD_ERR_UNSUPPORTED, "renumbering takes the CSR arrays in host memory");
            LGD_REQUIRE(n > 0 && row_ptr != nullptr, LGD_ERR_INVALID, "node count must be positive");
            const int64_t nnz = row_ptr[n];
            LGD_REQUIRE(nnz == 0 || (col && w), LGD_ERR_INVALID, "null matrix arrays");
            const std::vector<int32_t> order = rcm_order(n, row_ptr, col);
            std::vector<int32_t> inv(n);
            for (int k = 0; k < n; ++k) inv[order[k]] = k;
            std::vector<int64_t> rp2((size_t)n + 1, 0);
            std::vector<int32_t> col2((size_t)nnz);
            std::vector<double> w2((size_t)nnz);
            for (int k = 0; k < n; ++k) {
                const int r = order[k];
                int64_t o = rp2[k];
                for (int64_t e = row_ptr[r]; e < row_ptr[r + 1]; ++e, ++o) {
                    col2[(size_t)o] = inv[col[e]];
                    w2[(size_t)o] = w[e];
                }
                rp2[(size_t)k + 1] = o;
            }
            lgd_sell *h = nullptr;
            const int rc = lgd_sell_create_from_csr(n, rp2.data(), col2.data(), w2.data(), C, sigma, 0, precision,
                                                    flags & ~LGD_SELL_RENUMBER, &h);
            if (rc != LGD_OK) {
                char msg[512];
                lgd_gpu_last_error(msg, sizeof(msg));
                throw Error(rc, std::string("renumbered matrix: ") + msg);
            }
            Sell& s = sell_of(h);
            int32_t *d_order = nullptr;
            try {
                LGD_CHECK_CUDA(cudaMalloc(&d_order, sizeof(int32_t) * (size_t)n));
                LGD_CHECK_CUDA(cudaMemcpyAsync(d_order, order.data(), sizeof(int32_t) * (size_t)n,
                                               cudaMemcpyHostToDevice, s.stream));
                compose_perm_kernel<<<(unsigned)std::min(152 * 16, (n + 255) / 256), 256, 0, s.stream>>>(s.d_perm, d_order,
                                                                                                         n);
                check_launch("sell renumbering");
                LGD_CHECK_CUDA(cudaStreamSynchronize(s.stream));
            } catch (...) {
                cudaFree(d_order);
                lgd_sell_destroy(h);
                throw;
            }
            cudaFree(d_order);
            s.flags = flags;
            *out = h;
        });
    }
    return guard([&] {
        using namespace sbuild;
        LGD_REQUIRE(out != nullptr, LGD_ERR_INVALID, "null output");
        *out = nullptr;
        LGD_REQUIRE(n > 0, LGD_ERR_INVALID, "node count must be positive");
        LGD_REQUIRE(C >= 1 && sigma >= 1, LGD_ERR_INVALID, "C and sigma must be at least 1");
        LGD_REQUIRE(sigma <= LGD_SELL_GPU_MAX_SIGMA, LGD_ERR_UNSUPPORTED,
                    "the device builder takes sigma <= 4096 (use lgd_sell_plan / lgd_sell_fill)");
        LGD_REQUIRE(precision == 8 || precision == 4, LGD_ERR_INVALID, "precision must be 8 (FP64) or 4 (FP32)");
        LGD_REQUIRE(row_ptr != nullptr, LGD_ERR_INVALID, "null row_ptr");
        Sell *s = new Sell();
        std::memset(s, 0, sizeof(Sell));
        s->n = n;
        s->C = C;
        s->n_chunks = (n - 1) / C + 1;
        s->rows_padded = s->n_chunks * C;
        s->precision = precision;
        s->flags = flags;
        int64_t *d_rp = nullptr;
        int32_t *d_col = nullptr;
        double *d_w = nullptr;
        int *d_len = nullptr, *d_inv = nullptr, *d_err = nullptr;
        long long *d_total = nullptr;
        auto release = [&] {
            if (!device_input) {
                cudaFree(d_rp);
                cudaFree(d_col);
                cudaFree(d_w);
            }
            cudaFree(d_len);
            cudaFree(d_inv);
            cudaFree(d_err);
            cudaFree(d_total);
        };
        try {
            LGD_CHECK_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
            cudaStream_t st = s->stream;
            long long nnz = 0;
            if (device_input) {
                d_rp = const_cast<int64_t *>(row_ptr);
                d_col = const_cast<int32_t *>(col);
                d_w = const_cast<double *>(w);
                int64_t last = 0;
                LGD_CHECK_CUDA(cudaMemcpyAsync(&last, row_ptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
                LGD_CHECK_CUDA(cudaStreamSynchronize(st));
                nnz = last;
            } else {
                nnz = row_ptr[n];
                LGD_CHECK_CUDA(cudaMalloc(&d_rp, sizeof(int64_t) * ((size_t)n + 1)));
                LGD_CHECK_CUDA(cudaMemcpyAsync(d_rp, row_ptr, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
                if (nnz > 0) {
                    LGD_REQUIRE(col && w, LGD_ERR_INVALID, "null matrix arrays");
                    LGD_CHECK_CUDA(cudaMalloc(&d_col, sizeof(int32_t) * (size_t)nnz));
                    LGD_CHECK_CUDA(cudaMalloc(&d_w, sizeof(double) * (size_t)nnz));
                    LGD_CHECK_CUDA(cudaMemcpyAsync(d_col, col, sizeof(int32_t) * (size_t)nnz, cudaMemcpyHostToDevice, st));
                    LGD_CHECK_CUDA(cudaMemcpyAsync(d_w, w, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, st));
                }
            }
            LGD_REQUIRE(nnz >= 0, LGD_ERR_INVALID, "row_ptr must be non-decreasing");
            LGD_REQUIRE(nnz == 0 || (d_col && d_w), LGD_ERR_INVALID, "null matrix arrays");
            LGD_CHECK_CUDA(cudaMalloc(&d_len, sizeof(int) * (size_t)n));
            LGD_CHECK_CUDA(cudaMalloc(&d_inv, sizeof(int) * (size_t)n));
            LGD_CHECK_CUDA(cudaMalloc(&d_err, sizeof(int)));
            LGD_CHECK_CUDA(cudaMalloc(&d_total, sizeof(long long)));
            LGD_CHECK_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), st));
            LGD_CHECK_CUDA(cudaMalloc(&s->d_perm, sizeof(int) * (size_t)n));
            LGD_CHECK_CUDA(cudaMalloc(&s->d_row_length, sizeof(int) * (size_t)s->rows_padded));
            LGD_CHECK_CUDA(cudaMalloc(&s->d_chunk_offset, sizeof(int) * ((size_t)s->n_chunks + 1)));
            const int blocks = (int)std::min<long long>(152LL * 16, ((long long)s->rows_padded + 255) / 256);
            lengths_kernel<<<blocks, 256, 0, st>>>(d_rp, n, d_len, d_err);
            int P = 1;
            while (P < std::min(sigma, n)) P <<= 1;
            const int windows = (n + sigma - 1) / sigma;
            window_sort_kernel<<<windows, SORT_THREADS, sizeof(uint32_t) * P, st>>>(d_len, n, sigma, P, s->d_perm);
            row_length_kernel<<<blocks, 256, 0, st>>>(d_len, s->d_perm, n, s->rows_padded, s->d_row_length, d_inv);
            chunk_scan_kernel<<<1, 1024, 0, st>>>(s->d_row_length, C, s->n_chunks, s->d_chunk_offset, d_total, d_err);
            check_launch("sell build (plan)");
            int err = 0;
            long long total = 0;
            LGD_CHECK_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
            LGD_CHECK_CUDA(cudaMemcpyAsync(&total, d_total, sizeof(long long), cudaMemcpyDeviceToHost, st));
            LGD_CHECK_CUDA(cudaStreamSynchronize(st));
            LGD_REQUIRE(!(err & E_ROWPTR), LGD_ERR_INVALID, "row_ptr must start at 0 and be non-decreasing");
            LGD_REQUIRE(!(err & E_LONGROW), LGD_ERR_UNSUPPORTED,
                        "a row has more than 1024 entries (use lgd_sell_plan / lgd_sell_fill)");
            LGD_REQUIRE(!(err & E_TOTAL), LGD_ERR_RANGE, "more than 2^31-1 SELL value slots");
            s->total = total;
            LGD_CHECK_CUDA(cudaMalloc(&s->d_values, (size_t)precision * std::max<long long>(total, 1)));
            LGD_CHECK_CUDA(cudaMalloc(&s->d_column, sizeof(int) * std::max<long long>(total, 1)));
            LGD_CHECK_CUDA(cudaMemsetAsync(s->d_values, 0, (size_t)precision * std::max<long long>(total, 1), st));
            LGD_CHECK_CUDA(cudaMemsetAsync(s->d_column, 0, sizeof(int) * std::max<long long>(total, 1), st));
            if (nnz > 0) {
                const int fblocks = (int)std::min<long long>(152LL * 64, ((long long)n + 7) / 8);
                if (precision == 8) {
                    fill_kernel<double><<<fblocks, 256, 0, st>>>(d_rp, d_col, d_w, s->d_perm, d_inv, s->d_chunk_offset,
                                                                  n, C, total, (double *)s->d_values, s->d_column, d_err);
                } else {
                    fill_kernel<float><<<fblocks, 256, 0, st>>>(d_rp, d_col, d_w, s->d_perm, d_inv, s->d_chunk_offset,
                                                                 n, C, total, (float *)s->d_values, s->d_column, d_err);
                }
                check_launch("sell build (fill)");
            }
            for (int bb = 0; bb < 2; ++bb) {
                LGD_CHECK_CUDA(cudaMalloc(&s->d_x[bb], (size_t)precision * s->rows_padded));
                LGD_CHECK_CUDA(cudaMemsetAsync(s->d_x[bb], 0, (size_t)precision * s->rows_padded, st));
            }
            LGD_CHECK_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
            LGD_CHECK_CUDA(cudaStreamSynchronize(st));
            LGD_REQUIRE(!(err & E_COLUMN), LGD_ERR_RANGE, "column id outside the node set");
            release();
        } catch (...) {
            release();
            sell_free(*s);
            delete s;
            throw;
        }
        *out = reinterpret_cast<lgd_sell *>(s);
    });
}

int lgd_sell_get_layout(lgd_sell *h, int32_t *chunk_offset, int32_t *row_length, double *values, int32_t *column,
                        int32_t *perm, int64_t *total)
{
    return guard([&] {
        Sell& s = sell_of(h);
        cudaStream_t st = s.stream;
        if (total) *total = s.total;
        if (chunk_offset) {
            LGD_CHECK_CUDA(cudaMemcpyAsync(chunk_offset, s.d_chunk_offset, sizeof(int) * ((size_t)s.n_chunks + 1),
                                           cudaMemcpyDeviceToHost, st));
        }
        if (row_length) {
            LGD_CHECK_CUDA(cudaMemcpyAsync(row_length, s.d_row_length, sizeof(int) * (size_t)s.rows_padded,
                                           cudaMemcpyDeviceToHost, st));
        }
        if (column && s.total > 0) {
            LGD_CHECK_CUDA(cudaMemcpyAsync(column, s.d_column, sizeof(int) * (size_t)s.total, cudaMemcpyDeviceToHost, st));
        }
        if (perm) {
            LGD_REQUIRE(s.d_perm != nullptr, LGD_ERR_INVALID, "the handle has no permutation");
            LGD_CHECK_CUDA(cudaMemcpyAsync(perm, s.d_perm, sizeof(int) * (size_t)s.n, cudaMemcpyDeviceToHost, st));
        }
        if (values && s.total > 0) {
            if (s.precision == 8) {
                LGD_CHECK_CUDA(cudaMemcpyAsync(values, s.d_values, sizeof(double) * (size_t)s.total,
                                               cudaMemcpyDeviceToHost, st));
            } else {
                std::vector<float> vf((size_t)s.total);
                LGD_CHECK_CUDA(cudaMemcpyAsync(vf.data(), s.d_values, sizeof(float) * (size_t)s.total,
                                               cudaMemcpyDeviceToHost, st));
                LGD_CHECK_CUDA(cudaStreamSynchronize(st));
                for (size_t i = 0; i < vf.size(); ++i) values[i] = vf[i];
            }
        }
        LGD_CHECK_CUDA(cudaStreamSynchronize(st));
    });
}

int lgd_sell_destroy(lgd_sell *h)
{
    return guard([&] {
        if (!h) return;
        Sell& s = sell_of(h);
        sell_free(s);
        delete &s;
    });
}

static void sell_copy_x(Sell& s, int which, double *host, size_t bytes, bool up, bool logical)
{
    LGD_REQUIRE(which == 0 || which == 1, LGD_ERR_INVALID, "which must be 0 or 1");
    LGD_REQUIRE(host != nullptr, LGD_ERR_INVALID, "null host buffer");
    LGD_REQUIRE(bytes == sizeof(double) * (size_t)s.n, LGD_ERR_INVALID, "byte count must be n doubles");
    LGD_REQUIRE(!logical || s.d_perm != nullptr, LGD_ERR_INVALID, "no permutation was given at create");
    double *tmp = nullptr;
    LGD_CHECK_CUDA(cudaMallocAsync(&tmp, bytes, s.stream));
    void *x = s.d_x[which ? 1 - s.cur : s.cur];
    const int *perm = logical ? s.d_perm : nullptr;
    const int blocks = std::min(152 * 8, (s.n + 255) / 256);
    if (up) {
        LGD_CHECK_CUDA(cudaMemcpyAsync(tmp, host, bytes, cudaMemcpyHostToDevice, s.stream));
        if (s.precision == 8) {
            permute_in_kernel<double><<<blocks, 256, 0, s.stream>>>(tmp, perm, (double *)x, s.n);
        } else {
            permute_in_kernel<float><<<blocks, 256, 0, s.stream>>>(tmp, perm, (float *)x, s.n);
        }
    } else {
        if (s.precision == 8) {
            permute_out_kernel<double><<<blocks, 256, 0, s.stream>>>((const double *)x, perm, tmp, s.n);
        } else {
            permute_out_kernel<float><<<blocks, 256, 0, s.stream>>>((const float *)x, perm, tmp, s.n);
        }
        LGD_CHECK_CUDA(cudaMemcpyAsync(host, tmp, bytes, cudaMemcpyDeviceToHost, s.stream));
    }
    check_launch("sell permute");
    ++s.launches;
    LGD_CHECK_CUDA(cudaFreeAsync(tmp, s.stream));
    LGD_CHECK_CUDA(cudaStreamSynchronize(s.stream));
}

int lgd_sell_upload_x(lgd_sell *h, int which, int logical, const double *x, size_t bytes)
{
    return guard([&] { sell_copy_x(sell_of(h), which, const_cast<double *>(x), bytes, true, logical != 0); });
}

int lgd_sell_download_x(lgd_sell *h, int which, int logical, double *x, size_t bytes)
{
    return guard([&] { sell_copy_x(sell_of(h), which, x, bytes, false, logical != 0); });
}

int lgd_sell_step(lgd_sell *h, int count)
{
    return guard([&] {
        Sell& s = sell_of(h);
        LGD_REQUIRE(count >= 0, LGD_ERR_INVALID, "negative step count");
        for (int i = 0; i < count; ++i) {
            launch_sell(s, 0, s.n);
            s.cur = 1 - s.cur;
        }
    });
}

int lgd_sell_update_rows(lgd_sell *h, int row_begin, int row_end)
{
    return guard([&] {
        Sell& s = sell_of(h);
        LGD_REQUIRE(0 <= row_begin && row_begin <= row_end && row_end <= s.n, LGD_ERR_RANGE,
                    "row range outside the node set");
        launch_sell(s, row_begin, row_end);
    });
}

int lgd_sell_swap(lgd_sell *h)
{
    return guard([&] {
        Sell& s = sell_of(h);
        s.cur = 1 - s.cur;
    });
}

int lgd_sell_x_device(lgd_sell *h, int which, void **ptr, int64_t *rows_padded)
{
    return guard([&] {
        Sell& s = sell_of(h);
        LGD_REQUIRE(which == 0 || which == 1, LGD_ERR_INVALID, "which must be 0 (current) or 1 (next)");
        LGD_REQUIRE(ptr != nullptr, LGD_ERR_INVALID, "null output");
        *ptr = which == 0 ? s.d_x[s.cur] : s.d_x[1 - s.cur];
        if (rows_padded) *rows_padded = s.rows_padded;
    });
}

int lgd_sell_synchronize(lgd_sell *h)
{
    return guard([&] { LGD_CHECK_CUDA(cudaStreamSynchronize(sell_of(h).stream)); });
}

int lgd_sell_stream(lgd_sell *h, void **stream)
{
    return guard([&] {
        LGD_REQUIRE(stream != nullptr, LGD_ERR_INVALID, "null output");
        *stream = (void *)sell_of(h).stream;
    });
}

int lgd_sell_set_variant(lgd_sell *h, int variant)
{
    return guard([&] {
        Sell& s = sell_of(h);
        LGD_REQUIRE(variant >= 0 && variant <= 5, LGD_ERR_INVALID, "SELL kernel variant must lie in [0, 5]");
        s.variant = variant;
    });
}

int lgd_sell_launch_count(lgd_sell *h, uint64_t *count)
{
    return guard([&] {
        LGD_REQUIRE(count != nullptr, LGD_ERR_INVALID, "null output");
        *count = sell_of(h).launches;
    });
}

}  // extern "C"
