// lgd_sum_f64_static: an FP64 sum for callers that must not allocate device
// memory - the same sum as lgd_gpu_checksum, added in a different order
// (blocks of 65536 values and a tree on the device), so not bit-identical
// to it.
//
// Who needs it: code that runs inside another framework's stream and memory
// pool - a Writer or Steerer plugin called in the middle of a simulation
// step, a solver embedded in an application with its own caching
// allocator - where a cudaMalloc/cudaFree pair would synchronise the whole
// device, stall the other streams and fragment the pool, and code with a
// fixed, pre-committed memory budget.  The regular checksum takes its
// per-block partial sums from memory the library allocates; this variant
// keeps them in a fixed file-scope device array instead.
//
// Limits and sharing: the scratch holds LGD_SUM_STATIC_MAX_PARTIALS partial
// sums, one per block of LGD_SUM_STATIC_CHUNK values, so at most
// LGD_SUM_STATIC_MAX_N values per call; larger inputs are rejected with
// LGD_ERR_RANGE.  Every GPU that loads the library holds this array
// (128 KiB) until the process exits.  All calls on a device share it and it
// keeps the last call's partials: calls whose work overlaps on the GPU
// (different streams without ordering between them) race on it.
#include <mutex>

#include "lgd_internal.h"

namespace lgd {

static const int kThreads = 256;

// partial sums of the blocks of the latest call on this device
static __device__ __align__(256) double g_sum_scratch[LGD_SUM_STATIC_MAX_PARTIALS];

// Block b sums values [b * CHUNK, min(n, (b + 1) * CHUNK)): thread t takes
// every kThreads-th value from b * CHUNK + t, then a fixed tree.
__global__ void __launch_bounds__(kThreads)
static_sum_partials_kernel(const double *__restrict__ v, long long n, double *__restrict__ partials)
{
    __shared__ double red[kThreads];
    const long long begin = (long long)blockIdx.x * LGD_SUM_STATIC_CHUNK;
    const long long end = min(n, begin + (long long)LGD_SUM_STATIC_CHUNK);
    double acc = 0.0;
    for (long long i = begin + threadIdx.x; i < end; i += kThreads) {
        acc += v[i];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

// One block adds the count partials of this call (those were all written by
// the partials kernel just before, so nothing needs clearing) and writes
// the total; count = 0 writes 0.
__global__ void __launch_bounds__(kThreads)
static_sum_final_kernel(const double *__restrict__ partials, int count, double *__restrict__ out)
{
    __shared__ double red[kThreads];
    double acc = 0.0;
    for (int i = threadIdx.x; i < count; i += kThreads) acc += partials[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// Device address of the scratch array, looked up once per device and
// context with that device current.  (In host code the array's name is only
// a host-side stand-in: passing it to a kernel would reach the wrong
// memory.)  The cache is keyed on the device's current context as well:
// after a cudaDeviceReset the primary context is created anew, the module
// is loaded again and the array may move, so a new context means a new
// lookup.  cudaGetSymbolAddress allocates nothing.
static const int kMaxDevices = 64;
static std::mutex g_scratch_mutex;
static double *g_scratch_ptr[kMaxDevices];
static void *g_scratch_ctx[kMaxDevices];

typedef int (*CtxGetCurrentFn)(void **);

// the driver's cuCtxGetCurrent, through the runtime's entry-point query
static CtxGetCurrentFn ctx_get_current()
{
    static const CtxGetCurrentFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            p = nullptr;
        }
        return (CtxGetCurrentFn)p;
    }();
    return fn;
}

static double *scratch_for_current_device()
{
    int dev = 0;
    LGD_CHECK_CUDA(cudaGetDevice(&dev));
    LGD_REQUIRE(dev >= 0 && dev < kMaxDevices, LGD_ERR_UNSUPPORTED, "device index above 63");
    const CtxGetCurrentFn get = ctx_get_current();
    LGD_REQUIRE(get != nullptr, LGD_ERR_CUDA, "cuCtxGetCurrent is not available");
    void *ctx = nullptr;
    if (get(&ctx) != 0) ctx = nullptr;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (ctx == nullptr || !g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
        // (the lookup also makes the device's primary context current when
        // no context is yet)
        double *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_sum_scratch);
        if (e != cudaSuccess || ptr == nullptr) {
            throw Error(LGD_ERR_CUDA, std::string("cudaGetSymbolAddress of the sum scratch failed: ") +
                                          cudaGetErrorString(e));
        }
        if (get(&ctx) != 0) ctx = nullptr;
        g_scratch_ptr[dev] = ptr;
        g_scratch_ctx[dev] = ctx;
    }
    return g_scratch_ptr[dev];
}

}  // namespace lgd

using namespace lgd;

extern "C" int lgd_sum_f64_static(const double *d_values, long long n, double *d_result, void *stream)
{
    return guard([&] {
        LGD_REQUIRE(n >= 0, LGD_ERR_INVALID, "negative value count");
        LGD_REQUIRE(n <= LGD_SUM_STATIC_MAX_N, LGD_ERR_RANGE,
                    "lgd_sum_f64_static takes at most LGD_SUM_STATIC_MAX_N (2^30) values per call; "
                    "its fixed scratch holds 16384 block partials of 65536 values each");
        LGD_REQUIRE(d_result != nullptr, LGD_ERR_INVALID, "null result pointer");
        LGD_REQUIRE(n == 0 || d_values != nullptr, LGD_ERR_INVALID, "null value pointer");
        double *scratch = scratch_for_current_device();
        cudaStream_t s = (cudaStream_t)stream;
        const int blocks = (int)((n + LGD_SUM_STATIC_CHUNK - 1) / LGD_SUM_STATIC_CHUNK);
        if (blocks > 0) {
            static_sum_partials_kernel<<<blocks, kThreads, 0, s>>>(d_values, n, scratch);
            check_launch("static sum partials");
        }
        static_sum_final_kernel<<<1, kThreads, 0, s>>>(scratch, blocks, d_result);
        check_launch("static sum final");
    });
}
