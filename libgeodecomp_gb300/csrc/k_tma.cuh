// Device helpers of the TMA-fed kernels: mbarriers with bounded waits,
// tiled cp.async.bulk.tensor loads, paired shared-memory loads.
#ifndef LGD_K_TMA_CUH
#define LGD_K_TMA_CUH

#include <cuda.h>
#include <stdint.h>

namespace lgd {
namespace tmak {

// about two seconds of clock cycles: a wait that runs out reports an error
// instead of hanging the GPU
constexpr long long WAIT_CYCLES = 4000000000LL;

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
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

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long long limit = WAIT_CYCLES)
{
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > limit) return false;
    }
    return true;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// two consecutive elements of 4 or 8 bytes in one shared-memory load
template<typename T>
__device__ __forceinline__ void lds_pair(const unsigned char *p, T& a, T& b)
{
    if (sizeof(T) == 8) {
        const longlong2 v = *reinterpret_cast<const longlong2 *>(p);
        a = *reinterpret_cast<const T *>(&v.x);
        b = *reinterpret_cast<const T *>(&v.y);
    } else {
        const int2 v = *reinterpret_cast<const int2 *>(p);
        a = *reinterpret_cast<const T *>(&v.x);
        b = *reinterpret_cast<const T *>(&v.y);
    }
}

// two consecutive elements in one store (shared or global memory)
template<typename T>
__device__ __forceinline__ void st_pair(void *p, T a, T b)
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

}  // namespace tmak
}  // namespace lgd

#endif
