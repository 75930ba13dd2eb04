// tma_util.cuh -- mbarrier and TMA tensor-load helpers (inline PTX) shared by
// the TMA-staged kernels.  Every wait is bounded: mbar_wait gives up after a
// second and returns false, and the kernel reports the case.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace suli {

// a wait gives up after TMA_WAIT_NS of the global timer (or TMA_WAIT_MAX
// polls, should the timer not advance)
constexpr unsigned long long TMA_WAIT_NS = 1000000000ull;   // one second
constexpr unsigned TMA_WAIT_MAX = 1u << 24;

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arm(uint64_t *b, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned a, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n selp.b32 %0, 1, 0, P;\n}\n"
                 : "=r"(ok)
                 : "r"(a), "r"(parity)
                 : "memory");
    return ok != 0;
}
// bounded wait for phase `parity` of barrier b: false when it gave up (the
// global timer is read once every 256 polls)
__device__ __forceinline__ bool mbar_wait(uint64_t *b, unsigned parity)
{
    const unsigned a = smem_u32(b);
    unsigned long long t0 = 0ull;
    for (unsigned it = 0; it < TMA_WAIT_MAX; ++it) {
        if (mbar_try(a, parity)) return true;
        if ((it & 255u) == 255u) {
            const unsigned long long now = global_ns();
            if (t0 == 0ull) t0 = now;
            else if (now - t0 > TMA_WAIT_NS) return false;
        }
    }
    return false;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace suli
