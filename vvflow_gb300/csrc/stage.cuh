// Shared-memory staging by the bulk copy engine (TMA, cp.async.bulk) with mbarrier
// completion.  Every wait is bounded: a wait that runs out returns false and the caller
// reports VVGPU_ERR_TIMEOUT after draining its copies in flight.
#pragma once

#include <cstdint>

namespace vvgpu {

// polls of one staging wait before it gives up (a few hundred ms on a GB300)
constexpr uint32_t STAGE_SPINS = 1u << 22;

__device__ __forceinline__ uint32_t stage_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// one arrival expected per phase (the arrive.expect_tx of the issuing lane)
__device__ __forceinline__ void stage_bar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(stage_u32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// arrive on the barrier and add `bytes` to the phase's expected transaction count
__device__ __forceinline__ void stage_expect(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(stage_u32(bar)), "r"(bytes)
                 : "memory");
}

// order this thread's earlier shared-memory accesses before its later bulk copies
__device__ __forceinline__ void stage_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// global -> shared bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned),
// completing on `bar`
__device__ __forceinline__ void stage_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     stage_u32(dst)),
                 "l"(src), "r"(bytes), "r"(stage_u32(bar))
                 : "memory");
}

// bounded wait for the completion of phase `parity`; false when `spins` polls ran out
__device__ __forceinline__ bool stage_wait(uint64_t* bar, uint32_t parity, uint32_t spins) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < spins && !done; it++)
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(stage_u32(bar)), "r"(parity)
            : "memory");
    return done != 0;
}

}  // namespace vvgpu
