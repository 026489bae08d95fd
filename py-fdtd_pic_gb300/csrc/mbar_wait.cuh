// Bounded waits on an mbarrier phase, shared by the tensor-core DFT and the wait self-test.
#pragma once
#include <stdint.h>

namespace fdtdpic {

constexpr long long TC_WAIT_LIMIT = 1LL << 26;  // mbarrier polls before giving up

__device__ __forceinline__ uint32_t tc_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity));
    return done;
}

// Bounded wait on an mbarrier phase: 1 when it completed, 0 when `limit` polls ran out.
__device__ __forceinline__ uint32_t tc_wait(uint32_t bar, uint32_t parity,
                                            long long limit = TC_WAIT_LIMIT)
{
    for (long long spins = 0; spins < limit; ++spins)
        if (tc_try_wait(bar, parity)) return 1u;
    return 0u;
}

}  // namespace fdtdpic
