// Tests of the device-side bounded waits, for the host's test suite: one thread waits on
// something nothing completes and must give up, report it, and return.  These are the wait
// functions the persistent kernels use (tile_wait: the tiled PIC kernel's neighbour flags with a
// %globaltimer deadline; tc_wait: the tensor-core DFT's mbarrier phases with a poll limit), so a
// test can see a wait run out without faulting or hanging anything.
#include <cuda_runtime.h>

#include "mbar_wait.cuh"
#include "pic_tiled.cuh"

namespace {

__global__ void wait_selftest_kernel(int which, long long limit, int32_t *out, int32_t *flag_abort)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const long long t0 = fdtdpic::globaltimer();
    int code = 0;
    if (which == 0) {
        // a neighbour flag that nothing raises: flag_abort[0] is the flag, [1] the abort word
        flag_abort[0] = 0;
        flag_abort[1] = 0;
        __threadfence();
        const bool ok = fdtdpic::tile_wait(flag_abort, 1, flag_abort + 1, t0 + limit);
        code = ok ? 0 : *(volatile int32_t *)(flag_abort + 1);
    } else {
        // an mbarrier (one expected arrival) that nothing arrives on
        __shared__ __align__(8) unsigned long long bar;
        const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const uint32_t done = fdtdpic::tc_wait(b, 0u, limit);
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(b) : "memory");
        code = done ? 0 : FDTDPIC_ERR_TIMEOUT;
    }
    out[0] = code;
    out[1] = (int32_t)min((fdtdpic::globaltimer() - t0) / 1000, (long long)INT32_MAX);
}

}  // namespace

extern "C" int fdtdpic_wait_selftest(int which, int64_t limit, int32_t *d_out, int32_t *d_scratch,
                                     fdtdpic_stream_t stream)
{
    if (!d_out || (which == 0 && !d_scratch) || which < 0 || which > 1 || limit < 1)
        return FDTDPIC_ERR_ARG;
    // at most 2 s of deadline or 2^26 polls: a test's wait stays short
    if ((which == 0 && limit > 2000000000LL) || (which == 1 && limit > (1LL << 26)))
        return FDTDPIC_ERR_ARG;
    wait_selftest_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(which, (long long)limit, d_out,
                                                             d_scratch);
    return fdtdpic::cuda_status(cudaGetLastError());
}
