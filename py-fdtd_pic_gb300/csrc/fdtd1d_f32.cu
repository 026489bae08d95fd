// FP32 instantiation of the FDTD kernels (FP64 only for near-degenerate Kerr cubics).
#include "fdtd1d_launch.cuh"

namespace fdtdpic {

int run_batch_f32(const BatchArgs<float> &a, int threads, int grid, cudaStream_t st)
{
    return launch_batch<float>(a, threads, grid, st);
}

int run_global_f32(const FdtdInstance &h, const BatchArgs<float> &a, cudaStream_t st)
{
    return launch_global<float>(h, a, st);
}

}  // namespace fdtdpic
