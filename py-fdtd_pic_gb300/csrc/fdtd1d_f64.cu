// FP64 instantiation of the FDTD kernels.  Built with -fmad=false: products and sums round
// separately, in the order the reference's loops write them, so the parity path reproduces the
// FP64 CPU oracle to rounding of the transcendental functions only.
#include "fdtd1d_launch.cuh"

namespace fdtdpic {

int run_batch_f64(const BatchArgs<double> &a, int threads, int grid, cudaStream_t st)
{
    return launch_batch<double>(a, threads, grid, st);
}

int run_global_f64(const FdtdInstance &h, const BatchArgs<double> &a, cudaStream_t st)
{
    return launch_global<double>(h, a, st);
}

__global__ void cubic_root0_kernel(int n, const double *coef, double *out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = cubic_root0_f64(coef[4 * i], coef[4 * i + 1], coef[4 * i + 2], coef[4 * i + 3]);
}

int run_cubic_root0(int n, const double *coef, double *out, cudaStream_t st)
{
    if (n <= 0) return FDTDPIC_OK;
    int blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    cubic_root0_kernel<<<blocks, 256, 0, st>>>(n, coef, out);
    return cuda_status(cudaGetLastError());
}

}  // namespace fdtdpic
