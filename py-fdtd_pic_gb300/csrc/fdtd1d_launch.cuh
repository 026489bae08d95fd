// Host-side launchers for the FDTD kernels, instantiated once per state type in
// fdtd1d_f64.cu (built with -fmad=false so FP64 rounds in the reference's operation order)
// and fdtd1d_f32.cu (FMA contraction on).
#pragma once
#include "fdtd1d_kernel.cuh"

namespace fdtdpic {

int cuda_status(cudaError_t e);

template <typename T>
int launch_batch(const BatchArgs<T> &a, int threads, int grid, cudaStream_t st)
{
    int dev = 0, sms = 0, max_optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FDTDPIC_ERR_NODEV;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (a.smem_bytes < 0 || a.smem_bytes > max_optin) return FDTDPIC_ERR_OOM;
    if (threads <= 0) threads = 256;
    if (threads > 1024 || (threads % 32) != 0) return FDTDPIC_ERR_ARG;
    auto kern = fdtd_batch_kernel<T>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)a.smem_bytes);
    if (e != cudaSuccess) return cuda_status(e);
    if (grid <= 0) {
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, (size_t)a.smem_bytes);
        if (e != cudaSuccess) return cuda_status(e);
        if (per_sm < 1) return FDTDPIC_ERR_OOM;
        grid = per_sm * sms;
    }
    if (grid > a.n_inst) grid = a.n_inst;
    e = cudaMemsetAsync(a.queue, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) return cuda_status(e);
    kern<<<grid, threads, (size_t)a.smem_bytes, st>>>(a);
    return cuda_status(cudaGetLastError());
}

template <typename T>
int launch_global(const FdtdInstance &h, const BatchArgs<T> &a, cudaStream_t st)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FDTDPIC_ERR_NODEV;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t n = (int64_t)h.nz + 1;
    const int threads = 256;
    int64_t blocks = (n + threads - 1) / threads;
    if (blocks > 8LL * sms) blocks = 8LL * sms;
    if (blocks < 1) blocks = 1;
    if (!h.resume) fdtd_global_init_kernel<T><<<(int)blocks, threads, 0, st>>>(a);
    for (int t = h.step_begin; t < h.step_end; ++t) {
        fdtd_global_e_kernel<T><<<(int)blocks, threads, 0, st>>>(a, t);
        fdtd_global_h_kernel<T><<<(int)blocks, threads, 0, st>>>(a, t);
        fdtd_global_probe_kernel<T><<<(int)blocks, threads, 0, st>>>(a, t);
    }
    fdtd_global_finish_kernel<T><<<(int)blocks, threads, 0, st>>>(a);
    return cuda_status(cudaGetLastError());
}

}  // namespace fdtdpic
