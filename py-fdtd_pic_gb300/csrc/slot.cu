// C ABI of the served-request slots (fdtdpic_slot_*, fdtdpic_slots_run).  Built with
// -fmad=false, like the PIC units, so a beam request's step rounds as fdtdpic_run's does.
#include <stddef.h>

#include "slot_kernel.cuh"

namespace fdtdpic {

int check_instance(const FdtdInstance &I);

// CTAs per SM the slot kernel runs at with this block size and shared memory (0 on error).
template <typename T>
static int slots_per_sm(int threads, int64_t smem_bytes)
{
    int per_sm = 0;
    if (cudaFuncSetAttribute(fdtdpic_slot_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_bytes) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fdtdpic_slot_kernel<T>, threads,
                                                      (size_t)smem_bytes) != cudaSuccess)
        return 0;
    return per_sm;
}

template <typename T>
static int launch_slots(const SlotArgs &a, int threads, int grid, cudaStream_t st)
{
    int dev = 0, sms = 0, max_optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FDTDPIC_ERR_NODEV;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    // 1 KiB stays for the kernel's static shared variables
    if (a.smem_bytes < 0 || a.smem_bytes > (int64_t)max_optin - 1024) return FDTDPIC_ERR_OOM;
    if (threads <= 0) threads = 512;
    if (threads > 1024 || (threads % 32) != 0) return FDTDPIC_ERR_ARG;
    auto kern = fdtdpic_slot_kernel<T>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)a.smem_bytes);
    if (e != cudaSuccess) return cuda_status(e);
    if (grid <= 0) {
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads,
                                                          (size_t)a.smem_bytes);
        if (e != cudaSuccess) return cuda_status(e);
        if (per_sm < 1) return FDTDPIC_ERR_OOM;
        grid = per_sm * sms;
    }
    if (grid > a.n_items) grid = a.n_items;
    e = cudaMemsetAsync(a.queue, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) return cuda_status(e);
    kern<<<grid, threads, (size_t)a.smem_bytes, st>>>(a);
    return cuda_status(cudaGetLastError());
}

}  // namespace fdtdpic

using namespace fdtdpic;

extern "C" {

int fdtdpic_slot_layout(int64_t *out, int n)
{
    const int64_t v[] = {
        (int64_t)sizeof(FdtdSlot),          offsetof(FdtdSlot, inst),
        offsetof(FdtdSlot, pml_tab),        offsetof(FdtdSlot, src),
        offsetof(FdtdSlot, state),          offsetof(FdtdSlot, probe),
        offsetof(FdtdSlot, hist),           offsetof(FdtdSlot, n_part),
        offsetof(FdtdSlot, clo),            offsetof(FdtdSlot, chi),
        offsetof(FdtdSlot, reserved),       offsetof(FdtdSlot, cell),
        offsetof(FdtdSlot, frac),           offsetof(FdtdSlot, ux),
        offsetof(FdtdSlot, uz),             offsetof(FdtdSlot, hyp),
        offsetof(FdtdSlot, jx),             offsetof(FdtdSlot, jz),
        offsetof(FdtdSlot, acc),            offsetof(FdtdSlot, kE),
        offsetof(FdtdSlot, kH),             offsetof(FdtdSlot, sc),
        offsetof(FdtdSlot, kJ),             offsetof(FdtdSlot, kJz),
        offsetof(FdtdSlot, jscale),         offsetof(FdtdSlot, status),
        (int64_t)sizeof(FdtdSlotItem)};
    const int total = (int)(sizeof(v) / sizeof(v[0]));
    if (out)
        for (int i = 0; i < n && i < total; ++i) out[i] = v[i];
    return total;
}

int fdtdpic_slot_check(int precision, const FdtdSlot *s)
{
    if (!s || (precision != FDTDPIC_F64 && precision != FDTDPIC_F32)) return FDTDPIC_ERR_ARG;
    const FdtdInstance &I = s->inst;
    if (check_instance(I) != FDTDPIC_OK) return FDTDPIC_ERR_ARG;
    if (!s->pml_tab || !s->src || !s->state || !s->probe) return FDTDPIC_ERR_ARG;
    if (I.hist_rows > 0 && I.hist_interval > 0 && !s->hist) return FDTDPIC_ERR_ARG;
    if (s->n_part < 0 || s->n_part > FDTDPIC_MAX_PARTICLES) return FDTDPIC_ERR_ARG;
    if (s->n_part > 0) {
        if (s->clo < 2 || s->chi <= s->clo || s->chi > I.nz - 2) return FDTDPIC_ERR_ARG;
        if (!s->cell || !s->frac || !s->ux || !s->uz || !s->hyp || !s->jx || !s->jz || !s->acc)
            return FDTDPIC_ERR_ARG;
        if (!(s->jscale > 0.0) || !(s->sc > 0.0 && s->sc < 1.0)) return FDTDPIC_ERR_ARG;
    }
    return FDTDPIC_OK;
}

int64_t fdtdpic_slot_smem_bytes(int precision, const FdtdSlot *s)
{
    if (fdtdpic_slot_check(precision, s) != FDTDPIC_OK) return 0;
    const int64_t n = (int64_t)s->inst.nz + 1;
    if (s->n_part > 0) return 2 * (precision == FDTDPIC_F64 ? 2 : 1) * n * 8;
    return precision == FDTDPIC_F64 ? resident_elems<double>(s->inst) * 8
                                    : resident_elems<float>(s->inst) * 4;
}

int fdtdpic_slots_grid(int precision, int64_t smem_bytes, int threads_per_cta)
{
    int dev = 0, sms = 0, max_optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem_bytes < 0 || smem_bytes > (int64_t)max_optin - 1024) return 0;
    if (threads_per_cta <= 0) threads_per_cta = 512;
    if (threads_per_cta > 1024 || (threads_per_cta % 32) != 0) return 0;
    int per_sm = 0;
    if (precision == FDTDPIC_F64) per_sm = slots_per_sm<double>(threads_per_cta, smem_bytes);
    else if (precision == FDTDPIC_F32) per_sm = slots_per_sm<float>(threads_per_cta, smem_bytes);
    return per_sm * sms;
}

int fdtdpic_slots_run(int precision, FdtdSlot *d_slots, int n_slots, const FdtdSlotItem *d_items,
                      int n_items, int32_t *d_queue, int64_t smem_bytes, int threads_per_cta,
                      int grid_ctas, fdtdpic_stream_t stream)
{
    if (n_items < 0 || n_slots < 0) return FDTDPIC_ERR_ARG;
    if (n_items == 0) return FDTDPIC_OK;
    if (!d_slots || !d_items || !d_queue) return FDTDPIC_ERR_ARG;
    const SlotArgs a{d_slots, n_slots, d_items, n_items, d_queue, smem_bytes};
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == FDTDPIC_F64) return launch_slots<double>(a, threads_per_cta, grid_ctas, st);
    if (precision == FDTDPIC_F32) return launch_slots<float>(a, threads_per_cta, grid_ctas, st);
    return FDTDPIC_ERR_ARG;
}

}  // extern "C"
