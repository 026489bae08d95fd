// fdtdpic_run_noalloc: the beam + field step for callers that cannot allocate device memory.
//
// Some callers of this library own no allocator: code running inside another framework's
// memory pool that forbids side allocations, plug-ins loaded into a host that has already
// reserved the whole device, or a capture/replay harness that must not see cudaMalloc between
// its launches.  fdtdpic_run needs caller-provided scratch (deposit accumulators, re-binning
// buffers); this entry point takes that scratch from a fixed array compiled into the library
// instead, so the caller passes only its inputs and outputs.
//
// The array is NOALLOC_SCRATCH_BYTES (24 MiB) of file-scope __device__ memory: every GPU that
// loads the library holds it until the process exits.  Runs whose scratch need
// (fdtdpic_scratch_bytes) exceeds it are rejected with FDTDPIC_ERR_OOM.  All calls share the
// array: calls that overlap on the GPU (different streams, or different host threads) race on it
// and must be serialised by the caller.  Nothing needs to be cleared between calls: every scratch
// word a run reads it first writes (the accumulators and bin counts are zeroed at the start of
// the call).  On first use on a device the call looks up the array's device address
// (cudaGetSymbolAddress with that device current) and keeps it; make that first call before any
// stream capture.  The kept address belongs to the device's current context: a process that
// calls cudaDeviceReset must not call this entry point on that device afterwards (the array is
// reloaded at another address).  The call allocates nothing: no cudaMalloc/cudaFree, no graph
// capture, no event or stream creation.  It takes the streaming kernels only: the persistent
// tiled path (PicBeam.path mode 2) needs scratch sized per tile and is refused (ERR_ARG).
#include <cuda_runtime.h>

#include <mutex>

#include "fdtdpic.h"
#include "pic_kernel.cuh"

namespace fdtdpic {
int check_instance(const FdtdInstance &I);
int run_pic_f64(const FdtdInstance &h, const BatchArgs<double> &fa, const PicBeam &bm,
                int32_t *cell, double *frac, double *ux, double *uz, int32_t *id, double *jx,
                double *jz, double *hyp, unsigned char *scratch, int32_t *status,
                FdtdPicTiming *timing, cudaStream_t st, bool allow_graphs);
int run_pic_f32(const FdtdInstance &h, const BatchArgs<float> &fa, const PicBeam &bm,
                int32_t *cell, float *frac, float *ux, float *uz, int32_t *id, float *jx,
                float *jz, float *hyp, unsigned char *scratch, int32_t *status,
                FdtdPicTiming *timing, cudaStream_t st, bool allow_graphs);
}  // namespace fdtdpic

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(24) << 20;
constexpr int NOALLOC_MAX_DEVICES = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Host-side device addresses of g_noalloc_scratch, one per device (the symbol's host name is
// not a device address).
void *g_noalloc_ptr[NOALLOC_MAX_DEVICES];
std::mutex g_noalloc_lock;  // first calls from several host threads look the address up once

int noalloc_scratch(unsigned char **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fdtdpic::cuda_status(e);
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return FDTDPIC_ERR_NODEV;
    std::lock_guard<std::mutex> guard(g_noalloc_lock);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return e != cudaSuccess ? fdtdpic::cuda_status(e) : FDTDPIC_ERR_CUDA;
        g_noalloc_ptr[dev] = p;
    }
    *out = (unsigned char *)g_noalloc_ptr[dev];
    return FDTDPIC_OK;
}

}  // namespace

extern "C" int fdtdpic_run_noalloc(int precision, const FdtdInstance *h_inst,
                                   const FdtdInstance *d_inst, const double *d_pml_tab,
                                   const double *d_src, void *d_state, void *d_probe,
                                   const PicBeam *beam, int32_t *d_cell, void *d_frac, void *d_ux,
                                   void *d_uz, int32_t *d_id, void *d_jx, void *d_jz, void *d_hyp,
                                   int32_t *d_status, fdtdpic_stream_t stream)
{
    using namespace fdtdpic;
    if (!h_inst || !d_inst || !d_pml_tab || !d_src || !d_state || !d_probe || !beam || !d_jx ||
        !d_jz || !d_hyp || !d_status)
        return FDTDPIC_ERR_ARG;
    int rc = check_instance(*h_inst);
    if (rc != FDTDPIC_OK) return rc;
    const PicBeam &b = *beam;
    if (b.n_part < 0 || b.clo < 2 || b.chi <= b.clo || b.chi > h_inst->nz - 2 || b.sort_every < 0 ||
        b.chunk < 0 || !(b.jscale > 0.0) || !(b.sc > 0.0 && b.sc < 1.0))
        return FDTDPIC_ERR_ARG;
    if (b.n_part > 0 && (!d_cell || !d_frac || !d_ux || !d_uz || !d_id)) return FDTDPIC_ERR_ARG;
    if (precision != FDTDPIC_F64 && precision != FDTDPIC_F32) return FDTDPIC_ERR_ARG;
    // the path word as fdtdpic_run checks it; the tiled path (mode 2) is not available here
    if ((b.path & ~(FDTDPIC_PATH_MODE | FDTDPIC_PATH_CELLS_INSIDE)) != 0 ||
        (b.path & FDTDPIC_PATH_MODE) > 1)
        return FDTDPIC_ERR_ARG;
    const int64_t need = fdtdpic_scratch_bytes(precision, h_inst->nz, b.n_part);
    if (need <= 0 || need > (int64_t)NOALLOC_SCRATCH_BYTES) return FDTDPIC_ERR_OOM;
    unsigned char *scr = nullptr;
    rc = noalloc_scratch(&scr);
    if (rc != FDTDPIC_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == FDTDPIC_F64) {
        BatchArgs<double> a{1, d_inst, nullptr, d_pml_tab, d_src, (double *)d_state,
                            (double *)d_probe, nullptr, nullptr, nullptr, nullptr, 0};
        return run_pic_f64(*h_inst, a, b, d_cell, (double *)d_frac, (double *)d_ux,
                           (double *)d_uz, d_id, (double *)d_jx, (double *)d_jz,
                           (double *)d_hyp, scr, d_status, nullptr, st, false);
    }
    BatchArgs<float> a{1, d_inst, nullptr, d_pml_tab, d_src, (float *)d_state, (float *)d_probe,
                       nullptr, nullptr, nullptr, nullptr, 0};
    return run_pic_f32(*h_inst, a, b, d_cell, (float *)d_frac, (float *)d_ux, (float *)d_uz,
                       d_id, (float *)d_jx, (float *)d_jz, (float *)d_hyp, scr, d_status,
                       nullptr, st, false);
}
