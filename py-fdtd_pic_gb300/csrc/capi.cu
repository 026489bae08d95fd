// C ABI of libfdtdpic.so: argument checks and dispatch to the typed launchers.
#include <stddef.h>
#include <string.h>

#include <math.h>

#include "fdtd1d_launch.cuh"
#include "pic_kernel.cuh"
#include "pic_pass.cuh"

#include <atomic>

namespace fdtdpic {

static std::atomic<long long> g_tiled_deadline_ns{0};

long long tiled_deadline_override_ns() { return g_tiled_deadline_ns.load(); }

int cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return FDTDPIC_OK;
    if (e == cudaErrorMemoryAllocation) return FDTDPIC_ERR_OOM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ||
        e == cudaErrorNoKernelImageForDevice)
        return FDTDPIC_ERR_NODEV;
    return FDTDPIC_ERR_CUDA;
}

int run_batch_f64(const BatchArgs<double> &a, int threads, int grid, cudaStream_t st);
int run_batch_f32(const BatchArgs<float> &a, int threads, int grid, cudaStream_t st);
int run_global_f64(const FdtdInstance &h, const BatchArgs<double> &a, cudaStream_t st);
int run_global_f32(const FdtdInstance &h, const BatchArgs<float> &a, cudaStream_t st);
int run_cubic_root0(int n, const double *coef, double *out, cudaStream_t st);
int run_pic_f64(const FdtdInstance &h, const BatchArgs<double> &fa, const PicBeam &bm,
                int32_t *cell, double *frac, double *ux, double *uz, int32_t *id, double *jx,
                double *jz, double *hyp, unsigned char *scratch, int32_t *status,
                FdtdPicTiming *timing, cudaStream_t st, bool allow_graphs = true);
int run_pic_f32(const FdtdInstance &h, const BatchArgs<float> &fa, const PicBeam &bm,
                int32_t *cell, float *frac, float *ux, float *uz, int32_t *id, float *jx,
                float *jz, float *hyp, unsigned char *scratch, int32_t *status,
                FdtdPicTiming *timing, cudaStream_t st, bool allow_graphs = true);

int run_pic_tiled_f64(const FdtdInstance &h, const BatchArgs<double> &fa, const PicBeam &bm,
                      const TileGeom &g, int32_t *cell, double *frac, double *ux, double *uz,
                      int32_t *id, double *jx, double *jz, double *hyp, unsigned char *scratch,
                      int32_t *status, FdtdPicTiming *timing, cudaStream_t st);
int run_pic_tiled_f32(const FdtdInstance &h, const BatchArgs<float> &fa, const PicBeam &bm,
                      const TileGeom &g, int32_t *cell, float *frac, float *ux, float *uz,
                      int32_t *id, float *jx, float *jz, float *hyp, unsigned char *scratch,
                      int32_t *status, FdtdPicTiming *timing, cudaStream_t st);

int run_pic_pass_f64(const FdtdInstance &h, const BatchArgs<double> &fa, const PicBeam &bm,
                     const PassGeom &g, int32_t *cell, double *frac, double *ux, double *uz,
                     int32_t *id, double *jx, double *jz, double *hyp, unsigned char *scratch,
                     int32_t *status, FdtdPicTiming *timing, cudaStream_t st);
int run_pic_pass_f32(const FdtdInstance &h, const BatchArgs<float> &fa, const PicBeam &bm,
                     const PassGeom &g, int32_t *cell, float *frac, float *ux, float *uz,
                     int32_t *id, float *jx, float *jz, float *hyp, unsigned char *scratch,
                     int32_t *status, FdtdPicTiming *timing, cudaStream_t st);

// Geometry of the temporally blocked path (path mode 3) on the current device, or ok=false when
// it does not apply (the beam must also be inside its domain: FDTDPIC_PATH_CELLS_INSIDE).
static PassGeom pass_geometry_dev(int precision, const FdtdInstance &h, const PicBeam &b)
{
    PassGeom g{};
    int dev = 0, max_optin = 0;
    if ((b.path & FDTDPIC_PATH_MODE) != 3 || !(b.path & FDTDPIC_PATH_CELLS_INSIDE) ||
        cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess)
        return g;
    return pass_geometry(precision, h, b, max_optin);
}

// Tiling of a beam run on the current device, or ok=false when the tiled path does not apply
// (fewer than two tiles of the minimum width, or a tile's fields beyond shared memory).
static TileGeom tiled_geometry(int precision, const FdtdInstance &h, const PicBeam &b)
{
    TileGeom g{};
    int dev = 0, sms = 0, max_optin = 0;
    if ((b.path & FDTDPIC_PATH_MODE) != 2 || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess)
        return g;
    g = tile_geometry(h, b, sms);
    // 1 KiB stays for the kernel's static shared variables
    if (g.ok && tile_smem_bytes(precision, g.wmax) > (int64_t)max_optin - 1024) g.ok = false;
    return g;
}

// ---- captured PIC step blocks (replayed by calls with identical arguments) -------------
static PicGraphEntry g_graphs[16];
static int g_graph_count = 0, g_graph_next = 0;

PicGraphEntry *pic_graph_lookup(const void *key, size_t len)
{
    for (int i = 0; i < g_graph_count; ++i)
        if (g_graphs[i].key_len == len && memcmp(g_graphs[i].key, key, len) == 0) return &g_graphs[i];
    return nullptr;
}

void pic_graph_store(const void *key, size_t len, cudaGraphExec_t exec)
{
    if (len > sizeof(g_graphs[0].key)) return;
    PicGraphEntry &e = g_graphs[g_graph_next];
    // an evicted graph may still be running: cudaGraphExecDestroy frees an executable graph that
    // is in flight when its launches complete, so no device-wide wait is needed here
    if (g_graph_next < g_graph_count && e.exec) cudaGraphExecDestroy(e.exec);
    memcpy(e.key, key, len);
    e.key_len = len;
    e.exec = exec;
    g_graph_next = (g_graph_next + 1) % 16;
    if (g_graph_count < 16) ++g_graph_count;
}

cudaStream_t pic_capture_stream()
{
    static cudaStream_t streams[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    if (!streams[dev] && cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking) != cudaSuccess)
        return nullptr;
    return streams[dev];
}

int check_instance(const FdtdInstance &I)
{
    if (I.nz < 2 || I.nz > FDTDPIC_MAX_CELLS || I.n_steps < 0 || I.step_begin < 0 ||
        I.step_end < I.step_begin ||
        I.step_end > I.n_steps)
        return FDTDPIC_ERR_ARG;
    if (I.pml < 0 || 2 * (int64_t)I.pml + 1 > (int64_t)I.nz + 1) return FDTDPIC_ERR_ARG;
    if (I.mode < FDTD_MODE_FREESPACE || I.mode > FDTD_MODE_KERR) return FDTDPIC_ERR_ARG;
    if (I.nzsrc < 0 || I.nzsrc > I.nz) return FDTDPIC_ERR_ARG;
    if (I.front < 0 || I.rear < I.front || I.rear > I.nz) return FDTDPIC_ERR_ARG;
    for (int p = 0; p < 2; ++p)
        if (I.probe_lo[p] <= I.probe_hi[p] && (I.probe_cell[p] < 0 || I.probe_cell[p] > I.nz))
            return FDTDPIC_ERR_ARG;
    if (I.hist_interval < 0 || I.hist_rows < 0) return FDTDPIC_ERR_ARG;
    if (I.sc == 0.0) return FDTDPIC_ERR_ARG;
    return FDTDPIC_OK;
}

}  // namespace fdtdpic

using namespace fdtdpic;

extern "C" {

int fdtdpic_abi_version(void) { return FDTDPIC_ABI_VERSION; }

const char *fdtdpic_strerror(int code)
{
    switch (code) {
    case FDTDPIC_OK: return "ok";
    case FDTDPIC_ERR_ARG: return "invalid argument";
    case FDTDPIC_ERR_OOM: return "does not fit in memory";
    case FDTDPIC_ERR_TIMEOUT: return "device-side wait timed out";
    case FDTDPIC_ERR_NUMERIC: return "non-finite state";
    case FDTDPIC_ERR_CUDA: return "CUDA runtime error";
    case FDTDPIC_ERR_NODEV: return "no usable sm_103 device";
    default: return "unknown error";
    }
}

int fdtdpic_instance_layout(int64_t *out, int n)
{
    const int64_t v[] = {
        (int64_t)sizeof(FdtdInstance),
        offsetof(FdtdInstance, nz), offsetof(FdtdInstance, n_steps),
        offsetof(FdtdInstance, step_begin), offsetof(FdtdInstance, step_end),
        offsetof(FdtdInstance, pml), offsetof(FdtdInstance, cpml_lo),
        offsetof(FdtdInstance, cpml_hi), offsetof(FdtdInstance, front),
        offsetof(FdtdInstance, rear), offsetof(FdtdInstance, nzsrc),
        offsetof(FdtdInstance, tfsf), offsetof(FdtdInstance, mode),
        offsetof(FdtdInstance, pol_active), offsetof(FdtdInstance, resume),
        offsetof(FdtdInstance, hist_interval), offsetof(FdtdInstance, hist_rows),
        offsetof(FdtdInstance, probe_cell), offsetof(FdtdInstance, probe_lo),
        offsetof(FdtdInstance, probe_hi), offsetof(FdtdInstance, ue),
        offsetof(FdtdInstance, ue_slab), offsetof(FdtdInstance, uh),
        offsetof(FdtdInstance, uh_slab), offsetof(FdtdInstance, dtdz),
        offsetof(FdtdInstance, eps0), offsetof(FdtdInstance, sc),
        offsetof(FdtdInstance, pol_a), offsetof(FdtdInstance, pol_b),
        offsetof(FdtdInstance, pol_c), offsetof(FdtdInstance, kerr_a),
        offsetof(FdtdInstance, kerr_b), offsetof(FdtdInstance, kerr_c),
        offsetof(FdtdInstance, nl_e0), offsetof(FdtdInstance, nl_e0chi),
        offsetof(FdtdInstance, pml_offset), offsetof(FdtdInstance, src_offset),
        offsetof(FdtdInstance, probe_offset), offsetof(FdtdInstance, state_offset),
        offsetof(FdtdInstance, hist_offset), offsetof(FdtdInstance, srcs_offset)};
    const int nv = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n && i < nv; ++i) out[i] = v[i];
    return nv;
}

int fdtdpic_device_sms(int *sms)
{
    int dev = 0;
    if (!sms) return FDTDPIC_ERR_ARG;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e);
    return cuda_status(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev));
}

int64_t fdtd1d_resident_smem_bytes(const FdtdInstance *inst, int precision)
{
    if (!inst || (precision != FDTDPIC_F64 && precision != FDTDPIC_F32)) return 0;
    if (check_instance(*inst) != FDTDPIC_OK) return 0;
    const int64_t bytes = (precision == FDTDPIC_F64 ? resident_elems<double>(*inst) * 8
                                                    : resident_elems<float>(*inst) * 4);
    // 227 KiB is the sm_100-family opt-in maximum per CTA, of which 1 KiB stays for the
    // kernel's static shared variables; the launch re-checks the device.
    return bytes <= 226 * 1024 ? bytes : 0;
}

int fdtd1d_run_batch(int precision, int n_inst, const FdtdInstance *d_inst, const int32_t *d_order,
                     const double *d_pml_tab, const double *d_src, void *d_state, void *d_probe,
                     void *d_hist, int32_t *d_queue, int32_t *d_status, int32_t *d_fallbacks,
                     int64_t smem_bytes, int threads_per_cta, int grid_ctas,
                     fdtdpic_stream_t stream)
{
    if (n_inst <= 0) return n_inst == 0 ? FDTDPIC_OK : FDTDPIC_ERR_ARG;
    if (!d_inst || !d_pml_tab || !d_src || !d_state || !d_probe || !d_queue)
        return FDTDPIC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == FDTDPIC_F64) {
        BatchArgs<double> a{n_inst, d_inst, d_order, d_pml_tab, d_src, (double *)d_state,
                            (double *)d_probe, (double *)d_hist, d_queue, d_status, d_fallbacks,
                            smem_bytes};
        return run_batch_f64(a, threads_per_cta, grid_ctas, st);
    }
    if (precision == FDTDPIC_F32) {
        BatchArgs<float> a{n_inst, d_inst, d_order, d_pml_tab, d_src, (float *)d_state,
                           (float *)d_probe, (float *)d_hist, d_queue, d_status, d_fallbacks,
                           smem_bytes};
        return run_batch_f32(a, threads_per_cta, grid_ctas, st);
    }
    return FDTDPIC_ERR_ARG;
}

int fdtd1d_run_global(int precision, const FdtdInstance *h_inst, const FdtdInstance *d_inst,
                      const double *d_pml_tab, const double *d_src, void *d_state, void *d_probe,
                      void *d_hist, int32_t *d_status, int32_t *d_fallbacks,
                      fdtdpic_stream_t stream)
{
    if (!h_inst || !d_inst || !d_pml_tab || !d_src || !d_state || !d_probe) return FDTDPIC_ERR_ARG;
    int rc = check_instance(*h_inst);
    if (rc != FDTDPIC_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == FDTDPIC_F64) {
        BatchArgs<double> a{1, d_inst, nullptr, d_pml_tab, d_src, (double *)d_state,
                            (double *)d_probe, (double *)d_hist, nullptr, d_status, d_fallbacks, 0};
        return run_global_f64(*h_inst, a, st);
    }
    if (precision == FDTDPIC_F32) {
        BatchArgs<float> a{1, d_inst, nullptr, d_pml_tab, d_src, (float *)d_state,
                           (float *)d_probe, (float *)d_hist, nullptr, d_status, d_fallbacks, 0};
        return run_global_f32(*h_inst, a, st);
    }
    return FDTDPIC_ERR_ARG;
}

int fdtdpic_cubic_root0(int n, const double *d_coef, double *d_out, fdtdpic_stream_t stream)
{
    if (n < 0 || (n > 0 && (!d_coef || !d_out))) return FDTDPIC_ERR_ARG;
    return run_cubic_root0(n, d_coef, d_out, (cudaStream_t)stream);
}

int64_t fdtdpic_scratch_bytes(int precision, int nz, int n_part)
{
    if ((precision != FDTDPIC_F64 && precision != FDTDPIC_F32) || nz < 2 || n_part < 0) return 0;
    return (int64_t)pic_scratch_layout(precision, nz, n_part).total;
}

double fdtdpic_pic_jscale(const PicBeam *bm)
{
    if (!bm || bm->n_part < 0) return 0.0;
    // |one node's sum| <= n_part * max(|kJ|, |kJz|) (|ux/gamma| < 1, |cell displacement| < 1)
    const double bound = (double)(bm->n_part > 0 ? bm->n_part : 1) *
                         fmax(fabs(bm->kJ), fabs(bm->kJz)) * 1.0001;
    if (!(bound > 0.0) || !isfinite(bound)) return 1.0;
    const int S = (int)floor(62.0 - log2(bound));
    return ldexp(1.0, S);
}

int64_t fdtdpic_pic_scratch_bytes(int precision, const FdtdInstance *inst, const PicBeam *beam)
{
    if (!inst || !beam || (precision != FDTDPIC_F64 && precision != FDTDPIC_F32)) return 0;
    if (check_instance(*inst) != FDTDPIC_OK) return 0;
    int64_t need = fdtdpic_scratch_bytes(precision, inst->nz, beam->n_part);
    const PassGeom pg = pass_geometry_dev(precision, *inst, *beam);
    if (pg.ok) return (int64_t)pass_scratch_layout(precision, inst->nz, pg).total;
    const TileGeom tg = tiled_geometry(precision, *inst, *beam);
    if (tg.ok) {
        const int64_t t = (int64_t)tile_scratch_layout(precision, tg).total;
        const bool tiled = (beam->path & FDTDPIC_PATH_MODE) == 2;
        if (tiled || t > need) need = tiled ? t : (t > need ? t : need);
    }
    return need;
}

int fdtdpic_pass_plan(int precision, const FdtdInstance *inst, const PicBeam *beam,
                      int64_t smem_optin, int64_t *out, int n_out)
{
    if (!inst || !beam || (precision != FDTDPIC_F64 && precision != FDTDPIC_F32) || smem_optin < 0)
        return FDTDPIC_ERR_ARG;
    if (check_instance(*inst) != FDTDPIC_OK) return FDTDPIC_ERR_ARG;
    const PicBeam &b = *beam;
    if (b.n_part < 0 || b.n_part > FDTDPIC_MAX_PARTICLES || b.clo < 2 || b.chi <= b.clo ||
        b.chi > inst->nz - 2 || b.sort_every < 0 || b.chunk < 0)
        return FDTDPIC_ERR_ARG;
    const PassGeom g = pass_geometry(precision, *inst, b, smem_optin);
    if (!g.ok) return FDTDPIC_ERR_ARG;
    const int64_t v[] = {g.S, g.H, g.G, g.wmin, g.wmax, g.Lmax, g.pcap, g.smem1, g.smem2,
                         (int64_t)pass_scratch_layout(precision, inst->nz, g).total};
    const int nv = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; out && i < n_out && i < nv; ++i) out[i] = v[i];
    return nv;
}

int fdtdpic_run(int precision, const FdtdInstance *h_inst, const FdtdInstance *d_inst,
                const double *d_pml_tab, const double *d_src, void *d_state, void *d_probe,
                const PicBeam *beam, int32_t *d_cell, void *d_frac, void *d_ux, void *d_uz,
                int32_t *d_id, void *d_jx, void *d_jz, void *d_hyp, void *d_scratch,
                int64_t scratch_bytes, int32_t *d_status, FdtdPicTiming *timing,
                fdtdpic_stream_t stream)
{
    if (!h_inst || !d_inst || !d_pml_tab || !d_src || !d_state || !d_probe || !beam || !d_jx ||
        !d_jz || !d_hyp || !d_scratch || !d_status)
        return FDTDPIC_ERR_ARG;
    int rc = check_instance(*h_inst);
    if (rc != FDTDPIC_OK) return rc;
    const PicBeam &b = *beam;
    // |cell displacement| per step < sc must stay below one cell for the Jz deposit
    if (b.n_part < 0 || b.n_part > FDTDPIC_MAX_PARTICLES || b.clo < 2 || b.chi <= b.clo ||
        b.chi > h_inst->nz - 2 || b.sort_every < 0 || b.chunk < 0 || !(b.jscale > 0.0) ||
        !(b.sc > 0.0 && b.sc < 1.0))
        return FDTDPIC_ERR_ARG;
    if (b.n_part > 0 && (!d_cell || !d_frac || !d_ux || !d_uz || !d_id)) return FDTDPIC_ERR_ARG;
    if (precision != FDTDPIC_F64 && precision != FDTDPIC_F32) return FDTDPIC_ERR_ARG;
    if ((b.path & ~(FDTDPIC_PATH_MODE | FDTDPIC_PATH_CELLS_INSIDE)) != 0 ||
        (b.path & FDTDPIC_PATH_MODE) > 3)
        return FDTDPIC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *scr = (unsigned char *)d_scratch;
    if ((b.path & FDTDPIC_PATH_MODE) == 3) {
        const PassGeom pg = pass_geometry_dev(precision, *h_inst, b);
        if (!pg.ok) return FDTDPIC_ERR_ARG;
        if (scratch_bytes < (int64_t)pass_scratch_layout(precision, h_inst->nz, pg).total)
            return FDTDPIC_ERR_OOM;
        if (precision == FDTDPIC_F64) {
            BatchArgs<double> a{1, d_inst, nullptr, d_pml_tab, d_src, (double *)d_state,
                                (double *)d_probe, nullptr, nullptr, nullptr, nullptr, 0};
            return run_pic_pass_f64(*h_inst, a, b, pg, d_cell, (double *)d_frac, (double *)d_ux,
                                    (double *)d_uz, d_id, (double *)d_jx, (double *)d_jz,
                                    (double *)d_hyp, scr, d_status, timing, st);
        }
        BatchArgs<float> a{1, d_inst, nullptr, d_pml_tab, d_src, (float *)d_state,
                           (float *)d_probe, nullptr, nullptr, nullptr, nullptr, 0};
        return run_pic_pass_f32(*h_inst, a, b, pg, d_cell, (float *)d_frac, (float *)d_ux,
                                (float *)d_uz, d_id, (float *)d_jx, (float *)d_jz,
                                (float *)d_hyp, scr, d_status, timing, st);
    }
    const TileGeom tg = tiled_geometry(precision, *h_inst, b);
    const int64_t tiled_need = tg.ok ? (int64_t)tile_scratch_layout(precision, tg).total : -1;
    if (tg.ok && scratch_bytes >= tiled_need) {
        if (precision == FDTDPIC_F64) {
            BatchArgs<double> a{1, d_inst, nullptr, d_pml_tab, d_src, (double *)d_state,
                                (double *)d_probe, nullptr, nullptr, nullptr, nullptr, 0};
            return run_pic_tiled_f64(*h_inst, a, b, tg, d_cell, (double *)d_frac, (double *)d_ux,
                                     (double *)d_uz, d_id, (double *)d_jx, (double *)d_jz,
                                     (double *)d_hyp, scr, d_status, timing, st);
        }
        BatchArgs<float> a{1, d_inst, nullptr, d_pml_tab, d_src, (float *)d_state,
                           (float *)d_probe, nullptr, nullptr, nullptr, nullptr, 0};
        return run_pic_tiled_f32(*h_inst, a, b, tg, d_cell, (float *)d_frac, (float *)d_ux,
                                 (float *)d_uz, d_id, (float *)d_jx, (float *)d_jz,
                                 (float *)d_hyp, scr, d_status, timing, st);
    }
    if ((b.path & FDTDPIC_PATH_MODE) == 2) return tg.ok ? FDTDPIC_ERR_OOM : FDTDPIC_ERR_ARG;
    if (scratch_bytes < fdtdpic_scratch_bytes(precision, h_inst->nz, b.n_part)) return FDTDPIC_ERR_OOM;
    if (precision == FDTDPIC_F64) {
        BatchArgs<double> a{1, d_inst, nullptr, d_pml_tab, d_src, (double *)d_state,
                            (double *)d_probe, nullptr, nullptr, nullptr, nullptr, 0};
        return run_pic_f64(*h_inst, a, b, d_cell, (double *)d_frac, (double *)d_ux,
                           (double *)d_uz, d_id, (double *)d_jx, (double *)d_jz,
                           (double *)d_hyp, scr, d_status, timing, st);
    }
    BatchArgs<float> a{1, d_inst, nullptr, d_pml_tab, d_src, (float *)d_state, (float *)d_probe,
                       nullptr, nullptr, nullptr, nullptr, 0};
    return run_pic_f32(*h_inst, a, b, d_cell, (float *)d_frac, (float *)d_ux, (float *)d_uz,
                       d_id, (float *)d_jx, (float *)d_jz, (float *)d_hyp, scr, d_status, timing, st);
}

}  // extern "C"

extern "C" int fdtdpic_set_run_deadline(int64_t ns)
{
    if (ns < 0) return FDTDPIC_ERR_ARG;
    fdtdpic::g_tiled_deadline_ns.store((long long)ns);
    return FDTDPIC_OK;
}
