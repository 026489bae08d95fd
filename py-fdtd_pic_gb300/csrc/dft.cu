// Batched probe-trace DFT: X[r, f] = sum_n x[r, n] exp(-2 pi i f_k n dt) for R traces and F
// frequencies, the contraction behind reflection-vs-frequency (TransformHandler.RefTester,
// TransformHandler.py:34-78, takes the FFT of each probe trace; here every requested
// frequency is evaluated directly, so frequencies need not sit on FFT bins).
//
// Twiddles: cos/sin(2 pi frac(f_k n dt)) with the phase reduced in FP64 (n up to 2^31, so the
// product needs FP64 before reduction) and the trigonometric values rounded to FP32, stored as
// a [F][S] table of float2 built once per (freqs, dt, S).
// Contraction: one CTA computes a 32-trace x 64-frequency tile; K (time) is walked in chunks of
// DFT_KC steps staged through shared memory; each thread accumulates its 2 x 4 complex outputs
// in FP32 within a chunk and adds the chunk into FP64 accumulators, which bounds the FP32
// rounding to one chunk's worth of terms.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "fdtdpic.h"

namespace fdtdpic {

int cuda_status(cudaError_t e);

constexpr int DFT_TR = 32;   // traces per CTA
constexpr int DFT_TF = 64;   // frequencies per CTA
constexpr int DFT_KC = 64;   // time steps per chunk
constexpr int DFT_THREADS = 256;

__global__ void dft_twiddle_kernel(const double *freqs, int F, int S, double dt, float2 *tw)
{
    const int64_t total = (int64_t)F * S;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(i / S);
        const int n = (int)(i % S);
        const double cyc = freqs[k] * dt * (double)n;  // cycles
        const double fr = cyc - floor(cyc);            // in [0, 1)
        float s, c;
        sincospif((float)(2.0 * fr), &s, &c);
        tw[i] = make_float2(c, -s);  // exp(-i 2 pi fr)
    }
}

// Trace r, sample n sits at x[(r / rp) * ldp + (r % rp) * sp + n * sn]: rp = 2, ldp = 2S,
// sp = 1, sn = 2 reads the engine's per-instance [steps][2] probe blocks in place.
template <typename TIn>
__global__ void __launch_bounds__(DFT_THREADS) dft_kernel(const TIn *x, int R, int S, int rp,
                                                          int64_t ldp, int64_t sp, int64_t sn,
                                                          const float2 *tw, int F, double *out)
{
    __shared__ float xs[DFT_KC][DFT_TR + 1];
    __shared__ float2 ts[DFT_KC][DFT_TF];
    const int r0 = blockIdx.y * DFT_TR, f0 = blockIdx.x * DFT_TF;
    const int tid = threadIdx.x;
    // thread tile: 2 traces x 4 frequencies; 16 x 16 threads
    const int tr = (tid / 16) * 2, tf = (tid % 16) * 4;
    double accr[2][4], acci[2][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) accr[a][b] = acci[a][b] = 0.0;
    for (int n0 = 0; n0 < S; n0 += DFT_KC) {
        for (int i = tid; i < DFT_KC * DFT_TR; i += DFT_THREADS) {
            const int kk = i % DFT_KC, rr = i / DFT_KC;
            const int r = r0 + rr, n = n0 + kk;
            xs[kk][rr] = (r < R && n < S) ? (float)x[(int64_t)(r / rp) * ldp + (int64_t)(r % rp) * sp + (int64_t)n * sn] : 0.f;
        }
        for (int i = tid; i < DFT_KC * DFT_TF; i += DFT_THREADS) {
            const int kk = i % DFT_KC, ff = i / DFT_KC;
            const int f = f0 + ff, n = n0 + kk;
            ts[kk][ff] = (f < F && n < S) ? tw[(int64_t)f * S + n] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        float cr[2][4], ci[2][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) cr[a][b] = ci[a][b] = 0.f;
#pragma unroll 4
        for (int kk = 0; kk < DFT_KC; ++kk) {
            const float x0 = xs[kk][tr], x1 = xs[kk][tr + 1];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const float2 w = ts[kk][tf + b];
                cr[0][b] = fmaf(x0, w.x, cr[0][b]);
                ci[0][b] = fmaf(x0, w.y, ci[0][b]);
                cr[1][b] = fmaf(x1, w.x, cr[1][b]);
                ci[1][b] = fmaf(x1, w.y, ci[1][b]);
            }
        }
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                accr[a][b] += (double)cr[a][b];
                acci[a][b] += (double)ci[a][b];
            }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int r = r0 + tr + a, f = f0 + tf + b;
            if (r < R && f < F) {
                out[((int64_t)r * F + f) * 2 + 0] = accr[a][b];
                out[((int64_t)r * F + f) * 2 + 1] = acci[a][b];
            }
        }
}

// |X_refl(f)| / |X_inc(f)| for pairs of traces (2i: incident, 2i+1: reflected/transmitted).
__global__ void dft_ratio_kernel(const double *X, int n_pairs, int F, double *ratio)
{
    const int64_t total = (int64_t)n_pairs * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = i / F, f = i % F;
        const double *a = X + ((2 * p) * F + f) * 2;
        const double *b = X + ((2 * p + 1) * F + f) * 2;
        const double ma = hypot(a[0], a[1]), mb = hypot(b[0], b[1]);
        ratio[i] = ma > 0.0 ? mb / ma : 0.0;
    }
}

}  // namespace fdtdpic

using namespace fdtdpic;

extern "C" {

int64_t fdtdpic_dft_twiddle_bytes(int F, int S)
{
    if (F <= 0 || S <= 0) return 0;
    return (int64_t)F * S * (int64_t)sizeof(float2);
}

int fdtdpic_dft_twiddles(const double *d_freqs, int F, int S, double dt, void *d_tw,
                         fdtdpic_stream_t stream)
{
    if (!d_freqs || !d_tw || F <= 0 || S <= 0 || !(dt > 0.0)) return FDTDPIC_ERR_ARG;
    const int64_t total = (int64_t)F * S;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 8192) blocks = 8192;
    dft_twiddle_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_freqs, F, S, dt, (float2 *)d_tw);
    return cuda_status(cudaGetLastError());
}

int fdtdpic_dft_probes(int precision, const void *d_traces, int R, int S, int rp, int64_t ldp,
                       int64_t sp, int64_t sn, const void *d_tw, int F, double *d_out,
                       fdtdpic_stream_t stream)
{
    if (!d_traces || !d_tw || !d_out || R < 0 || S <= 0 || F <= 0 || rp < 1 || ldp < 0 ||
        sp < 0 || sn < 1)
        return FDTDPIC_ERR_ARG;
    if (R == 0) return FDTDPIC_OK;
    dim3 grid((F + DFT_TF - 1) / DFT_TF, (R + DFT_TR - 1) / DFT_TR);
    if (grid.y > 65535) return FDTDPIC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == FDTDPIC_F32)
        dft_kernel<float><<<grid, DFT_THREADS, 0, st>>>((const float *)d_traces, R, S, rp, ldp, sp,
                                                        sn, (const float2 *)d_tw, F, d_out);
    else if (precision == FDTDPIC_F64)
        dft_kernel<double><<<grid, DFT_THREADS, 0, st>>>((const double *)d_traces, R, S, rp, ldp,
                                                         sp, sn, (const float2 *)d_tw, F, d_out);
    else
        return FDTDPIC_ERR_ARG;
    return cuda_status(cudaGetLastError());
}

int fdtdpic_reflection_ratio(const double *d_X, int n_pairs, int F, double *d_ratio,
                             fdtdpic_stream_t stream)
{
    if (!d_X || !d_ratio || n_pairs < 0 || F <= 0) return FDTDPIC_ERR_ARG;
    if (n_pairs == 0) return FDTDPIC_OK;
    const int64_t total = (int64_t)n_pairs * F;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 8192) blocks = 8192;
    dft_ratio_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_X, n_pairs, F, d_ratio);
    return cuda_status(cudaGetLastError());
}

}  // extern "C"
