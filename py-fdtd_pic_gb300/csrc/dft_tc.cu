// Batched probe DFT on the 5th-generation tensor cores (tcgen05, kind::f16, BF16 operands,
// FP32 accumulation in tensor memory), split-BF16x3.
//
// The DFT of real traces at F frequencies is the real GEMM
//     C[r][j] = sum_n x[r][n] B[n][j],   B[n][2q] = cos(2 pi f_q n dt), B[n][2q+1] = -sin(...)
// so C[r][2q], C[r][2q+1] are Re and Im of X[r, f_q] (the interleaved output of
// fdtdpic_dft_probes).  Each operand is split into two BF16 halves, x = xh + xl and
// B = Bh + Bl (xl = bf16(x - xh)), and C ~= xh Bh + xh Bl + xl Bh: three BF16 MMAs per K step,
// about 16 significant bits per product, FP32 sums.  Time is walked in chunks of TC_KC steps;
// after each chunk the FP32 accumulator is read out of tensor memory and added into FP64 sums in
// shared memory, so FP32 rounding is bounded by one chunk's terms (as in the CUDA-core form).
//
// One CTA of 128 threads owns a 128-trace x 64-column tile (32 frequencies).  Per chunk all
// threads stage xh/xl and Bh/Bl into shared memory in the canonical no-swizzle K-major layout
// (8-row x 16-byte core matrices), one thread issues the 12 MMAs (4 K steps x 3 products) and
// commits them to an mbarrier, every thread waits (bounded), then reads its own row (tensor
// memory lane) with tcgen05.ld and adds it into the FP64 tile.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "fdtdpic.h"

namespace fdtdpic {

int cuda_status(cudaError_t e);

constexpr int TC_M = 128;          // traces per CTA = MMA M = tensor memory lanes
constexpr int TC_N = 64;           // output columns per CTA (32 frequencies x re/im) = MMA N
constexpr int TC_Q = TC_N / 2;     // frequencies per CTA
constexpr int TC_KC = 64;          // time steps per chunk
constexpr int TC_KSTEP = 16;       // K of one kind::f16 MMA
constexpr int TC_THREADS = 128;
constexpr int TC_TMEM_COLS = 64;   // FP32 accumulator columns (power of two >= 32)
// no-swizzle K-major layout: core matrix = 8 rows x 8 BF16 (128 B); LBO = next core matrix along
// K, SBO = next 8 rows
constexpr uint32_t TC_LBO = 128;
constexpr uint32_t TC_SBO = (TC_KC / 8) * 128;                 // 1024 B
constexpr uint32_t TC_A_BYTES = (TC_M / 8) * TC_SBO;            // 16 KiB per half
constexpr uint32_t TC_B_BYTES = (TC_N / 8) * TC_SBO;            // 8 KiB per half
constexpr uint32_t TC_ACC_BYTES = TC_M * TC_N * 8;              // FP64 tile, 64 KiB
constexpr uint32_t TC_SMEM = 2 * TC_A_BYTES + 2 * TC_B_BYTES + TC_ACC_BYTES + 64;
constexpr long long TC_WAIT_LIMIT = 1LL << 26;  // mbarrier polls before giving up

// Byte offset of element (row, k) of a K-major operand tile in the core-matrix layout.
__device__ __forceinline__ uint32_t tc_off(int row, int k)
{
    return (uint32_t)(row >> 3) * TC_SBO + (uint32_t)(k >> 3) * TC_LBO + (uint32_t)(row & 7) * 16 +
           (uint32_t)(k & 7) * 2;
}

// Shared-memory matrix descriptor: start >> 4 [0,14), LBO >> 4 [16,30), SBO >> 4 [32,46),
// descriptor version 1 [46,48), base offset 0, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((TC_LBO >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((TC_SBO >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor, kind::f16: D F32 [4,6)=1, A BF16 [7,10)=1, B BF16 [10,13)=1, both
// K-major, N >> 3 at [17,23), M >> 4 at [24,29).
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) |
                              ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(TC_IDESC), "r"(acc));
}

__device__ __forceinline__ void tc_split(float v, __nv_bfloat16 &hi, __nv_bfloat16 &lo)
{
    hi = __float2bfloat16_rn(v);
    lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

template <typename TIn>
__global__ void __launch_bounds__(TC_THREADS, 1)
    dft_tc_kernel(const TIn *x, int R, int S, int rp, int64_t ldp, int64_t sp, int64_t sn,
                  const float2 *tw, int F, double *out, int32_t *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *a_hi = sm, *a_lo = sm + TC_A_BYTES;
    unsigned char *b_hi = a_lo + TC_A_BYTES, *b_lo = b_hi + TC_B_BYTES;
    double *acc = reinterpret_cast<double *>(b_lo + TC_B_BYTES);  // [TC_N][TC_M]
    uint64_t *bar = reinterpret_cast<uint64_t *>(acc + TC_M * TC_N);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int r0 = blockIdx.y * TC_M, q0 = blockIdx.x * TC_Q;

    for (int i = tid; i < TC_M * TC_N; i += TC_THREADS) acc[i] = 0.0;
    const uint32_t bar_a = (uint32_t)__cvta_generic_to_shared(bar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {
        const uint32_t slot_a = (uint32_t)__cvta_generic_to_shared(tmem_slot);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_a),
                     "r"(TC_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    const uint32_t sa_hi = (uint32_t)__cvta_generic_to_shared(a_hi);
    const uint32_t sa_lo = (uint32_t)__cvta_generic_to_shared(a_lo);
    const uint32_t sb_hi = (uint32_t)__cvta_generic_to_shared(b_hi);
    const uint32_t sb_lo = (uint32_t)__cvta_generic_to_shared(b_lo);
    // this thread's tensor-memory lane (warp w reads lanes 32w..32w+31)
    const uint32_t t_row = tmem + ((uint32_t)(warp * 32) << 16);

    bool ok = true;
    int phase = 0;
    for (int n0 = 0; n0 < S && ok; n0 += TC_KC) {
        // stage the chunk: traces (rows r0.., k fastest) and twiddles (columns 2q, 2q+1)
        for (int i = tid; i < TC_M * TC_KC; i += TC_THREADS) {
            const int row = i / TC_KC, k = i % TC_KC;
            const int r = r0 + row, n = n0 + k;
            float v = 0.f;
            if (r < R && n < S)
                v = (float)x[(int64_t)(r / rp) * ldp + (int64_t)(r % rp) * sp + (int64_t)n * sn];
            __nv_bfloat16 h, l;
            tc_split(v, h, l);
            const uint32_t o = tc_off(row, k);
            *reinterpret_cast<__nv_bfloat16 *>(a_hi + o) = h;
            *reinterpret_cast<__nv_bfloat16 *>(a_lo + o) = l;
        }
        for (int i = tid; i < TC_Q * TC_KC; i += TC_THREADS) {
            const int q = i / TC_KC, k = i % TC_KC;
            const int f = q0 + q, n = n0 + k;
            const float2 w = (f < F && n < S) ? tw[(int64_t)f * S + n] : make_float2(0.f, 0.f);
            __nv_bfloat16 h, l;
            tc_split(w.x, h, l);
            *reinterpret_cast<__nv_bfloat16 *>(b_hi + tc_off(2 * q, k)) = h;
            *reinterpret_cast<__nv_bfloat16 *>(b_lo + tc_off(2 * q, k)) = l;
            tc_split(w.y, h, l);
            *reinterpret_cast<__nv_bfloat16 *>(b_hi + tc_off(2 * q + 1, k)) = h;
            *reinterpret_cast<__nv_bfloat16 *>(b_lo + tc_off(2 * q + 1, k)) = l;
        }
        // generic-proxy stores -> visible to the tensor cores (async proxy)
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < TC_KC / TC_KSTEP; ++s) {
                const uint32_t ko = (uint32_t)s * 2 * TC_LBO;  // two core matrices per K step
                tc_mma(tmem, tc_desc(sa_hi + ko), tc_desc(sb_hi + ko), s > 0 ? 1u : 0u);
                tc_mma(tmem, tc_desc(sa_hi + ko), tc_desc(sb_lo + ko), 1u);
                tc_mma(tmem, tc_desc(sa_lo + ko), tc_desc(sb_hi + ko), 1u);
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    bar_a));
        }
        // wait for the chunk's MMAs (bounded); the CTA decides together whether they completed
        long long spins = 0;
        uint32_t done = 0;
        while (!done) {
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}\n"
                : "=r"(done)
                : "r"(bar_a), "r"(phase));
            if (!done && ++spins > TC_WAIT_LIMIT) break;
        }
        if (!__syncthreads_and((int)done)) {
            ok = false;
            if (tid == 0) atomicOr(err, 1);
            break;
        }
        phase ^= 1;
        asm volatile("tcgen05.fence::after_thread_sync;");
        // this thread's row of the FP32 accumulator -> FP64 sums
#pragma unroll
        for (int c0 = 0; c0 < TC_N; c0 += 16) {
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
                "%13,%14,%15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                  "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                  "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                : "r"(t_row + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
            for (int j = 0; j < 16; ++j) acc[(c0 + j) * TC_M + tid] += (double)__uint_as_float(v[j]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();  // operands and accumulator are free for the next chunk
        asm volatile("tcgen05.fence::after_thread_sync;");
    }
    // every thread left the loop at the same chunk (the CTA-wide vote above); on a timeout the
    // MMAs already issued are waited for, bounded, before the tensor memory is freed
    if (!ok) {
        long long spins = 0;
        uint32_t done = 0;
        while (!done && ++spins < TC_WAIT_LIMIT)
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}\n"
                : "=r"(done)
                : "r"(bar_a), "r"(phase));
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TC_TMEM_COLS));
    if (!ok) return;
    const int r = r0 + tid;
    if (r < R)
        for (int c = 0; c < TC_N; ++c) {
            const int f = q0 + (c >> 1);
            if (f < F) out[((int64_t)r * F + f) * 2 + (c & 1)] = acc[c * TC_M + tid];
        }
}

}  // namespace fdtdpic

using namespace fdtdpic;

extern "C" {

int fdtdpic_dft_probes_tc(int precision, const void *d_traces, int R, int S, int rp, int64_t ldp,
                          int64_t sp, int64_t sn, const void *d_tw, int F, double *d_out,
                          int32_t *d_err, fdtdpic_stream_t stream)
{
    if (!d_traces || !d_tw || !d_out || !d_err || R < 0 || S <= 0 || F <= 0 || rp < 1 ||
        ldp < 0 || sp < 0 || sn < 1)
        return FDTDPIC_ERR_ARG;
    if (R == 0) return FDTDPIC_OK;
    int dev = 0, major = 0, minor = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FDTDPIC_ERR_NODEV;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major != 10 || minor != 3) return FDTDPIC_ERR_NODEV;  // built for sm_103a only
    dim3 grid((F + TC_Q - 1) / TC_Q, (R + TC_M - 1) / TC_M);
    if (grid.y > 65535) return FDTDPIC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    if (precision == FDTDPIC_F32) {
        e = cudaFuncSetAttribute(dft_tc_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)TC_SMEM);
        if (e != cudaSuccess) return cuda_status(e);
        dft_tc_kernel<float><<<grid, TC_THREADS, TC_SMEM, st>>>(
            (const float *)d_traces, R, S, rp, ldp, sp, sn, (const float2 *)d_tw, F, d_out, d_err);
    } else if (precision == FDTDPIC_F64) {
        e = cudaFuncSetAttribute(dft_tc_kernel<double>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
        if (e != cudaSuccess) return cuda_status(e);
        dft_tc_kernel<double><<<grid, TC_THREADS, TC_SMEM, st>>>(
            (const double *)d_traces, R, S, rp, ldp, sp, sn, (const float2 *)d_tw, F, d_out, d_err);
    } else {
        return FDTDPIC_ERR_ARG;
    }
    return cuda_status(cudaGetLastError());
}

}  // extern "C"
