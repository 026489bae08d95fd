// Batched probe DFT on the 5th-generation tensor cores (tcgen05, kind::f16, BF16 operands,
// FP32 accumulation in tensor memory), split-BF16x3.
//
// The DFT of real traces at F frequencies is the real GEMM
//     C[r][j] = sum_n x[r][n] B[n][j],   B[n][2q] = cos(2 pi f_q n dt), B[n][2q+1] = -sin(...)
// so C[r][2q], C[r][2q+1] are Re and Im of X[r, f_q] (the interleaved output of
// fdtdpic_dft_probes).  Each operand is split into two BF16 halves, x = xh + xl and
// B = Bh + Bl (xl = bf16(x - xh)), and C ~= xh Bh + xh Bl + xl Bh: three BF16 MMAs per K step,
// about 16 significant bits per product, FP32 sums in tensor memory over TC_FLUSH chunks of
// TC_KC steps, then compensated FP32 sums (a float pair per output, error-free two-sum) in
// shared memory: the group sums' rounding is bounded by one flush group of 1024 steps, and the
// sums across groups keep ~48 bits without the narrow FP64 pipe.
//
// Three launches:
//   dft_tc_pack_traces   traces -> BF16 hi/lo operand tiles, one 32 KiB block per (128 traces,
//                        64 steps), already in the MMA's shared-memory layout (canonical
//                        no-swizzle K-major: 8-row x 16-byte core matrices)
//   dft_tc_pack_twiddles twiddle table -> 16 KiB blocks per (32 frequencies x re/im, 64 steps)
//   dft_tc_kernel        one CTA per 128-trace x 64-column tile: a two-stage pipeline of bulk
//                        asynchronous copies (cp.async.bulk, mbarrier transaction counts) feeding
//                        the tensor cores; one thread issues the 12 MMAs of a chunk and commits
//                        them to an mbarrier; every wait is bounded.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mbar_wait.cuh"
#include "fdtdpic.h"

namespace fdtdpic {

int cuda_status(cudaError_t e);

constexpr int TC_M = 128;          // traces per CTA = MMA M = tensor memory lanes
constexpr int TC_N = 64;           // output columns per CTA (32 frequencies x re/im) = MMA N
constexpr int TC_Q = TC_N / 2;     // frequencies per CTA
constexpr int TC_KC = 64;          // time steps per chunk (one pipeline stage)
constexpr int TC_KSTEP = 16;       // K of one kind::f16 MMA
constexpr int TC_FLUSH = 16;       // chunks summed in FP32 before the compensated sums
constexpr int TC_THREADS = 128;
constexpr int TC_TMEM_COLS = 64;   // FP32 accumulator columns (power of two >= 32)
constexpr uint32_t TC_LBO = 128;                          // next core matrix along K
constexpr uint32_t TC_SBO = (TC_KC / 8) * 128;            // next 8 rows: 1024 B
constexpr uint32_t TC_A_HALF = (TC_M / 8) * TC_SBO;        // 16 KiB
constexpr uint32_t TC_B_HALF = (TC_N / 8) * TC_SBO;        // 8 KiB
constexpr uint32_t TC_A_BLOCK = 2 * TC_A_HALF;             // hi then lo
constexpr uint32_t TC_B_BLOCK = 2 * TC_B_HALF;
constexpr uint32_t TC_STAGE = TC_A_BLOCK + TC_B_BLOCK;     // 48 KiB
constexpr uint32_t TC_ACC_BYTES = TC_M * TC_N * 8;         // float-pair tile, 64 KiB
constexpr uint32_t TC_SMEM = 2 * TC_STAGE + TC_ACC_BYTES + 64;

// Byte offset of element (row, k) of a K-major operand tile in the core-matrix layout.
__host__ __device__ __forceinline__ uint32_t tc_off(int row, int k)
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

// Bulk copy of one operand block into a stage; completes bytes on the stage's mbarrier.
__device__ __forceinline__ void tc_bulk_load(uint32_t dst, const void *src, uint32_t bytes,
                                             uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_expect(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ uint32_t tc_pack2(__nv_bfloat16 a, __nv_bfloat16 b)
{
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// Split 8 consecutive K values into the hi and lo 16-byte rows of a core matrix.
__device__ __forceinline__ void tc_split8(const float *v, uint4 &hi, uint4 &lo)
{
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * i]);
        const __nv_bfloat16 h1 = __float2bfloat16_rn(v[2 * i + 1]);
        const __nv_bfloat16 l0 = __float2bfloat16_rn(v[2 * i] - __bfloat162float(h0));
        const __nv_bfloat16 l1 = __float2bfloat16_rn(v[2 * i + 1] - __bfloat162float(h1));
        h[i] = tc_pack2(h0, h1);
        l[i] = tc_pack2(l0, l1);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// One thread per (row tile, chunk, row, 8-step group); 8 threads cover one trace's 64 steps.
template <typename TIn>
__global__ void dft_tc_pack_traces(const TIn *x, int R, int S, int rp, int64_t ldp, int64_t sp,
                                   int64_t sn, int n_kc, int64_t total, unsigned char *tiles)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int kb = (int)(i & 7);
        const int row = (int)((i >> 3) % TC_M);
        const int64_t blk = (i >> 3) / TC_M;  // rt * n_kc + kc
        const int kc = (int)(blk % n_kc), rt = (int)(blk / n_kc);
        const int r = rt * TC_M + row, n0 = kc * TC_KC + kb * 8;
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = n0 + j;
            v[j] = (r < R && n < S)
                       ? (float)x[(int64_t)(r / rp) * ldp + (int64_t)(r % rp) * sp + (int64_t)n * sn]
                       : 0.f;
        }
        uint4 hi, lo;
        tc_split8(v, hi, lo);
        unsigned char *b = tiles + blk * TC_A_BLOCK + tc_off(row, kb * 8);
        *reinterpret_cast<uint4 *>(b) = hi;
        *reinterpret_cast<uint4 *>(b + TC_A_HALF) = lo;
    }
}

// One thread per (column tile, chunk, frequency, 8-step group): the cos row 2q and the -sin
// row 2q+1 of the block.
__global__ void dft_tc_pack_twiddles(const float2 *tw, int F, int S, int n_kc, int64_t total,
                                     unsigned char *tiles)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int kb = (int)(i & 7);
        const int q = (int)((i >> 3) % TC_Q);
        const int64_t blk = (i >> 3) / TC_Q;  // ct * n_kc + kc
        const int kc = (int)(blk % n_kc), ct = (int)(blk / n_kc);
        const int f = ct * TC_Q + q, n0 = kc * TC_KC + kb * 8;
        float c[8], s[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = n0 + j;
            const float2 w = (f < F && n < S) ? tw[(int64_t)f * S + n] : make_float2(0.f, 0.f);
            c[j] = w.x;
            s[j] = w.y;
        }
        uint4 hi, lo;
        unsigned char *b = tiles + blk * TC_B_BLOCK;
        tc_split8(c, hi, lo);
        *reinterpret_cast<uint4 *>(b + tc_off(2 * q, kb * 8)) = hi;
        *reinterpret_cast<uint4 *>(b + TC_B_HALF + tc_off(2 * q, kb * 8)) = lo;
        tc_split8(s, hi, lo);
        *reinterpret_cast<uint4 *>(b + tc_off(2 * q + 1, kb * 8)) = hi;
        *reinterpret_cast<uint4 *>(b + TC_B_HALF + tc_off(2 * q + 1, kb * 8)) = lo;
    }
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    dft_tc_kernel(const unsigned char *a_tiles, const unsigned char *b_tiles, int n_kc, int R,
                  int F, double *out, int32_t *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    float2 *acc = reinterpret_cast<float2 *>(sm + 2 * TC_STAGE);  // [TC_N][TC_M] (sum, error)
    uint64_t *bars = reinterpret_cast<uint64_t *>(acc + TC_M * TC_N);  // full[0], full[1], mma
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 3);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int ct = blockIdx.x, rt = blockIdx.y;
    const int r0 = rt * TC_M, q0 = ct * TC_Q;
    const unsigned char *a_src = a_tiles + (int64_t)rt * n_kc * TC_A_BLOCK;
    const unsigned char *b_src = b_tiles + (int64_t)ct * n_kc * TC_B_BLOCK;

    for (int i = tid; i < TC_M * TC_N; i += TC_THREADS) acc[i] = make_float2(0.f, 0.f);
    const uint32_t s_base = (uint32_t)__cvta_generic_to_shared(sm);
    const uint32_t full0 = (uint32_t)__cvta_generic_to_shared(bars);
    const uint32_t mma_bar = full0 + 16;
    if (tid == 0) {
        for (int b = 0; b < 3; ++b)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0 + 8 * b));
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
    const uint32_t t_row = tmem + ((uint32_t)(warp * 32) << 16);  // lanes 32w..32w+31

    auto issue_loads = [&](int c) {
        const uint32_t st = s_base + (uint32_t)(c & 1) * TC_STAGE;
        const uint32_t bar = full0 + 8u * (uint32_t)(c & 1);
        tc_expect(bar, TC_STAGE);
        tc_bulk_load(st, a_src + (int64_t)c * TC_A_BLOCK, TC_A_BLOCK, bar);
        tc_bulk_load(st + TC_A_BLOCK, b_src + (int64_t)c * TC_B_BLOCK, TC_B_BLOCK, bar);
    };
    if (tid == 0) issue_loads(0);

    bool ok = true;
    int issued = 1;      // chunks whose loads were issued
    int mma_issued = 0;  // chunks whose MMAs were issued
    for (int c = 0; c < n_kc; ++c) {
        const int s = c & 1;
        if (tid == 0 && c + 1 < n_kc) {  // the other stage was freed by chunk c-1's MMAs
            issue_loads(c + 1);
        }
        if (c + 1 < n_kc) issued = c + 2;
        if (!__syncthreads_and((int)tc_wait(full0 + 8u * s, (uint32_t)((c >> 1) & 1)))) {
            ok = false;
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (tid == 0) {
            const uint32_t a_hi = s_base + (uint32_t)s * TC_STAGE, a_lo = a_hi + TC_A_HALF;
            const uint32_t b_hi = a_hi + TC_A_BLOCK, b_lo = b_hi + TC_B_HALF;
            const bool fresh = (c % TC_FLUSH) == 0;
#pragma unroll
            for (int k = 0; k < TC_KC / TC_KSTEP; ++k) {
                const uint32_t ko = (uint32_t)k * 2 * TC_LBO;  // two core matrices per K step
                tc_mma(tmem, tc_desc(a_hi + ko), tc_desc(b_hi + ko), (fresh && k == 0) ? 0u : 1u);
                tc_mma(tmem, tc_desc(a_hi + ko), tc_desc(b_lo + ko), 1u);
                tc_mma(tmem, tc_desc(a_lo + ko), tc_desc(b_hi + ko), 1u);
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    mma_bar));
        }
        mma_issued = c + 1;
        if (!__syncthreads_and((int)tc_wait(mma_bar, (uint32_t)(c & 1)))) {
            ok = false;
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        if ((c % TC_FLUSH) == TC_FLUSH - 1 || c == n_kc - 1) {
            // this thread's row of the FP32 accumulator -> the compensated sums
#pragma unroll
            for (int c0 = 0; c0 < TC_N; c0 += 16) {
                uint32_t v[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,"
                    "%11,%12,%13,%14,%15}, [%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                      "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                      "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                    : "r"(t_row + (uint32_t)c0));
                asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    float2 &a2 = acc[(c0 + j) * TC_M + tid];
                    const float b = __uint_as_float(v[j]);
                    const float s2 = __fadd_rn(a2.x, b);  // two-sum: s2 + e == a2.x + b exactly
                    const float bp = __fsub_rn(s2, a2.x);
                    const float e = __fadd_rn(__fsub_rn(a2.x, __fsub_rn(s2, bp)), __fsub_rn(b, bp));
                    a2.x = s2;
                    a2.y = __fadd_rn(a2.y, e);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();  // accumulator read before the next chunk's first MMA
        asm volatile("tcgen05.fence::after_thread_sync;");
    }
    if (!ok) {
        // a wait gave up: record it, then wait (bounded) for every copy and MMA this CTA started
        // before its shared and tensor memory are released
        if (tid == 0) {
            atomicOr(err, 1);
            for (int c = issued - 2 < 0 ? 0 : issued - 2; c < issued; ++c)  // latest per stage
                tc_wait(full0 + 8u * (c & 1), (uint32_t)((c >> 1) & 1));
            if (mma_issued > 0) tc_wait(mma_bar, (uint32_t)((mma_issued - 1) & 1));
        }
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
            if (f < F) {
                const float2 a2 = acc[c * TC_M + tid];
                out[((int64_t)r * F + f) * 2 + (c & 1)] = (double)a2.x + (double)a2.y;
            }
        }
}

struct TcLayout {
    int n_rt, n_ct, n_kc;
    int64_t a_bytes, b_bytes, total;
};

inline TcLayout tc_layout(int R, int S, int F)
{
    TcLayout L{};
    L.n_rt = (R + TC_M - 1) / TC_M;
    L.n_ct = (F + TC_Q - 1) / TC_Q;
    L.n_kc = (S + TC_KC - 1) / TC_KC;
    L.a_bytes = (int64_t)L.n_rt * L.n_kc * TC_A_BLOCK;
    L.b_bytes = (int64_t)L.n_ct * L.n_kc * TC_B_BLOCK;
    L.total = L.a_bytes + L.b_bytes;
    return L;
}

}  // namespace fdtdpic

using namespace fdtdpic;

extern "C" {

int64_t fdtdpic_dft_tc_scratch_bytes(int R, int S, int F)
{
    if (R <= 0 || S <= 0 || F <= 0) return 0;
    return tc_layout(R, S, F).total;
}

int fdtdpic_dft_probes_tc(int precision, const void *d_traces, int R, int S, int rp, int64_t ldp,
                          int64_t sp, int64_t sn, const void *d_tw, int F, double *d_out,
                          void *d_scratch, int64_t scratch_bytes, int32_t *d_err,
                          fdtdpic_stream_t stream)
{
    if (!d_traces || !d_tw || !d_out || !d_err || !d_scratch || R < 0 || S <= 0 || F <= 0 ||
        rp < 1 || ldp < 0 || sp < 0 || sn < 1)
        return FDTDPIC_ERR_ARG;
    if (R == 0) return FDTDPIC_OK;
    if (((uintptr_t)d_scratch & 15) != 0) return FDTDPIC_ERR_ARG;  // bulk copies: 16-B aligned
    const TcLayout L = tc_layout(R, S, F);
    if (scratch_bytes < L.total) return FDTDPIC_ERR_OOM;
    int dev = 0, major = 0, minor = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FDTDPIC_ERR_NODEV;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (major != 10 || minor != 3) return FDTDPIC_ERR_NODEV;  // built for sm_103a only
    if (L.n_rt > 65535) return FDTDPIC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *a_tiles = (unsigned char *)d_scratch;
    unsigned char *b_tiles = a_tiles + L.a_bytes;
    const int64_t a_work = (int64_t)L.n_rt * L.n_kc * TC_M * 8;
    const int64_t b_work = (int64_t)L.n_ct * L.n_kc * TC_Q * 8;
    const int pack_blocks = 16 * sms;
    if (precision == FDTDPIC_F32)
        dft_tc_pack_traces<float><<<pack_blocks, 256, 0, st>>>((const float *)d_traces, R, S, rp,
                                                               ldp, sp, sn, L.n_kc, a_work, a_tiles);
    else if (precision == FDTDPIC_F64)
        dft_tc_pack_traces<double><<<pack_blocks, 256, 0, st>>>(
            (const double *)d_traces, R, S, rp, ldp, sp, sn, L.n_kc, a_work, a_tiles);
    else
        return FDTDPIC_ERR_ARG;
    dft_tc_pack_twiddles<<<pack_blocks, 256, 0, st>>>((const float2 *)d_tw, F, S, L.n_kc, b_work,
                                                      b_tiles);
    cudaError_t e = cudaFuncSetAttribute(dft_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)TC_SMEM);
    if (e != cudaSuccess) return cuda_status(e);
    dim3 grid(L.n_ct, L.n_rt);
    dft_tc_kernel<<<grid, TC_THREADS, TC_SMEM, st>>>(a_tiles, b_tiles, L.n_kc, R, F, d_out, d_err);
    return cuda_status(cudaGetLastError());
}

}  // extern "C"
