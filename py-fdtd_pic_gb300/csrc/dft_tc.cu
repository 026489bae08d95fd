// Batched probe DFT on the 5th-generation tensor cores (tcgen05, kind::f16, BF16 operands,
// FP32 accumulation in tensor memory), split-BF16x3.
//
// The DFT of real traces at F frequencies is the real GEMM
//     C[r][j] = sum_n x[r][n] B[n][j],   B[n][2q] = cos(2 pi f_q n dt), B[n][2q+1] = -sin(...)
// so C[r][2q], C[r][2q+1] are Re and Im of X[r, f_q] (the interleaved output of
// fdtdpic_dft_probes).  Each operand is split into two BF16 halves, x = xh + xl and
// B = Bh + Bl (xl = bf16(x - xh)), and C ~= xh Bh + xh Bl + xl Bh: three BF16 MMAs per K step,
// about 16 significant bits per product, FP32 sums in tensor memory over TC_FLUSH chunks of
// TC_KC steps, then compensated FP32 sums (a float pair per output, error-free two-sum), also in
// tensor memory: the group sums' rounding is bounded by one flush group of 1024 steps, and the
// sums across groups keep ~48 bits without the narrow FP64 pipe.
//
// Three launches:
//   dft_tc_pack_traces   traces -> BF16 hi/lo operand tiles, one 32 KiB block per (128 traces,
//                        64 steps), already in the MMA's shared-memory layout (canonical
//                        no-swizzle K-major: 8-row x 16-byte core matrices)
//   dft_tc_pack_twiddles twiddle table -> 32 KiB blocks per (64 frequencies x re/im, 64 steps)
//   dft_tc_kernel        one CTA per 128-trace x 128-column tile, warp-specialised: a producer
//                        thread streams the chunks' operand blocks through a three-stage ring
//                        of bulk asynchronous copies (cp.async.bulk, mbarrier transaction
//                        counts); an MMA thread issues each chunk's 12 MMAs as soon as its
//                        stage is full and frees the stage with a commit, never waiting for
//                        the MMAs themselves; the flush groups alternate between two tensor-
//                        memory accumulators, so four epilogue warps fold one group into the
//                        compensated sums while the tensor cores fill the other.  Every wait
//                        is bounded.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mbar_wait.cuh"
#include "fdtdpic.h"

namespace fdtdpic {

int cuda_status(cudaError_t e);

constexpr int TC_M = 128;          // traces per CTA = MMA M = tensor memory lanes
constexpr int TC_N = 128;          // output columns per CTA (64 frequencies x re/im) = MMA N
constexpr int TC_Q = TC_N / 2;     // frequencies per CTA
constexpr int TC_KC = 64;          // time steps per chunk (one pipeline stage)
constexpr int TC_KSTEP = 16;       // K of one kind::f16 MMA
constexpr int TC_FLUSH = 16;       // chunks summed in FP32 before the compensated sums
constexpr int TC_STAGES = 3;
constexpr int TC_EPI_WARPS = 4;    // epilogue warps: warp w reads tensor memory lanes 32w ..
constexpr int TC_THREADS = 32 * (TC_EPI_WARPS + 2);  // + the producer warp and the MMA warp
constexpr int TC_TMEM_COLS = 512;  // accumulators [0, 2N), sums [2N, 3N), errors [3N, 4N)
constexpr uint32_t TC_LBO = 128;                          // next core matrix along K
constexpr uint32_t TC_SBO = (TC_KC / 8) * 128;            // next 8 rows: 1024 B
constexpr uint32_t TC_A_HALF = (TC_M / 8) * TC_SBO;        // 16 KiB
constexpr uint32_t TC_B_HALF = (TC_N / 8) * TC_SBO;        // 16 KiB
constexpr uint32_t TC_A_BLOCK = 2 * TC_A_HALF;             // hi then lo
constexpr uint32_t TC_B_BLOCK = 2 * TC_B_HALF;
constexpr uint32_t TC_STAGE = TC_A_BLOCK + TC_B_BLOCK;     // 64 KiB
constexpr int TC_BARS = 2 * TC_STAGES + 4;                 // full, empty, accfull, accempty
constexpr uint32_t TC_SMEM = TC_STAGES * TC_STAGE + 8 * TC_BARS + 16;

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

__device__ __forceinline__ void tc_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
        bar));
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&v)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
          "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tc_st16(uint32_t taddr, const uint32_t (&v)[16])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
        "%13,%14,%15,%16};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
        "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]),
        "r"(v[15])
        : "memory");
}

// Barriers (mbarrier phases): full[s] completes when stage s's copies land (the j-th time:
// chunk s + 3j), empty[s] when the MMAs reading it complete (chunk s + 3j), accfull[b] when the
// MMAs of flush group b + 2j complete, accempty[b] when the epilogue has read group b + 2j.
__global__ void __launch_bounds__(TC_THREADS, 1)
    dft_tc_kernel(const unsigned char *a_tiles, const unsigned char *b_tiles, int n_kc, int R,
                  int F, double *out, int32_t *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + TC_STAGES * TC_STAGE);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + TC_BARS);
    __shared__ int s_abort, s_loads, s_mmas;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ct = blockIdx.x, rt = blockIdx.y;
    const int r0 = rt * TC_M, q0 = ct * TC_Q;
    const unsigned char *a_src = a_tiles + (int64_t)rt * n_kc * TC_A_BLOCK;
    const unsigned char *b_src = b_tiles + (int64_t)ct * n_kc * TC_B_BLOCK;
    const uint32_t s_base = (uint32_t)__cvta_generic_to_shared(sm);
    const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(bars);
    auto full_bar = [&](int st) { return bar0 + 8u * (uint32_t)st; };
    auto empty_bar = [&](int st) { return bar0 + 8u * (uint32_t)(TC_STAGES + st); };
    auto accfull_bar = [&](int b) { return bar0 + 8u * (uint32_t)(2 * TC_STAGES + b); };
    auto accempty_bar = [&](int b) { return bar0 + 8u * (uint32_t)(2 * TC_STAGES + 2 + b); };
    if (tid == 0) {
        for (int i = 0; i < 2 * TC_STAGES + 2; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8u * (uint32_t)i));
        for (int b = 0; b < 2; ++b)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(accempty_bar(b)),
                         "r"(32 * TC_EPI_WARPS));
        asm volatile("fence.mbarrier_init.release.cluster;");
        s_abort = 0;
        s_loads = 0;
        s_mmas = 0;
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
    const int n_groups = (n_kc + TC_FLUSH - 1) / TC_FLUSH;

    if (warp == TC_EPI_WARPS) {
        // producer: chunk c into stage c % 3 once the MMAs of chunk c - 3 have freed it
        if (lane == 0) {
            for (int c = 0; c < n_kc; ++c) {
                const int st = c % TC_STAGES, k = c / TC_STAGES;
                if (k > 0 && !tc_wait(empty_bar(st), (uint32_t)((k - 1) & 1))) {
                    atomicOr(&s_abort, 1);
                    break;
                }
                if (*(volatile int *)&s_abort) break;
                const uint32_t dst = s_base + (uint32_t)st * TC_STAGE;
                tc_expect(full_bar(st), TC_STAGE);
                tc_bulk_load(dst, a_src + (int64_t)c * TC_A_BLOCK, TC_A_BLOCK, full_bar(st));
                tc_bulk_load(dst + TC_A_BLOCK, b_src + (int64_t)c * TC_B_BLOCK, TC_B_BLOCK,
                             full_bar(st));
                s_loads = c + 1;
            }
        }
    } else if (warp == TC_EPI_WARPS + 1) {
        // MMA issuer: chunk c's 12 MMAs into accumulator (c / TC_FLUSH) % 2 as soon as its stage
        // is full; a commit frees the stage, another after a group's last chunk hands the
        // accumulator to the epilogue
        if (lane == 0) {
            for (int c = 0; c < n_kc; ++c) {
                const int st = c % TC_STAGES, k = c / TC_STAGES;
                const int g = c / TC_FLUSH, b = g & 1;
                const bool first = (c % TC_FLUSH) == 0;
                const bool last = (c % TC_FLUSH) == TC_FLUSH - 1 || c == n_kc - 1;
                if (first && g >= 2 &&
                    !tc_wait(accempty_bar(b), (uint32_t)(((g >> 1) - 1) & 1))) {
                    atomicOr(&s_abort, 1);
                    break;
                }
                if (!tc_wait(full_bar(st), (uint32_t)(k & 1))) {
                    atomicOr(&s_abort, 1);
                    break;
                }
                if (*(volatile int *)&s_abort) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t a_hi = s_base + (uint32_t)st * TC_STAGE, a_lo = a_hi + TC_A_HALF;
                const uint32_t b_hi = a_hi + TC_A_BLOCK, b_lo = b_hi + TC_B_HALF;
                const uint32_t d = tmem + (uint32_t)(b * TC_N);
#pragma unroll
                for (int kk = 0; kk < TC_KC / TC_KSTEP; ++kk) {
                    const uint32_t ko = (uint32_t)kk * 2 * TC_LBO;  // two core matrices per K step
                    tc_mma(d, tc_desc(a_hi + ko), tc_desc(b_hi + ko), (first && kk == 0) ? 0u : 1u);
                    tc_mma(d, tc_desc(a_hi + ko), tc_desc(b_lo + ko), 1u);
                    tc_mma(d, tc_desc(a_lo + ko), tc_desc(b_hi + ko), 1u);
                }
                tc_commit(empty_bar(st));
                if (last) tc_commit(accfull_bar(b));
                s_mmas = c + 1;
            }
        }
    } else {
        // epilogue: each thread one trace (tensor memory lane 32 warp + lane); per group, the
        // FP32 accumulator folded into the (sum, error) pairs by an error-free two-sum; the last
        // group's pairs go out as sum + error in FP64
        const uint32_t t_lane = tmem + ((uint32_t)(warp * 32) << 16);
        const int r = r0 + warp * 32 + lane;
        for (int g = 0; g < n_groups; ++g) {
            const int b = g & 1;
            if (!tc_wait(accfull_bar(b), (uint32_t)((g >> 1) & 1))) {
                atomicOr(&s_abort, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const bool fin = g == n_groups - 1;
#pragma unroll 1
            for (int c0 = 0; c0 < TC_N; c0 += 16) {
                uint32_t v[16], su[16], er[16];
                tc_ld16(t_lane + (uint32_t)(b * TC_N + c0), v);
                if (g > 0) {
                    tc_ld16(t_lane + (uint32_t)(2 * TC_N + c0), su);
                    tc_ld16(t_lane + (uint32_t)(3 * TC_N + c0), er);
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const float x = __uint_as_float(v[j]);
                    float sum = x, e = 0.f;
                    if (g > 0) {
                        const float a0 = __uint_as_float(su[j]);
                        sum = __fadd_rn(a0, x);  // two-sum: sum + t == a0 + x exactly
                        const float bp = __fsub_rn(sum, a0);
                        const float t = __fadd_rn(__fsub_rn(a0, __fsub_rn(sum, bp)),
                                                  __fsub_rn(x, bp));
                        e = __fadd_rn(__uint_as_float(er[j]), t);
                    }
                    su[j] = __float_as_uint(sum);
                    er[j] = __float_as_uint(e);
                }
                if (fin) {
                    if (r < R)
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const int col = c0 + j, f = q0 + (col >> 1);
                            if (f < F)
                                out[((int64_t)r * F + f) * 2 + (col & 1)] =
                                    (double)__uint_as_float(su[j]) + (double)__uint_as_float(er[j]);
                        }
                } else {
                    tc_st16(t_lane + (uint32_t)(2 * TC_N + c0), su);
                    tc_st16(t_lane + (uint32_t)(3 * TC_N + c0), er);
                }
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;");
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(accempty_bar(b))
                         : "memory");
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (s_abort && tid == 0) {
        // a wait gave up: record it, then wait (bounded) for the copies and MMAs this CTA
        // started before its shared and tensor memory are released
        atomicOr(err, 1);
        for (int c = s_loads - TC_STAGES < 0 ? 0 : s_loads - TC_STAGES; c < s_loads; ++c)
            tc_wait(full_bar(c % TC_STAGES), (uint32_t)((c / TC_STAGES) & 1));
        for (int c = s_mmas - TC_STAGES < 0 ? 0 : s_mmas - TC_STAGES; c < s_mmas; ++c)
            tc_wait(empty_bar(c % TC_STAGES), (uint32_t)((c / TC_STAGES) & 1));
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TC_TMEM_COLS));
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
