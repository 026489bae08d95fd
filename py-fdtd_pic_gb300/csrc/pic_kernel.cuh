// Electron-beam PIC coupled to the 1D FDTD grid, templated on the state type T.
//
// Per step t (fields: E^t, H^(t+1/2) in Hy, H^(t-1/2) in Hyp):
//   pic_push_kernel : gather, relativistic Boris push, move, deposit Jx^(t+1/2) and Jz into
//                     int64 fixed-point accumulators (exact integer sums: bit-identical results
//                     for any particle order or thread schedule; no float atomics)
//   pic_e_kernel    : Hyp <- Hy; Jx, Jz <- accumulators (then zeroed); E phase with -Jx
//   pic_h_kernel    : H phase, probes, snapshots
// and every sort_every steps a counting re-bin of the particles by cell (histogram, scan,
// scatter), which keeps each CTA's particles within a few cells so its deposits land in a small
// shared-memory window (exact 64-bit adds from pairs of 32-bit shared atomics).
#pragma once
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>


#include "bounds.cuh"
#include "fdtd1d_kernel.cuh"

namespace fdtdpic {

int cuda_status(cudaError_t e);

// Programmatic dependent launch: the push and field kernels of consecutive steps are launched
// with programmatic stream serialization, each lets the next one launch as soon as all its own
// CTAs run (pdl_trigger), and each waits for its predecessor's completion and memory (pdl_wait)
// only after the set-up that does not read it (shared-memory copies of the constants, clearing
// the deposit window).  Steps then pay no launch gap and overlap those prologues.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), int grid, int block, cudaStream_t st,
                              Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

constexpr int PIC_WIN = 256;      // shared-memory deposit window (nodes) per CTA
constexpr int PIC_THREADS = 256;  // push kernel CTA size
constexpr int FIELD_UH_FUSED = 2; // H cells per thread in the push launch's H CTAs (fewer
                                  // registers than pic_h_kernel's, which the push CTAs share)

// Fixed-point words per current component: FP32 keeps one int64 word (scale 2^S),
// FP64 two (the remainder below 2^-S kept at a further 2^40).
template <typename T>
struct Fix;
template <>
struct Fix<float> {
    static constexpr int W = 1;
    // x = v * 2^S rounded to an integer using 32-bit conversions only (the 64-bit ones run on
    // the narrow FP64 pipe).  |x| < 2^31: one conversion.  Otherwise x is a multiple of 2^8 or
    // more, so x - floor(x / 2^32) * 2^32 is exact in float and fits an unsigned 32-bit integer.
    __device__ static void split(float v, double, float scale_f, long long *w)
    {
        const float x = v * scale_f;
        if (fabsf(x) < 2147483648.f) {
            w[0] = (long long)__float2int_rn(x);
        } else {
            const float h = floorf(x * 2.3283064365386963e-10f);  // 2^-32
            const float r = fmaf(-h, 4294967296.f, x);               // exact
            w[0] = (long long)((unsigned long long)(long long)__float2int_rn(h) << 32) +
                   (long long)__float2uint_rn(r);
        }
    }
    __device__ static float to_float(unsigned long long u, float inv_f)
    {
        const long long v = (long long)u;
        const int hi = (int)(v >> 32);
        const unsigned lo = (unsigned)(v & 0xffffffffull);
        return fmaf((float)hi, 4294967296.f, (float)lo) * inv_f;
    }
    __device__ static float join(const unsigned long long *w, double, float inv_f)
    {
        return to_float(w[0], inv_f);
    }
    // words at base[w*stride + l]
    __device__ static float join2(const unsigned long long *base, size_t, int l, double,
                                  float inv_f)
    {
        return to_float(base[l], inv_f);
    }
};
template <>
struct Fix<double> {
    static constexpr int W = 2;
    __device__ static void split(double v, double scale, float, long long *w)
    {
        const double x = v * scale;
        const double hi = floor(x);
        w[0] = (long long)hi;
        w[1] = __double2ll_rn((x - hi) * 1099511627776.0);  // 2^40
    }
    __device__ static double join(const unsigned long long *w, double inv, float)
    {
        return (double)(long long)w[0] * inv + (double)(long long)w[1] * (inv * (1.0 / 1099511627776.0));
    }
    __device__ static double join2(const unsigned long long *base, size_t stride, int l, double inv,
                                   float)
    {
        return (double)(long long)base[l] * inv +
               (double)(long long)base[stride + l] * (inv * (1.0 / 1099511627776.0));
    }
};

template <typename T>
struct PicArgs {
    int n_part, nz, clo, chi, chunk;
    T kE, kH, sc, kJ, kJz;
    double jscale, jinv;
    float jscale_f, jinv_f;
    int32_t *cell;
    T *frac, *ux, *uz;
    const T *ex, *hy, *hyp;
    unsigned long long *acc;  // [2*W][nz+1]: Jx words then Jz words
    int32_t *status;
    int deposit_jz;  // Jz (a diagnostic: no field uses it) only on the call's last step
    int hblocks;     // launches that carry an H phase: its CTAs, ahead of the push CTAs
};

// One particle's step (everything but the wrap), shared by the streaming and tiled kernels.
// FP64 keeps the oracle's operation order (divisions by gamma); FP32 uses rsqrt/fast-divide.
template <typename T>
struct Moved {
    int c1;       // new cell before the periodic wrap
    T f1, ux, uz; // new fraction and momenta
    int nx0;      // Jx nodes nx0, nx0+1 (CIC at the half-step midpoint)
    T jx0, jx1;
};

// Jz of one particle's move (only the call's last step deposits it): half nodes nzA, nzB (nzB < 0
// when the particle stays in its cell) and their values, from the start (c, f) and the move.
template <typename T>
struct MovedJz {
    int nzA, nzB;
    T jzA, jzB;
};
template <typename T>
__device__ __forceinline__ MovedJz<T> particle_jz(int c, T f, const Moved<T> &m, T kJz)
{
    MovedJz<T> z;
    const int c1 = m.c1;
    const T f1 = m.f1;
    if (c1 == c) {
        z.nzA = c; z.jzA = kJz * (f1 - f);
        z.nzB = -1; z.jzB = T(0);
    } else if (c1 == c + 1) {
        z.nzA = c; z.jzA = kJz * (T(1) - f);
        z.nzB = c + 1; z.jzB = kJz * f1;
    } else {
        z.nzA = c - 1; z.jzA = -kJz * (T(1) - f1);
        z.nzB = c; z.jzB = -kJz * f;
    }
    return z;
}

// 1/sqrt(x) for x >= 1 (here 1 + u^2): the hardware approximation with subnormal handling
// dropped, which for normal inputs and results is the value rsqrtf returns
__device__ __forceinline__ float rsqrt_ge1(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

template <typename T>
__device__ __forceinline__ void particle_step(T E, T H, int c, T f, T ux, T uz, T kE, T kH, T sc,
                                              T kJ, Moved<T> &m)
{
    const T uxm = (sizeof(T) == 8) ? ux + kE * E : (T)fmaf((float)kE, (float)E, (float)ux);
    const T uzm = uz;
    T uxn, uzn, dz, jxv;
    if constexpr (sizeof(T) == 8) {
        const T gm = sqrt(T(1) + uxm * uxm + uzm * uzm);
        const T ty = kH * H / gm;
        const T sy = T(2) * ty / (T(1) + ty * ty);
        const T uxp = uxm - uzm * ty;
        const T uzp = uzm + uxm * ty;
        uxn = (uxm - uzp * sy) + kE * E;
        uzn = uzm + uxp * sy;
        const T g = sqrt(T(1) + uxn * uxn + uzn * uzn);
        dz = sc * uzn / g;
        jxv = kJ * uxn / g;
    } else {
        // fused operations written out (fmaf), so the rounding does not depend on how the
        // compiler contracts this code in each kernel that inlines it (the unit is built
        // with -fmad=false)
        const float gmi = rsqrt_ge1(fmaf(uzm, uzm, fmaf(uxm, uxm, 1.f)));
        const float ty = kH * H * gmi;
        const float sy = __fdividef(2.f * ty, fmaf(ty, ty, 1.f));
        const float uxp = fmaf(-uzm, ty, uxm);
        const float uzp = fmaf(uxm, ty, uzm);
        uxn = fmaf(kE, E, fmaf(-uzp, sy, uxm));
        uzn = fmaf(uxp, sy, uzm);
        const float gi = rsqrt_ge1(fmaf(uzn, uzn, fmaf(uxn, uxn, 1.f)));
        dz = sc * uzn * gi;
        jxv = kJ * uxn * gi;
    }
    T fm = f + T(0.5) * dz;
    int cm = c;
    if (fm >= T(1)) { cm += 1; fm -= T(1); } else if (fm < T(0)) { cm -= 1; fm += T(1); }
    m.nx0 = cm;
    m.jx0 = jxv * (T(1) - fm);
    m.jx1 = jxv * fm;
    T f1 = f + dz;
    int c1 = c;
    if (f1 >= T(1)) { c1 += 1; f1 -= T(1); } else if (f1 < T(0)) { c1 -= 1; f1 += T(1); }
    m.c1 = c1;
    m.f1 = f1;
    m.ux = uxn;
    m.uz = uzn;
}

// Exact 64-bit add into shared memory from two native 32-bit atomics (little-endian halves):
// the low half's returned old value gives this addition's carry, so the pair always holds the
// exact 64-bit sum; the high half is skipped when it gains nothing.
__device__ __forceinline__ void smem_add_u64(unsigned long long *p, unsigned long long v)
{
    unsigned *w = reinterpret_cast<unsigned *>(p);
    const unsigned lo = (unsigned)v, hi = (unsigned)(v >> 32);
    const unsigned old = atomicAdd(w, lo);
    const unsigned hadd = hi + ((old + lo < old) ? 1u : 0u);
    if (hadd) atomicAdd(w + 1, hadd);
}

// Sum a uint64 over the 32 lanes of a full warp exactly (wrap-around two's complement): three
// pieces of at most 22 bits through the warp reduction unit, so no piece's sum overflows 32 bits.
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
    const unsigned c0 = (unsigned)(v & 0x3FFFFFull);
    const unsigned c1 = (unsigned)((v >> 22) & 0x3FFFFFull);
    const unsigned c2 = (unsigned)(v >> 44);
    const unsigned long long s0 = __reduce_add_sync(0xffffffffu, c0);
    const unsigned long long s1 = __reduce_add_sync(0xffffffffu, c1);
    const unsigned long long s2 = __reduce_add_sync(0xffffffffu, c2);
    return s0 + (s1 << 22) + (s2 << 44);
}

// Exact sum of an int32 over the 32 lanes of a full warp: the 16-bit halves through the
// reduction unit (each sum fits 32 bits), joined in 64 bits.
__device__ __forceinline__ unsigned long long warp_sum_i32(int v)
{
    const int hi = __reduce_add_sync(0xffffffffu, v >> 16);
    const unsigned lo = __reduce_add_sync(0xffffffffu, (unsigned)(v & 0xffff));
    return (unsigned long long)((long long)hi * 65536 + (long long)lo);
}

// Add each lane's word to arr[idx] (idx < 0: nothing), all 32 lanes calling.  The particles
// are in cell order, so a warp's nodes form a few runs of equal values (a dense beam: one or two):
// with at most three runs the warp sums the words of each distinct node and one lane adds the
// sum; otherwise every lane adds its own word (shared atomics that rarely collide at low
// density).  Integer sums: the result does not depend on which way a warp takes.
__device__ __forceinline__ void warp_add_u64(unsigned long long *arr, int idx, unsigned long long v)
{
    const int lane = threadIdx.x & 31;
    const int i0 = __shfl_sync(0xffffffffu, idx, 0);
    if (__all_sync(0xffffffffu, idx == i0)) {  // one node for the whole warp
        if (i0 < 0) return;
        const unsigned long long sum = warp_sum_u64(v);
        if (lane == 0 && sum != 0ull) smem_add_u64(arr + i0, sum);
        return;
    }
    const int prev = __shfl_up_sync(0xffffffffu, idx, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || idx != prev);
    if (__popc(heads) <= 3) {
        unsigned todo = __ballot_sync(0xffffffffu, idx >= 0);
        while (todo) {
            const int src = __ffs(todo) - 1;
            const int node = __shfl_sync(0xffffffffu, idx, src);
            const bool mine = idx == node;
            const unsigned long long sum = warp_sum_u64(mine ? v : 0ull);
            if (lane == src && sum != 0ull) smem_add_u64(arr + node, sum);
            todo &= ~__ballot_sync(0xffffffffu, mine);
        }
    } else if (idx >= 0 && v != 0ull) {
        smem_add_u64(arr + idx, v);
    }
}

// One deposit slot for the whole warp (every lane calls it; invalid lanes pass node = -1):
// nodes inside the CTA's shared window go through warp_add_u64, the rest straight into the
// global accumulators.
template <int W>
__device__ __forceinline__ void deposit_slot(unsigned long long *win, unsigned long long *acc,
                                             int nz1, int base, int word0, int node,
                                             const long long *val, int32_t *bounds = nullptr)
{
    const int rel = node - base;
    const bool in_win = node >= 0 && rel >= 0 && rel < PIC_WIN;
    const bool out = node >= 0 && !in_win && FDTD_IN(node, nz1, bounds);
#pragma unroll
    for (int w = 0; w < W; ++w) {
        warp_add_u64(win + (size_t)(word0 + w) * PIC_WIN, in_win ? rel : -1,
                     (unsigned long long)val[w]);
        if (out && val[w] != 0) atomicAdd(acc + (size_t)(word0 + w) * nz1 + node,
                                          (unsigned long long)val[w]);
    }
}

// The instance's update constants in the state type and its folded FP32 Kerr constants,
// computed once per call by pic_consts_kernel (the FP64 pipe is narrow; the field kernels then
// do no FP64 set-up of their own).
template <typename T>
struct FieldConsts {
    Scal<T> c;
    Kerr<T> kr;
};

template <typename T>
__global__ void pic_consts_kernel(const FdtdInstance *inst, FieldConsts<T> *out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        out->c = make_scal<T>(*inst);
        out->kr.setup(*inst);
    }
}

// Copy the call's constants into shared memory once per CTA (every thread calls it).
template <typename T>
__device__ inline void consts_block(const FieldConsts<T> *g, Scal<T> &c, Kerr<T> &kr)
{
    static_assert(sizeof(FieldConsts<T>) % 4 == 0, "FieldConsts is copied as 32-bit words");
    __shared__ FieldConsts<T> s_fc;
    __syncthreads();
    const int *src = reinterpret_cast<const int *>(g);
    int *dst = reinterpret_cast<int *>(&s_fc);
    for (int i = threadIdx.x; i < (int)(sizeof(FieldConsts<T>) / 4); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    c = s_fc.c;
    kr = s_fc.kr;
}

template <typename T>
struct PicField {
    BatchArgs<T> f;
    const FieldConsts<T> *fc;
    unsigned long long *acc;
    T *jx, *jz, *hyp;
    double jinv;
    float jinv_f;
    const int32_t *step;  // graph replay: first step of the replayed block (the launch argument
                          // is the offset within it); NULL: the launch argument is the step
    int last;             // the call's last step: Jz was deposited, Jz and Acubic are written out
};

template <typename T>
__device__ __forceinline__ int pic_step_index(const PicField<T> &a, int t)
{
    return a.step ? *a.step + t : t;
}

// E phase of cell k with the beam: Hyp <- Hy (H^(t+1/2) for the next push), currents out of the
// accumulators (which are zeroed for the next push), then the reference E phase with -Jx.
// Loads first (the accumulator words, then e_cell's field reads), stores after: the cell's
// loads then go out together instead of each waiting behind an earlier store.  Jz words are
// only non-zero on the call's last step (the only step that deposits them), so they are read,
// cleared and written out then, with the Acubic diagnostic; every other step skips them.
template <typename T, class S>
__device__ __forceinline__ void pic_e_cell(PicField<T> &a, const FdtdInstance &I, S &s,
                                           const Scal<T> &c, const Kerr<T> &kr, int k, int n,
                                           T src_e, T src_h, T *gA, int *nfb)
{
    constexpr int W = Fix<T>::W;
    unsigned long long wx[W], wz[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
        wx[w] = a.acc[(size_t)w * n + k];
        wz[w] = a.last ? a.acc[(size_t)(W + w) * n + k] : 0ull;
    }
    const T hyk = s.HyR(k);
    const T jxk = Fix<T>::join(wx, a.jinv, a.jinv_f);
    if (k >= 1) e_cell<T>(I, c, kr, s, k, src_e, src_h, true, jxk, a.last ? gA : nullptr, nfb, true);
    a.hyp[k] = hyk;
#pragma unroll
    for (int w = 0; w < W; ++w) a.acc[(size_t)w * n + k] = 0ull;
    a.jx[k] = jxk;
    if (a.last) {
#pragma unroll
        for (int w = 0; w < W; ++w) a.acc[(size_t)(W + w) * n + k] = 0ull;
        a.jz[k] = Fix<T>::join(wz, a.jinv, a.jinv_f);
    }
}

template <typename T, class S>
__device__ __forceinline__ void pic_probes(const PicField<T> &a, const FdtdInstance &I, S &s,
                                           int t, int gt, int gstride, int n)
{
    if (gt < 2 && t >= I.probe_lo[gt] && t <= I.probe_hi[gt])
        a.f.probe[I.probe_offset + (int64_t)t * 2 + gt] = s.Ex(I.probe_cell[gt]);
    if (a.f.hist && I.hist_interval > 0 && t > 0 && (t % I.hist_interval) == 0) {
        const int row = t / I.hist_interval;
        if (row < I.hist_rows)
            for (int k = gt; k < n; k += gstride)
                a.f.hist[I.hist_offset + (int64_t)row * n + k] = s.Ex(k);
    }
}

template <typename T>
__global__ void __launch_bounds__(256, 4) pic_e_kernel(PicField<T> a, int t_arg)
{
    constexpr int W = Fix<T>::W;
    pdl_trigger();
    const FdtdInstance &I = instance_block(a.f.inst[0]);
    GlobalStore<T, true> s = global_store<T, true>(I, a.f);
    Scal<T> c;
    Kerr<T> kr;
    consts_block<T>(a.fc, c, kr);
    // the step counter is only written between graph blocks, by launches that completed before
    // this block's first kernel started; the source pool is constant
    const int t = pic_step_index(a, t_arg);
    T src_e, src_h;
    source_block<T>(I, a.f.src, t, src_e, src_h);
    pdl_wait();  // the push's deposits
    const int n = I.nz + 1;
    T *gA = a.f.state + I.state_offset + (int64_t)FDTD_ST_A * n;
    const int stride = gridDim.x * blockDim.x;
    int nfb = 0;
    // FIELD_UE cells per thread per pass, their loads (accumulator words, Hy, Ex, Dx) issued before
    // any of them is updated; then per cell: Hyp <- Hy, accumulators cleared, the E phase with -Jx
    const bool dxm = I.mode != FDTD_MODE_FREESPACE;
    for (int k0 = blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += FIELD_UE * stride) {
        unsigned long long wx[FIELD_UE][W];
        T ex[FIELD_UE], hk[FIELD_UE], hkm[FIELD_UE], dx[FIELD_UE];
#pragma unroll
        for (int u = 0; u < FIELD_UE; ++u) {
            const int k = k0 + u * stride;
            const bool in = k < n;
#pragma unroll
            for (int w = 0; w < W; ++w) wx[u][w] = in ? a.acc[(size_t)w * n + k] : 0ull;
            hk[u] = in ? __ldg(s.hy + k) : T(0);
            hkm[u] = (in && k >= 1) ? __ldg(s.hy + k - 1) : T(0);
            ex[u] = in ? s.ex[k] : T(0);
            dx[u] = (in && dxm && k >= I.front && k < I.rear) ? s.dx[k] : T(0);
        }
#pragma unroll
        for (int u = 0; u < FIELD_UE; ++u) {
            const int k = k0 + u * stride;
            if (k >= n) break;
            const T jxk = Fix<T>::join(wx[u], a.jinv, a.jinv_f);
            const int kd = k >= 1 ? cell_kind(I, k) : CELL_GENERIC;
            if (kd == CELL_VACUUM) {
                // e_cell: ex + mul_c((hk - hkm) - jx, ue) * den, den = 1
                s.ex[k] = ex[u] + mul_c((hk[u] - hkm[u]) - jxk, c.ue, c.ue_lo);
            } else if (kd == CELL_KERR) {
                // e_cell's slab branch: Dx + mul_c((hk - hkm) - jx, dtdz) * den, the Kerr root, Ex
                const T d = dx[u] + mul_c((hk[u] - hkm[u]) - jxk, c.dtdz, c.dtdz_lo);
                const T A = kr.root(d, c.eps0, &nfb);
                if (a.last) gA[k] = A;
                s.dx[k] = d;
                s.ex[k] = div_c(d, c.e0r + c.e0chi * A, c.e0r_rel);
            } else if (k >= 1) {
                // PML, source and Lorentz cells: the whole e_cell on a register copy (their
                // polarisation and psi loaded here)
                const CellUse cu = cell_use(I, k);
                RegE<T> r{ex[u], hk[u], hkm[u], dx[u], cu.p ? s.p[k] : T(0),
                          cu.p ? s.pp[k] : T(0), cu.psie ? s.psie[k] : T(0), s.tab, k, s.W};
                e_cell<T>(I, c, kr, r, k, src_e, src_h, true, jxk, a.last ? gA : nullptr, &nfb,
                          true);
                e_cell_store<T>(I, s, k, r);
            }
            a.hyp[k] = hk[u];
#pragma unroll
            for (int w = 0; w < W; ++w) a.acc[(size_t)w * n + k] = 0ull;
            if (a.last) {  // Jz words are only deposited on the call's last step
                unsigned long long wz[W];
#pragma unroll
                for (int w = 0; w < W; ++w) {
                    wz[w] = a.acc[(size_t)(W + w) * n + k];
                    a.acc[(size_t)(W + w) * n + k] = 0ull;
                }
                a.jx[k] = jxk;
                a.jz[k] = Fix<T>::join(wz, a.jinv, a.jinv_f);
            }
        }
    }
    if (nfb && a.f.fallbacks) atomicAdd(a.f.fallbacks, nfb);
}

// The H phase over CTAs hb of nhb (every thread of the CTA calls it): pic_h_kernel's body, and
// the H part of the push launch that carries the previous step's H phase.  U cells per thread
// are loaded before any is updated.
template <typename T, int U>
__device__ __forceinline__ void pic_h_body(const PicField<T> &a, int t_arg, int hb, int nhb)
{
    const FdtdInstance &I = instance_block(a.f.inst[0]);
    GlobalStore<T, true> s = global_store<T, true>(I, a.f);
    Scal<T> c;
    Kerr<T> kr;
    consts_block<T>(a.fc, c, kr);
    const int t = pic_step_index(a, t_arg);
    const T src_h = src_h_at<T>(I, a.f.src, t);
    pdl_wait();  // the E phase
    const int n = I.nz + 1;
    const int gt = hb * blockDim.x + threadIdx.x;
    const int stride = nhb * blockDim.x;
    for (int k0 = 1 + gt; k0 < n - 1; k0 += U * stride) {
        T hy[U], e0[U], e1[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + u * stride;
            const bool in = k < n - 1;
            hy[u] = in ? s.hy[k] : T(0);
            e0[u] = in ? __ldg(s.ex + k) : T(0);
            e1[u] = in ? __ldg(s.ex + k + 1) : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + u * stride;
            if (k >= n - 1) break;
            if (cell_kind(I, k) != CELL_GENERIC) {
                // h_cell: hy + mul_c(ex[k+1] - ex[k], uh) * den with den = 1 (interior cells are
                // outside the slab or in a Kerr slab, so uh is the outside value)
                s.hy[k] = hy[u] + mul_c(e1[u] - e0[u], c.uh, c.uh_lo);
            } else {
                RegH<T> r{hy[u], e0[u], e1[u], cell_use(I, k).psih ? s.psih[k] : T(0), s.tab,
                          k, s.W};
                h_cell<T>(I, c, r, k, src_h);
                h_cell_store<T>(I, s, k, r);
            }
        }
    }
    if (gt == 0) tfsf_edge<T>(I, s, src_h);
    pic_probes<T>(a, I, s, t, gt, stride, n);
}

template <typename T>
__global__ void __launch_bounds__(256, 4) pic_h_kernel(PicField<T> a, int t_arg)
{
    pdl_trigger();
    pic_h_body<T, FIELD_U>(a, t_arg, blockIdx.x, gridDim.x);
}

// H^(t+1/2) of node k as the H phase computes it (h_cell), from H^(t-1/2) (hyp, which the E
// phase wrote) and E^t, for nodes outside the PML columns: den = 1 and no psi term, so only the
// TF/SF correction and the free-space slab's coefficient remain.
template <typename T>
struct HOnTheFly {
    T src_h, uh, uh_slab, uh_lo, uh_slab_lo;
    int tfsf_cell, slab_lo, slab_hi;
    int plain;  // no TF/SF cell and no slab coefficient: hy + mul_c(e1 - e0, uh) for every node
};
template <typename T>
__device__ __forceinline__ T h_on_the_fly(const HOnTheFly<T> &q, int k, T hy, T e0, T e1)
{
    if (k == q.tfsf_cell) hy = hy - q.src_h;
    const bool in = k >= q.slab_lo && k < q.slab_hi;
    return hy + mul_c(e1 - e0, in ? q.uh_slab : q.uh, in ? q.uh_slab_lo : q.uh_lo);
}

// One particle slot's Jx deposit for the whole warp (every lane calls it; a lane without a
// particle passes nx0 = -1 and zero values): nodes nx0 and nx0 + 1.  A warp whose values are
// all zero (particles no field has given transverse momentum) skips it: adding zeros changes
// nothing.
template <typename T>
__device__ __forceinline__ void push_deposit_jx(unsigned long long *win, const PicArgs<T> &a,
                                                int nz1, int base, int lane, int nx0, T jx0,
                                                T jx1)
{
    constexpr int W = Fix<T>::W;
    if (!__any_sync(0xffffffffu, jx0 != T(0) || jx1 != T(0))) return;
    const int nx1 = nx0 >= 0 ? nx0 + 1 : -1;
    if constexpr (sizeof(T) == 4) {
        // A re-binned dense beam: the warp's particles sit in one or two cells, so their left
        // nodes nx0 span m .. m + D with D <= 2 and the warp touches nodes m .. m + D + 1.  Node
        // m + k takes jx0 from the lanes with nx0 = m + k and jx1 from those with nx0 = m + k - 1,
        // one term per lane, so each node's sum is one warp reduction of a per-lane value.  The
        // integers are Fix<float>::split's (rint of v * 2^S): below 2^26 one reduction per node
        // (32 of them sum exactly in 32 bits); below 2^46 two, of the 22-bit low pieces and the
        // high parts.  Lane k adds node m + k's sum to the window.  Integer sums: the same bits
        // as the general path below.
        const bool has = nx0 >= 0;
        const int m = __reduce_min_sync(0xffffffffu, has ? nx0 : INT_MAX);
        const int d = has ? nx0 - m : -4;
        int D = __reduce_max_sync(0xffffffffu, has ? d : 0);
        const int r0 = m - base;
        if (D <= 2 && r0 >= 0 && r0 + D + 1 < PIC_WIN) {
            const float x0 = rintf(jx0 * a.jscale_f), x1 = rintf(jx1 * a.jscale_f);
            const float ax = fmaxf(fabsf(x0), fabsf(x1));
            long long s[4] = {0, 0, 0, 0};
            if (__all_sync(0xffffffffu, ax < 67108864.f)) {  // 2^26
                const int X0 = __float2int_rn(x0), X1 = __float2int_rn(x1);
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (k <= D + 1)
                        s[k] = __reduce_add_sync(0xffffffffu, d == k ? X0 : (d == k - 1 ? X1 : 0));
            } else if (__all_sync(0xffffffffu, ax < 70368744177664.f)) {  // 2^46
                const float h0 = floorf(x0 * 2.384185791015625e-07f);  // x / 2^22
                const float h1 = floorf(x1 * 2.384185791015625e-07f);
                const int H0 = __float2int_rn(h0), H1 = __float2int_rn(h1);
                const unsigned L0 = __float2uint_rn(fmaf(-h0, 4194304.f, x0));  // exact, < 2^22
                const unsigned L1 = __float2uint_rn(fmaf(-h1, 4194304.f, x1));
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (k <= D + 1) {
                        const int hs = __reduce_add_sync(
                            0xffffffffu, d == k ? H0 : (d == k - 1 ? H1 : 0));
                        const unsigned ls = __reduce_add_sync(
                            0xffffffffu, d == k ? L0 : (d == k - 1 ? L1 : 0u));
                        s[k] = (long long)hs * 4194304 + (long long)ls;
                    }
            } else {
                D = 99;  // the general path
            }
            if (D <= 2) {
                const long long v = lane == 0 ? s[0] : lane == 1 ? s[1] : lane == 2 ? s[2] : s[3];
                if (lane <= D + 1 && v != 0) smem_add_u64(win + r0 + lane, (unsigned long long)v);
                return;
            }
        }
        // A sparse beam (a few particles a cell: the warp spreads over more nodes than it has
        // lanes a node): every node inside the window, each lane adds its own two words.
        if (D < 99 && D > 2 && r0 >= 0 && r0 + D + 1 < PIC_WIN) {
            if (has) {
                long long v0, v1;
                Fix<T>::split(jx0, a.jscale, a.jscale_f, &v0);
                Fix<T>::split(jx1, a.jscale, a.jscale_f, &v1);
                if (v0 != 0) smem_add_u64(win + (nx0 - base), (unsigned long long)v0);
                if (v1 != 0) smem_add_u64(win + (nx0 + 1 - base), (unsigned long long)v1);
            }
            return;
        }
    }
    // the whole warp on one node pair: warp sums
    const int i0 = __shfl_sync(0xffffffffu, nx0, 0);
    const int r0 = i0 - base;
    const bool pair =
        __all_sync(0xffffffffu, nx0 == i0) && i0 >= 0 && r0 >= 0 && r0 + 1 < PIC_WIN;
    {
        long long vx0[W], vx1[W];
#pragma unroll
        for (int w = 0; w < W; ++w) vx0[w] = vx1[w] = 0;
        if (nx0 >= 0) {
            Fix<T>::split(jx0, a.jscale, a.jscale_f, vx0);
            Fix<T>::split(jx1, a.jscale, a.jscale_f, vx1);
        }
        if (pair) {
            // words that fit 32 bits (small currents) take the two-reduction sum
            bool fit = true;
#pragma unroll
            for (int w = 0; w < W; ++w)
                fit = fit && vx0[w] == (long long)(int)vx0[w] &&
                      vx1[w] == (long long)(int)vx1[w];
            const bool fit_all = __all_sync(0xffffffffu, fit);
#pragma unroll
            for (int w = 0; w < W; ++w) {
                const unsigned long long s0 = fit_all ? warp_sum_i32((int)vx0[w])
                                                      : warp_sum_u64((unsigned long long)vx0[w]);
                const unsigned long long s1 = fit_all ? warp_sum_i32((int)vx1[w])
                                                      : warp_sum_u64((unsigned long long)vx1[w]);
                if (lane == 0) {
                    if (s0 != 0ull) smem_add_u64(win + (size_t)w * PIC_WIN + r0, s0);
                    if (s1 != 0ull) smem_add_u64(win + (size_t)w * PIC_WIN + r0 + 1, s1);
                }
            }
        } else {
            deposit_slot<W>(win, a.acc, nz1, base, 0, nx0, vx0, a.status + 1);
            deposit_slot<W>(win, a.acc, nz1, base, 0, nx1, vx1, a.status + 1);
        }
    }
}

// The register budget is the compiler's (40 in FP32): capping it at 32 for a full SM of push
// CTAs left no room for the next kernel's early-launched CTAs (measured slower on one wave of
// CTAs, no faster on many).
//
// FUSE_H: the launch also carries the previous step's H phase (hf, step offset th) in its first
// a.hblocks CTAs, and the push CTAs take H^(t+1/2) at their two nodes from h_on_the_fly
// instead of reading Hy -- the values the H CTAs write, so the push no longer waits for the H
// phase and the step's chain is E, then push and H together.  The push CTAs read Hyp and Ex
// only, which nothing in the launch writes; the host takes this form when every node a particle
// can gather lies outside the PML columns (fdtdpic_run's beam domain [clo, chi)).
template <typename T, bool FUSE_H>
__global__ void __launch_bounds__(PIC_THREADS, (FUSE_H && sizeof(T) == 4) ? 6 : 1)
    pic_push_kernel(PicArgs<T> a, PicField<T> hf, int th)
{
    constexpr int W = Fix<T>::W;
    __shared__ unsigned long long win[2 * W * PIC_WIN];
    __shared__ int base_s;
    __shared__ HOnTheFly<T> q_s;
    pdl_trigger();
    int blk = blockIdx.x;
    if constexpr (FUSE_H) {
        if (blk < a.hblocks) {
            pic_h_body<T, FIELD_UH_FUSED>(hf, th, blk, a.hblocks);
            return;
        }
        blk -= a.hblocks;
    }
    const int b0 = blk * a.chunk;
    const int b1 = min(a.n_part, b0 + a.chunk);
    if (b0 >= b1) return;
    const int nz1 = a.nz + 1;
    // Jz words are deposited on the call's last step only: other steps clear and flush the
    // Jx half of the window alone
    const int win_words = (a.deposit_jz ? 2 : 1) * W * PIC_WIN;
    for (int i = threadIdx.x; i < win_words; i += blockDim.x) win[i] = 0ull;
    if constexpr (FUSE_H) {
        if (threadIdx.x == 0) {
            // the constant pool and the instance do not change; the step counter is written by
            // launches that completed before this one could start
            const FdtdInstance &I = hf.f.inst[0];
            HOnTheFly<T> q;
            q.src_h = src_h_at<T>(I, hf.f.src, pic_step_index(hf, th));
            q.uh = hf.fc->c.uh;
            q.uh_slab = hf.fc->c.uh_slab;
            q.uh_lo = hf.fc->c.uh_lo;
            q.uh_slab_lo = hf.fc->c.uh_slab_lo;
            q.tfsf_cell = I.tfsf ? I.nzsrc - 1 : INT_MIN;
            const bool fs = I.mode == FDTD_MODE_FREESPACE;
            q.slab_lo = fs ? I.front : 0;
            q.slab_hi = fs ? I.rear : 0;
            q.plain = !I.tfsf && !fs;
            q_s = q;
        }
    }
    pdl_wait();  // the previous step's fields and particles
    // this thread's next particle, loaded one iteration ahead so its loads overlap the current
    // particle's gathers and push; thread 0's first particle (b0) also places the deposit window
    int nc = 0;
    T nf = T(0), nux = T(0), nuz = T(0);
    if (b0 + (int)threadIdx.x < b1) {
        const int p = b0 + threadIdx.x;
        nc = a.cell[p]; nf = a.frac[p]; nux = a.ux[p]; nuz = a.uz[p];
    }
    if (threadIdx.x == 0) base_s = nc - 8;
    __syncthreads();
    const int base = base_s;
    const int Lc = a.chi - a.clo;
    const int iters = (b1 - b0 + blockDim.x - 1) / blockDim.x;
    const int lane = threadIdx.x & 31;
    int lost = 0;
    for (int it = 0; it < iters; ++it) {
        const int p = b0 + it * blockDim.x + threadIdx.x;
        bool valid = p < b1;
        int c = nc;
        T f = nf;
        const T ux0 = nux, uz0 = nuz;
        const int pn = p + blockDim.x;
        if (pn < b1) { nc = a.cell[pn]; nf = a.frac[pn]; nux = a.ux[pn]; nuz = a.uz[pn]; }
        if (valid && (c < 1 || c + 2 > a.nz)) { valid = false; ++lost; }
        // debug build: the gathers' cells c-1 .. c+2 and the particle's slot
        if (valid && !(FDTD_IN(c - 1, nz1, a.status + 1) && FDTD_IN(c + 2, nz1, a.status + 1) &&
                       FDTD_IN(p, a.n_part, a.status + 1)))
            valid = false;
        int nx0 = -1, nzA = -1, nzB = -1;
        T jx0 = T(0), jx1 = T(0);
        long long vzA[W], vzB[W];
#pragma unroll
        for (int w = 0; w < W; ++w) vzA[w] = vzB[w] = 0;
        if (valid) {
            int j;
            T fh;
            if (f >= T(0.5)) { j = c; fh = f - T(0.5); } else { j = c - 1; fh = f + T(0.5); }
            // the fields are read-only during the push: non-coherent loads
            T E, H;
            if constexpr (FUSE_H) {
                // E at j..j+2 covers the cells c, c+1 of the E gather and the nodes' updates
                const T e0 = __ldg(a.ex + j), e1 = __ldg(a.ex + j + 1), e2 = __ldg(a.ex + j + 2);
                const T p0 = __ldg(a.hyp + j), p1 = __ldg(a.hyp + j + 1);
                const bool up = j == c;
                E = (T(1) - f) * (up ? e0 : e1) + f * (up ? e1 : e2);
                const HOnTheFly<T> &q = q_s;
                T n0, n1;
                if (q.plain) {  // the same operations as h_on_the_fly without its two terms
                    n0 = p0 + mul_c(e1 - e0, q.uh, q.uh_lo);
                    n1 = p1 + mul_c(e2 - e1, q.uh, q.uh_lo);
                } else {
                    n0 = h_on_the_fly<T>(q, j, p0, e0, e1);
                    n1 = h_on_the_fly<T>(q, j + 1, p1, e1, e2);
                }
                H = (T(1) - fh) * (T(0.5) * (n0 + p0)) + fh * (T(0.5) * (n1 + p1));
            } else {
                E = (T(1) - f) * __ldg(a.ex + c) + f * __ldg(a.ex + c + 1);
                H = (T(1) - fh) * (T(0.5) * (__ldg(a.hy + j) + __ldg(a.hyp + j))) +
                    fh * (T(0.5) * (__ldg(a.hy + j + 1) + __ldg(a.hyp + j + 1)));
            }
            Moved<T> m;
            particle_step<T>(E, H, c, f, ux0, uz0, a.kE, a.kH, a.sc, a.kJ, m);
            const T uxn = m.ux, uzn = m.uz, f1 = m.f1;
            int c1 = m.c1;
            nx0 = m.nx0;
            jx0 = m.jx0;
            jx1 = m.jx1;
            if (a.deposit_jz) {
                const MovedJz<T> z = particle_jz<T>(c, f, m, a.kJz);
                nzA = z.nzA;
                nzB = z.nzB;
                Fix<T>::split(z.jzA, a.jscale, a.jscale_f, vzA);
                if (nzB >= 0) Fix<T>::split(z.jzB, a.jscale, a.jscale_f, vzB);
            }
            if (c1 >= a.chi) c1 -= Lc;
            else if (c1 < a.clo) c1 += Lc;
            a.cell[p] = c1;
            a.frac[p] = f1;
            a.ux[p] = uxn;
            a.uz[p] = uzn;
        }
        push_deposit_jx<T>(win, a, nz1, base, lane, nx0, jx0, jx1);
        if (a.deposit_jz) {
            deposit_slot<W>(win, a.acc, nz1, base, W, nzA, vzA, a.status + 1);
            deposit_slot<W>(win, a.acc, nz1, base, W, nzB, vzB, a.status + 1);
        }
    }
    if (lost) atomicAdd(a.status, lost);
    __syncthreads();
    for (int i = threadIdx.x; i < win_words; i += blockDim.x) {
        const unsigned long long v = win[i];
        const int word = i / PIC_WIN;
        const int node = base + (i % PIC_WIN);
        if (v != 0ull && node >= 0 && node < nz1) atomicAdd(a.acc + (size_t)word * nz1 + node, v);
    }
}

// The device step counter: set before the first replayed block, advanced by a block's length
// at the end of each block (one launch per block, not per step).
static __global__ void pic_advance_kernel(int32_t *step, int k) { *step += k; }
static __global__ void pic_set_step_kernel(int32_t *step, int t) { *step = t; }

// Whole field step in one CTA (grids up to PIC_FUSED_MAX cells): E phase, barrier, H phase,
// probes.  Saves a launch per step.
constexpr int PIC_FUSED_MAX = 1024;
template <typename T>
__global__ void __launch_bounds__(1024) pic_field_fused_kernel(PicField<T> a, int t_arg)
{
    const FdtdInstance &I = instance_block(a.f.inst[0]);
    const int t = pic_step_index(a, t_arg);
    GlobalStore<T> s = global_store<T>(I, a.f);
    Scal<T> c;
    Kerr<T> kr;
    consts_block<T>(a.fc, c, kr);
    T src_e, src_h;
    source_block<T>(I, a.f.src, t, src_e, src_h);
    const int n = I.nz + 1;
    T *gA = a.f.state + I.state_offset + (int64_t)FDTD_ST_A * n;
    int nfb = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        pic_e_cell<T>(a, I, s, c, kr, k, n, src_e, src_h, gA, &nfb);
    __syncthreads();
    for (int k = 1 + threadIdx.x; k < n - 1; k += blockDim.x) h_cell<T>(I, c, s, k, src_h);
    if (threadIdx.x == 0) tfsf_edge<T>(I, s, src_h);
    pic_probes<T>(a, I, s, t, threadIdx.x, blockDim.x, n);
    if (nfb && a.f.fallbacks) atomicAdd(a.f.fallbacks, nfb);
}

// ---- re-binning by cell (counting sort; order within a cell is not kept and does not matter)
// The particles are in cell order from the last re-binning (and have moved little since), so a
// warp's 32 particles form a few runs of equal cells: each run takes one atomic for all its
// lanes (run heads: lanes whose cell differs from the previous lane's).  The loops run whole
// warps (out-of-range lanes carry cell -1).

// Lanes of the run that lane `lane` heads (heads: the warp's run-head mask, lane a head).
__device__ __forceinline__ int run_length(unsigned heads, int lane)
{
    const unsigned later = heads & ~((2u << lane) - 1u);  // heads after this lane (none: 0)
    return (later ? __ffs(later) - 1 : 32) - lane;
}
// The head of the run holding lane `lane`.
__device__ __forceinline__ int run_head(unsigned heads, int lane)
{
    return 31 - __clz(heads & ((2u << lane) - 1u));
}

static __global__ void pic_hist_kernel(int n_part, const int32_t *cell, int32_t *counts, int nz1)
{
    const int lane = threadIdx.x & 31;
    for (int p0 = blockIdx.x * blockDim.x; p0 < n_part; p0 += gridDim.x * blockDim.x) {
        const int p = p0 + threadIdx.x;
        const int c0 = p < n_part ? cell[p] : -1;
        const int c = (c0 >= 0 && c0 < nz1) ? c0 : -1;
        const int prev = __shfl_up_sync(0xffffffffu, c, 1);
        const bool head = lane == 0 || c != prev;
        const unsigned heads = __ballot_sync(0xffffffffu, head);
        if (head && c >= 0) atomicAdd(counts + c, run_length(heads, lane));
    }
}

// Exclusive scan of counts[0..n) into cursor, three launches over tiles of SCAN_TILE counts:
// per-tile sums, a scan of the tile sums (one CTA), then each tile's scan plus its offset.
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_PER_THREAD = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_PER_THREAD;

inline int scan_tiles(int n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

// Block-wide exclusive scan of one int per thread (SCAN_THREADS threads); returns the total.
__device__ __forceinline__ int block_exclusive_scan(int v, int &excl)
{
    __shared__ int warp_tot[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_tot[lane] = w;  // inclusive
    }
    __syncthreads();
    const int before = wid ? warp_tot[wid - 1] : 0;
    excl = before + x - v;
    const int total = warp_tot[SCAN_THREADS / 32 - 1];
    __syncthreads();  // warp_tot may be reused by the next call
    return total;
}

static __global__ void __launch_bounds__(SCAN_THREADS) pic_scan_sums_kernel(const int32_t *counts,
                                                                             int32_t *tile_sum, int n)
{
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
    int s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_PER_THREAD; ++j)
        if (base + j < n) s += counts[base + j];
    int excl;
    const int tot = block_exclusive_scan(s, excl);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

static __global__ void __launch_bounds__(SCAN_THREADS) pic_scan_top_kernel(int32_t *tile_sum, int nt)
{
    int carry = 0;
    for (int b0 = 0; b0 < nt; b0 += SCAN_THREADS) {
        const int i = b0 + threadIdx.x;
        const int v = (i < nt) ? tile_sum[i] : 0;
        int excl;
        const int tot = block_exclusive_scan(v, excl);
        if (i < nt) tile_sum[i] = carry + excl;
        carry += tot;
    }
}

static __global__ void __launch_bounds__(SCAN_THREADS) pic_scan_final_kernel(const int32_t *counts,
                                                                              const int32_t *tile_off,
                                                                              int32_t *cursor, int n)
{
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
    int c[SCAN_PER_THREAD];
    int s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_PER_THREAD; ++j) {
        c[j] = (base + j < n) ? counts[base + j] : 0;
        s += c[j];
    }
    int run;
    block_exclusive_scan(s, run);
    run += tile_off[blockIdx.x];
#pragma unroll
    for (int j = 0; j < SCAN_PER_THREAD; ++j) {
        if (base + j < n) cursor[base + j] = run;
        run += c[j];
    }
}

template <typename T>
__global__ void pic_scatter_kernel(int n_part, const int32_t *cell, const T *frac, const T *ux,
                                   const T *uz, const int32_t *id, int32_t *cursor, int nz1,
                                   int32_t *cell2, T *frac2, T *ux2, T *uz2, int32_t *id2)
{
    const int lane = threadIdx.x & 31;
    for (int p0 = blockIdx.x * blockDim.x; p0 < n_part; p0 += gridDim.x * blockDim.x) {
        const int p = p0 + threadIdx.x;
        const bool in = p < n_part;
        const int c0 = in ? cell[p] : -1;
        const int c = (c0 >= 0 && c0 < nz1) ? c0 : -1;
        T f = T(0), x = T(0), z = T(0);
        int i = 0;
        if (c >= 0) { f = frac[p]; x = ux[p]; z = uz[p]; i = id[p]; }
        // each run of equal cells claims its slots with one atomic (see pic_hist_kernel)
        const int prev = __shfl_up_sync(0xffffffffu, c, 1);
        const bool head = lane == 0 || c != prev;
        const unsigned heads = __ballot_sync(0xffffffffu, head);
        int base = 0;
        if (head && c >= 0) base = atomicAdd(cursor + c, run_length(heads, lane));
        const int h = run_head(heads, lane);
        const int q = __shfl_sync(0xffffffffu, base, h) + (lane - h);
        if (c < 0 || q >= n_part) continue;
        if (!FDTD_IN(q, n_part, nullptr)) continue;
        cell2[q] = c;
        frac2[q] = f;
        ux2[q] = x;
        uz2[q] = z;
        id2[q] = i;
    }
}

template <typename T>
__global__ void pic_finish_kernel(const T *state, int n, int32_t *status)
{
    bool bad = false;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        bad |= !(isfinite((double)state[k]) && isfinite((double)state[n + k]));
    if (bad) atomicOr(status + 1, FDTD_STATUS_NONFINITE);
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Scratch layout shared by the size query and the launcher.
struct PicScratch {
    size_t acc, counts, cursor, step, tile_sum, consts, cell2, frac2, ux2, uz2, id2, total;
};
inline PicScratch pic_scratch_layout(int tsize, int nz, int n_part)
{
    PicScratch L;
    const size_t nz1 = (size_t)nz + 1;
    const int W = (tsize == 8) ? 2 : 1;
    size_t o = 0;
    L.acc = o; o = align256(o + 2 * W * nz1 * 8);
    L.counts = o; o = align256(o + (nz1 + 1) * 4);
    L.cursor = o; o = align256(o + (nz1 + 1) * 4);
    L.step = o; o = align256(o + 4);
    L.tile_sum = o; o = align256(o + ((nz1 + SCAN_TILE - 1) / SCAN_TILE + 1) * 4);
    L.consts = o; o = align256(o + sizeof(FieldConsts<double>));
    L.cell2 = o; o = align256(o + (size_t)n_part * 4);
    L.frac2 = o; o = align256(o + (size_t)n_part * tsize);
    L.ux2 = o; o = align256(o + (size_t)n_part * tsize);
    L.uz2 = o; o = align256(o + (size_t)n_part * tsize);
    L.id2 = o; o = align256(o + (size_t)n_part * 4);
    L.total = o;
    return L;
}

// Per-kernel-type CUDA-event timing (see FdtdPicTiming in fdtdpic.h).
struct PicTimer {
    FdtdPicTiming *out;
    cudaStream_t st;
    cudaEvent_t ev[2];
    int open;
    float *slot;
    void begin(float *which)
    {
        if (!out) return;
        cudaEventRecord(ev[0], st);
        slot = which;
    }
    void end()
    {
        if (!out) return;
        cudaEventRecord(ev[1], st);
        cudaEventSynchronize(ev[1]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[0], ev[1]);
        *slot += ms;
    }
};

template <typename T>
struct PicPlan {
    int threads, fblocks, pblocks, sblocks, nz1;
    bool fused;
    bool fuse_h;  // the push launch carries the previous step's H phase (pic_push_kernel FUSE_H)
    PicArgs<T> pa;
    PicField<T> pf;
    int32_t *counts, *cursor, *step, *tile_sum;
    // particle buffers: A = caller's, B = scratch
    int32_t *cellA, *cellB, *idA, *idB;
    T *fracA, *fracB, *uxA, *uxB, *uzA, *uzB;
};

// A step's H phase not yet launched: the next push launch carries it (fuse_h), or pic_flush_h
// launches it alone.
template <typename T>
struct PendingH {
    bool on;
    PicField<T> pf;
    int t;
};

template <typename T>
void pic_flush_h(PicPlan<T> &P, PendingH<T> &ph, cudaStream_t st, PicTimer *tm)
{
    if (!ph.on) return;
    if (tm) tm->begin(&tm->out->field_ms);
    launch_pdl(pic_h_kernel<T>, P.fblocks, P.threads, st, ph.pf, ph.t);
    if (tm) tm->end();
    ph.on = false;
}

// Enqueue one step; `in_b` selects which buffer holds the particles (flips when re-binning).
// The step's H phase is left pending in `ph` when the plan fuses it into the next push launch;
// the caller flushes it after the last step.
template <typename T>
void pic_enqueue_step(PicPlan<T> &P, const PicBeam &bm, int t, bool do_sort, bool &in_b,
                      bool device_step, cudaStream_t st, PicTimer *tm, bool last_step,
                      PendingH<T> &ph)
{
    if (do_sort) {
        pic_flush_h(P, ph, st, tm);
        int32_t *cS = in_b ? P.cellB : P.cellA, *cD = in_b ? P.cellA : P.cellB;
        int32_t *iS = in_b ? P.idB : P.idA, *iD = in_b ? P.idA : P.idB;
        T *fS = in_b ? P.fracB : P.fracA, *fD = in_b ? P.fracA : P.fracB;
        T *xS = in_b ? P.uxB : P.uxA, *xD = in_b ? P.uxA : P.uxB;
        T *zS = in_b ? P.uzB : P.uzA, *zD = in_b ? P.uzA : P.uzB;
        if (tm) tm->begin(&tm->out->sort_ms);
        cudaMemsetAsync(P.counts, 0, (size_t)(P.nz1 + 1) * 4, st);
        pic_hist_kernel<<<P.sblocks, P.threads, 0, st>>>(bm.n_part, cS, P.counts, P.nz1);
        const int ntile = scan_tiles(P.nz1);
        pic_scan_sums_kernel<<<ntile, SCAN_THREADS, 0, st>>>(P.counts, P.tile_sum, P.nz1);
        pic_scan_top_kernel<<<1, SCAN_THREADS, 0, st>>>(P.tile_sum, ntile);
        pic_scan_final_kernel<<<ntile, SCAN_THREADS, 0, st>>>(P.counts, P.tile_sum, P.cursor,
                                                               P.nz1);
        pic_scatter_kernel<T><<<P.sblocks, P.threads, 0, st>>>(bm.n_part, cS, fS, xS, zS, iS,
                                                              P.cursor, P.nz1, cD, fD, xD, zD, iD);
        if (tm) tm->end();
        in_b = !in_b;
    }
    P.pa.cell = in_b ? P.cellB : P.cellA;
    P.pa.frac = in_b ? P.fracB : P.fracA;
    P.pa.ux = in_b ? P.uxB : P.uxA;
    P.pa.uz = in_b ? P.uzB : P.uzA;
    if (bm.n_part > 0) {
        if (tm) tm->begin(&tm->out->push_ms);
        P.pa.deposit_jz = last_step ? 1 : 0;
        const bool with_h = ph.on && P.fuse_h;
        if (!with_h) pic_flush_h(P, ph, st, tm);
        P.pa.hblocks = with_h ? P.fblocks : 0;
        const int grid = P.pblocks + (with_h ? P.fblocks : 0);
        if (with_h)
            launch_pdl(pic_push_kernel<T, true>, grid, PIC_THREADS, st, P.pa, ph.pf, ph.t);
        else
            launch_pdl(pic_push_kernel<T, false>, grid, PIC_THREADS, st, P.pa, P.pf, 0);
        if (with_h) ph.on = false;
        if (tm) tm->end();
    } else {
        pic_flush_h(P, ph, st, tm);
    }
    PicField<T> pf = P.pf;
    pf.step = device_step ? P.step : nullptr;
    pf.last = last_step ? 1 : 0;
    if (tm) tm->begin(&tm->out->field_ms);
    if (P.fused) {
        pic_field_fused_kernel<T><<<1, 1024, 0, st>>>(pf, t);
        if (tm) tm->end();
    } else {
        launch_pdl(pic_e_kernel<T>, P.fblocks, P.threads, st, pf, t);
        if (tm) tm->end();
        ph.on = true;
        ph.pf = pf;
        ph.t = t;
        if (!P.fuse_h) pic_flush_h(P, ph, st, tm);
    }
}

// Captured step blocks, kept for replay by later calls with identical arguments.
struct PicGraphEntry {
    unsigned char key[512];
    size_t key_len;
    cudaGraphExec_t exec;
};
PicGraphEntry *pic_graph_lookup(const void *key, size_t len);
void pic_graph_store(const void *key, size_t len, cudaGraphExec_t exec);
cudaStream_t pic_capture_stream();

template <typename T>
int launch_pic(int precision_bytes, const FdtdInstance &h, const BatchArgs<T> &fa,
               const PicBeam &bm, int32_t *cell, T *frac, T *ux, T *uz, int32_t *id, T *jx, T *jz,
               T *hyp, unsigned char *scratch, int32_t *status, FdtdPicTiming *timing,
               cudaStream_t st, bool allow_graphs = true)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FDTDPIC_ERR_NODEV;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const PicScratch L = pic_scratch_layout(precision_bytes, h.nz, bm.n_part);
    const int nz1 = h.nz + 1;
    constexpr int W = Fix<T>::W;
    PicPlan<T> P;
    unsigned long long *acc = (unsigned long long *)(scratch + L.acc);
    P.counts = (int32_t *)(scratch + L.counts);
    P.cursor = (int32_t *)(scratch + L.cursor);
    P.step = (int32_t *)(scratch + L.step);
    P.tile_sum = (int32_t *)(scratch + L.tile_sum);
    P.cellA = cell; P.fracA = frac; P.uxA = ux; P.uzA = uz; P.idA = id;
    P.cellB = (int32_t *)(scratch + L.cell2);
    P.fracB = (T *)(scratch + L.frac2);
    P.uxB = (T *)(scratch + L.ux2);
    P.uzB = (T *)(scratch + L.uz2);
    P.idB = (int32_t *)(scratch + L.id2);
    P.nz1 = nz1;
    P.threads = 256;
    P.fblocks = (nz1 + P.threads - 1) / P.threads;
    if (P.fblocks > 8 * sms) P.fblocks = 8 * sms;
    P.fused = nz1 <= PIC_FUSED_MAX;
    PicArgs<T> &pa = P.pa;
    pa.n_part = bm.n_part; pa.nz = h.nz; pa.clo = bm.clo; pa.chi = bm.chi;
    pa.chunk = bm.chunk > 0 ? bm.chunk : 1024;
    pa.kE = (T)bm.kE; pa.kH = (T)bm.kH; pa.sc = (T)bm.sc; pa.kJ = (T)bm.kJ; pa.kJz = (T)bm.kJz;
    pa.jscale = bm.jscale; pa.jinv = 1.0 / bm.jscale;
    pa.jscale_f = (float)bm.jscale; pa.jinv_f = (float)(1.0 / bm.jscale);
    const T *st0 = fa.state + h.state_offset;
    pa.ex = st0 + (int64_t)FDTD_ST_EX * nz1;
    pa.hy = st0 + (int64_t)FDTD_ST_HY * nz1;
    pa.hyp = hyp;
    pa.acc = acc;
    pa.status = status;
    P.pf.f = fa; P.pf.acc = acc; P.pf.jx = jx; P.pf.jz = jz; P.pf.hyp = hyp;
    P.pf.jinv = pa.jinv; P.pf.jinv_f = pa.jinv_f; P.pf.step = nullptr; P.pf.last = 0;
    P.pf.fc = (const FieldConsts<T> *)(scratch + L.consts);
    P.pblocks = (bm.n_part + pa.chunk - 1) / pa.chunk;
    pa.hblocks = 0;
    {
        // The push launch carries the previous step's H phase when the caller guarantees the
        // particles' cells are in [clo, chi), every node a particle can then gather
        // (clo-1 .. chi) lies strictly inside [1, nz-1] and outside the PML columns
        // (h_on_the_fly's condition), and the launch is a few waves of push CTAs (its step is
        // latency-bound; in many-wave launches the push's extra arithmetic costs more than the
        // launch it saves).  Timed kernel by kernel, the fused launch counts as push time.
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pic_push_kernel<T, true>,
                                                          PIC_THREADS, 0) != cudaSuccess)
            per_sm = 0;
        const long long slots = (long long)per_sm * sms;
        const bool inside = bm.clo - 1 > h.pml && bm.clo - 1 >= 1 && bm.chi < nz1 - h.pml &&
                            bm.chi <= h.nz - 1;
        P.fuse_h = !P.fused && bm.n_part > 0 && inside && slots > 0 &&
                   (bm.path & FDTDPIC_PATH_CELLS_INSIDE) && (long long)P.pblocks <= 4 * slots;
        // a latency-bound step runs faster with fewer particles per thread (768 a CTA measured
        // best on GB300 for a one-to-two-wave beam); a launch of more than four waves with more
        // (on the 64M-particle instance, ms a step: 4096 a CTA 0.675, 2048 0.687, 1024 0.729,
        // 512 0.830)
        if (P.fuse_h && bm.chunk == 0) {
            pa.chunk = 768;
            P.pblocks = (bm.n_part + pa.chunk - 1) / pa.chunk;
        } else if (bm.chunk == 0 && slots > 0 && (long long)P.pblocks > 4 * slots) {
            pa.chunk = 4096;
            P.pblocks = (bm.n_part + pa.chunk - 1) / pa.chunk;
        }
    }
    P.sblocks = (bm.n_part + P.threads - 1) / P.threads;
    if (P.sblocks > 16 * sms) P.sblocks = 16 * sms;
    if (P.sblocks < 1) P.sblocks = 1;

    cudaError_t e = cudaMemsetAsync(acc, 0, (size_t)2 * W * nz1 * 8, st);
    if (e != cudaSuccess) return cuda_status(e);
    if (!h.resume) fdtd_global_init_kernel<T><<<P.fblocks, P.threads, 0, st>>>(fa);
    pic_consts_kernel<T><<<1, 32, 0, st>>>(fa.inst, (FieldConsts<T> *)(scratch + L.consts));

    PicTimer tmr{timing, st, {nullptr, nullptr}, 0, nullptr};
    if (timing) {
        *timing = FdtdPicTiming{};
        cudaEventCreate(&tmr.ev[0]);
        cudaEventCreate(&tmr.ev[1]);
    }
    const bool sorting = bm.sort_every > 0 && bm.n_part > 0;
    // one captured block = two re-binning periods, so the particles end where they started
    const int K = sorting ? 2 * bm.sort_every : 64;
    const int total = h.step_end - h.step_begin;
    // graph blocks never cover the last step (it deposits Jz), so at most (total-1)/K blocks
    const int nblocks = (timing || !allow_graphs || total < 1) ? 0 : (total - 1) / K;
    bool in_b = false;
    int t = h.step_begin;
    if (nblocks > 0) {
        struct Key {
            const void *p[16];
            FdtdInstance inst;
            PicBeam beam;
            int K, sms;
        } key;
        memset(&key, 0, sizeof(key));
        const void *ptrs[16] = {fa.inst, fa.src, fa.state, fa.probe, fa.hist, fa.pml_tab, cell,
                                frac, ux, uz, id, jx, jz, hyp, scratch, status};
        for (int i = 0; i < 16; ++i) key.p[i] = ptrs[i];
        key.inst = h;
        key.inst.step_begin = key.inst.step_end = key.inst.resume = 0;
        key.beam = bm;
        key.K = K;
        key.sms = sms;
        PicGraphEntry *ent = pic_graph_lookup(&key, sizeof(key));
        cudaGraphExec_t exec = ent ? ent->exec : nullptr;
        if (!exec) {
            cudaStream_t cs = pic_capture_stream();
            if (!cs) return FDTDPIC_ERR_CUDA;
            e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_status(e);
            bool cb = false;
            // a block starts with no H phase pending and ends with its last one launched, so
            // every replay is the same sequence
            PendingH<T> bh{};
            for (int j = 0; j < K; ++j)
                pic_enqueue_step<T>(P, bm, j, sorting && (j % bm.sort_every) == 0, cb, true, cs,
                                    nullptr, false, bh);
            pic_flush_h(P, bh, cs, nullptr);
            pic_advance_kernel<<<1, 1, 0, cs>>>(P.step, K);
            cudaGraph_t graph = nullptr;
            e = cudaStreamEndCapture(cs, &graph);
            if (e != cudaSuccess) return cuda_status(e);
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_status(e);
            pic_graph_store(&key, sizeof(key), exec);
        }
        pic_set_step_kernel<<<1, 1, 0, st>>>(P.step, t);
        for (int b = 0; b < nblocks; ++b) {
            e = cudaGraphLaunch(exec, st);
            if (e != cudaSuccess) return cuda_status(e);
        }
        t += nblocks * K;
    }
    PendingH<T> ph{};
    for (; t < h.step_end; ++t)
        pic_enqueue_step<T>(P, bm, t, sorting && ((t - h.step_begin) % bm.sort_every) == 0, in_b,
                            false, st, timing ? &tmr : nullptr, t == h.step_end - 1, ph);
    pic_flush_h(P, ph, st, timing ? &tmr : nullptr);
    if (in_b && bm.n_part > 0) {
        const size_t np = (size_t)bm.n_part;
        e = cudaMemcpyAsync(cell, P.cellB, np * 4, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(frac, P.fracB, np * sizeof(T), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ux, P.uxB, np * sizeof(T), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(uz, P.uzB, np * sizeof(T), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(id, P.idB, np * 4, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_status(e);
    }
    pic_finish_kernel<T><<<P.fblocks, P.threads, 0, st>>>(fa.state + h.state_offset, nz1, status);
    if (timing) {
        timing->steps = total;
        timing->path = P.fuse_h ? 3 : 1;
        cudaEventDestroy(tmr.ev[0]);
        cudaEventDestroy(tmr.ev[1]);
    }
    return cuda_status(cudaGetLastError());
}

}  // namespace fdtdpic
