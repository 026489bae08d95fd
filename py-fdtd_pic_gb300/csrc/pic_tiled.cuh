// Persistent, tiled FDTD + PIC kernel for grids small enough to spread over co-resident CTAs.
//
// One cooperative launch runs every step.  CTA b owns the cells [c0, c1) of a tile: their Ex,
// Hy, Hyp, Dx, P, psi live in shared memory for the whole run, and so do a halo of one node on
// each side.  Its particles live in a per-tile segment of global memory (double buffered, in the
// L2 for the workload sizes this path takes).  Per step:
//
//   push     gather from shared memory, Boris push, exact int64 deposits into per-warp
//            shared-memory copies of the tile's currents (nodes c0-1 .. c1+1); particles that
//            stay go to the next segment, the others to the left/right (or wrap-partner) outbox
//   round A  publish the halo deposits (Jx at c0-1 | c1, c1+1; Jz at c0-1 | c1) and the migrants;
//            wait for the neighbours' round A; add their deposits on my nodes, adopt migrants
//   E phase  the reference E phase on my cells with -Jx (fdtd1d_kernel.cuh, e_cell)
//   round B  publish Ex[c0], Ex[c0+1] (left) and Ex[c1-1] (right); wait for the neighbours'
//   H phase  my cells plus a redundant update of the halo cells c0-1 and c1 (the neighbours'
//            boundary Hy, computed bit for bit as their owners do), probes, snapshots
//
// Handshakes are per-tile step counters (release store after a fence, acquire load).  Every
// wait is bounded (iteration count and a %globaltimer deadline); a CTA that gives up raises a
// shared abort word, which every other wait also checks, and all CTAs return; the caller's
// status word then carries FDTD_STATUS_TIMEOUT.  An outbox or segment overflow aborts the same
// way with FDTD_STATUS_OVERFLOW.
// Deposits are exact integer sums, so the fields are bit-identical to the streaming kernels'.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_kernel.cuh"

namespace fdtdpic {

constexpr int TILE_THREADS = 512;
constexpr int PIC_UNROLL = 4;
constexpr int TILE_WARPS = TILE_THREADS / 32;
constexpr int MIG_DIRS = 3;  // 0: to the right tile, 1: to the left tile, 2: to the wrap partner

// Tile b covers cells [tile_begin(b), tile_begin(b+1)): widths differ by at most one cell.
__host__ __device__ inline int tile_begin(int b, int G, int n) { return (int)(((long long)b * n) / G); }
__host__ __device__ inline int tile_of(int k, int G, int n)
{
    int b = (int)(((long long)k * G) / n);
    while (b + 1 < G && tile_begin(b + 1, G, n) <= k) ++b;
    while (b > 0 && tile_begin(b, G, n) > k) --b;
    return b;
}

template <typename T>
struct TileArgs {
    BatchArgs<T> f;   // instance, tables, source, state, probe, hist
    int G, w;         // tiles and tile width (cells)
    int clo, chi;     // beam domain
    int wrap_lo, wrap_hi;  // tiles holding clo and chi-1
    int cap, mig_cap;
    T kE, kH, sc, kJ, kJz;
    double jscale, jinv;
    float jscale_f, jinv_f;
    int32_t *cell[2];
    T *frac[2], *ux[2], *uz[2];
    int32_t *id[2];
    int32_t *count;   // [2][G]
    int32_t *flags;   // [G][64]: round A at [0], round B at [32]
    unsigned long long *jhalo;  // [G][5][W]
    T *exhalo;        // [G][3]
    int32_t *migcount;  // [2 parities][G][3]
    int32_t *mcell;   // [2][G][3][mig_cap]
    T *mfrac, *mux, *muz;
    int32_t *mid;
    T *jx_out, *jz_out, *hyp_out;
    int32_t *status;  // [0] lost, [1] status bits
    int32_t *abort;   // first error code of any CTA (0: none)
    int32_t *final_seg;  // segment holding the particles after the run
    long long timeout_ns;
};

__device__ __forceinline__ int ld_acquire(const int32_t *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int32_t *p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Per-run deadline set by fdtdpic_set_run_deadline (0: the default); defined in capi.cu.
long long tiled_deadline_override_ns();

__device__ __forceinline__ long long globaltimer()
{
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Thread 0 only.  true when *flag >= target; false after an abort or the deadline.  A wait that
// starts after the deadline gives up at once, so a run past its time limit stops at its next
// wait whether or not that wait would have to spin.
__device__ inline bool tile_wait(const int32_t *flag, int target, int32_t *abort, long long deadline)
{
    if (globaltimer() > deadline) {
        atomicCAS(abort, 0, FDTDPIC_ERR_TIMEOUT);
        return false;
    }
    for (long long it = 0; it < (1LL << 34); ++it) {
        if (ld_acquire(flag) >= target) return true;
        if ((it & 255) == 255) {
            if (*(volatile int32_t *)abort) return false;
            if (globaltimer() > deadline) {
                atomicCAS(abort, 0, FDTDPIC_ERR_TIMEOUT);
                return false;
            }
        }
    }
    atomicCAS(abort, 0, FDTDPIC_ERR_TIMEOUT);
    return false;
}

// Cell k of this tile in shared memory; base = c0 - 1 (one halo node on each side).
template <typename T>
struct TileStore {
    T *ex, *hy, *dx, *p, *pp, *psie, *psih;
    const double *tab;
    int base, c0, W;
    __device__ T &Ex(int k) { return ex[k - base]; }
    __device__ T &Hy(int k) { return hy[k - base]; }
    __device__ T ExR(int k) { return ex[k - base]; }
    __device__ T HyR(int k) { return hy[k - base]; }
    __device__ T &Dx(int k) { return dx[k - c0]; }
    __device__ T &P(int k) { return p[k - c0]; }
    __device__ T &Pp(int k) { return pp[k - c0]; }
    __device__ T &PsiE(int, int k) { return psie[k - c0]; }
    __device__ T &PsiH(int, int k) { return psih[k - c0]; }
    __device__ T tab_at(int row, int col) const { return (T)tab[row * W + col]; }
};

__host__ __device__ inline int64_t tile_smem_bytes(int tsize, int w)
{
    const int W = (tsize == 8) ? 2 : 1;
    const int L = w + 3;
    int64_t b = (int64_t)tsize * (4 * L + 5 * w) + 8LL * (TILE_WARPS + 1) * 2 * W * L + 64;
    return (b + 15) & ~15LL;
}

template <typename T>
__global__ void __launch_bounds__(TILE_THREADS, 1) pic_tiled_kernel(TileArgs<T> a)
{
    constexpr int W = Fix<T>::W;
    extern __shared__ __align__(16) unsigned char sm_raw[];
    __shared__ int s_nstay, s_nout[MIG_DIRS], s_err, s_lost, s_count;
    __shared__ T s_src[2];
    const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    const int warp = tid >> 5;
    const FdtdInstance &I = instance_block(a.f.inst[0]);
    const int n = I.nz + 1;
    const int c0 = tile_begin(b, a.G, n);
    const int c1 = tile_begin(b + 1, a.G, n);
    const int base = c0 - 1;
    const int L = a.w + 3;  // local nodes base .. base+L-1 = c0-1 .. c1+1 (max width)

    // shared memory: fields, slab and PML state, currents
    T *ex = reinterpret_cast<T *>(sm_raw);
    T *hy = ex + L;
    T *hyp = hy + L;
    T *jloc = hyp + L;  // Jx of my nodes (state type), local index
    T *dx = jloc + L;
    T *pc = dx + a.w;
    T *pp = pc + a.w;
    T *psie = pp + a.w;
    T *psih = psie + a.w;
    unsigned long long *jw = reinterpret_cast<unsigned long long *>(
        reinterpret_cast<unsigned char *>(psih + a.w) + ((8 - (((uintptr_t)(psih + a.w)) & 7)) & 7));
    unsigned long long *jt = jw + (size_t)TILE_WARPS * 2 * W * L;  // tile sums [2W][L]

    TileStore<T> s;
    s.ex = ex; s.hy = hy; s.dx = dx; s.p = pc; s.pp = pp; s.psie = psie; s.psih = psih;
    s.tab = a.f.pml_tab + I.pml_offset;
    s.base = base; s.c0 = c0; s.W = 2 * I.pml + 1;

    // ---- load the tile (own cells + halos) from the global state
    const T *g = a.f.state + I.state_offset;
    const T *gEx = g + (int64_t)FDTD_ST_EX * n, *gHy = g + (int64_t)FDTD_ST_HY * n;
    for (int l = tid; l < L; l += nt) {
        const int k = base + l;
        const bool in = (k >= 0 && k < n);
        ex[l] = in ? gEx[k] : T(0);
        hy[l] = in ? gHy[k] : T(0);
        hyp[l] = in ? a.hyp_out[k] : T(0);
        jloc[l] = T(0);
    }
    for (int i = tid; i < a.w; i += nt) {
        const int k = c0 + i;
        const bool in = k < c1;
        dx[i] = in ? g[(int64_t)FDTD_ST_DX * n + k] : T(0);
        pc[i] = in ? g[(int64_t)FDTD_ST_P * n + k] : T(0);
        pp[i] = in ? g[(int64_t)FDTD_ST_PPREV * n + k] : T(0);
        psie[i] = in ? g[(int64_t)FDTD_ST_PSIE * n + k] : T(0);
        psih[i] = in ? g[(int64_t)FDTD_ST_PSIH * n + k] : T(0);
    }
    for (int i = tid; i < (TILE_WARPS + 1) * 2 * W * L; i += nt) jw[i] = 0ull;
    if (tid == 0) { s_err = 0; s_lost = 0; }
    const Scal<T> sc = make_scal<T>(I);
    Kerr<T> kr;
    kr.setup(I);
    T *gA = a.f.state + I.state_offset + (int64_t)FDTD_ST_A * n;
    const long long deadline = globaltimer() + a.timeout_ns;
    const int Lc = a.chi - a.clo;
    const bool has_left = b > 0, has_right = b < a.G - 1;
    int partner = -1;
    if (b == a.wrap_hi && a.wrap_lo != b && abs(a.wrap_lo - b) > 1) partner = a.wrap_lo;
    if (b == a.wrap_lo && a.wrap_hi != b && abs(a.wrap_hi - b) > 1) partner = a.wrap_hi;
    int32_t *myflags = a.flags + (size_t)b * 64;
    int cur = 0;
    int nfb = 0;
    __syncthreads();

    for (int t = I.step_begin; t < I.step_end; ++t) {
        const int target = t - I.step_begin + 1;
        const bool last = (t == I.step_end - 1);
        const int par = target & 1;  // migrant boxes alternate by step (the wrap partner does not
                                     // wait for my round B, so it may read a box one step late)
        const int nxt = cur ^ 1;
        // ---------------- push ----------------
        if (tid == 0) {
            s_nstay = 0;
            for (int d = 0; d < MIG_DIRS; ++d) s_nout[d] = 0;
            s_count = min(a.count[cur * a.G + b], a.cap);  // a bin overflow is reported, not read past
        }
        __syncthreads();
        const int np = s_count;
        const size_t seg = (size_t)b * a.cap;
        // this step's segment pointers in registers (selected, not indexed: a dynamic index into
        // the parameter struct's arrays would go through local memory)
        int32_t *const cellC = cur ? a.cell[1] : a.cell[0];
        int32_t *const cellN = cur ? a.cell[0] : a.cell[1];
        T *const fracC = cur ? a.frac[1] : a.frac[0];
        T *const fracN = cur ? a.frac[0] : a.frac[1];
        T *const uxC = cur ? a.ux[1] : a.ux[0];
        T *const uxN = cur ? a.ux[0] : a.ux[1];
        T *const uzC = cur ? a.uz[1] : a.uz[0];
        T *const uzN = cur ? a.uz[0] : a.uz[1];
        int32_t *const idC = cur ? a.id[1] : a.id[0];
        int32_t *const idN = cur ? a.id[0] : a.id[1];
        unsigned long long *myjw = jw + (size_t)warp * 2 * W * L;
        // warp-uniform loop: every lane runs every iteration, so the slot allocation below can
        // use full-warp ballots (one shared atomic per warp and destination)
        // PIC_UNROLL particles per thread per iteration, their loads issued together: the
        // segments sit in L2, and with 16 warps per SM one load batch at a time would leave the
        // SM waiting on L2 latency
        constexpr int U = PIC_UNROLL;
        const int iters = (np + nt * U - 1) / (nt * U);
        const int lane = tid & 31;
        const unsigned lt_mask = (1u << lane) - 1u;
        for (int it = 0; it < iters; ++it) {
            int cU[U], idU[U];
            T fU[U], uxU[U], uzU[U];
            bool vU[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int i = (it * U + u) * nt + tid;
                vU[u] = i < np;
                const size_t q = seg + (vU[u] ? i : 0);
                cU[u] = vU[u] ? cellC[q] : 0;
                fU[u] = vU[u] ? fracC[q] : T(0);
                uxU[u] = vU[u] ? uxC[q] : T(0);
                uzU[u] = vU[u] ? uzC[q] : T(0);
                idU[u] = vU[u] ? idC[q] : 0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
            bool valid = vU[u];
            const int c = cU[u];
            const T f = fU[u];
            if (valid && (c < c0 || c >= c1)) { atomicAdd(&s_lost, 1); valid = false; }
            // debug build: the tile's shared arrays around c (gathers c-1 .. c+2, deposits
            // c-1 .. c+2) and the particle's segment slot
            if (valid && !(FDTD_IN(c - 1 - base, L, a.status + 1) &&
                           FDTD_IN(c + 2 - base, L, a.status + 1) &&
                           FDTD_IN(seg + (size_t)((it * U + u) * nt + tid), (size_t)a.G * a.cap,
                                   a.status + 1)))
                valid = false;
            int dir = -2;  // -2: nothing to write, -1: stays, 0..2: outbox
            int cn = 0, pid = 0;
            Moved<T> m;
            if (valid) {
                int j;
                T fh;
                if (f >= T(0.5)) { j = c; fh = f - T(0.5); } else { j = c - 1; fh = f + T(0.5); }
                const T E = (T(1) - f) * ex[c - base] + f * ex[c + 1 - base];
                const T H = (T(1) - fh) * (T(0.5) * (hy[j - base] + hyp[j - base])) +
                            fh * (T(0.5) * (hy[j + 1 - base] + hyp[j + 1 - base]));
                particle_step<T>(E, H, c, f, uxU[u], uzU[u], a.kE, a.kH, a.sc, a.kJ, m);
                long long v[W];
                Fix<T>::split(m.jx0, a.jscale, a.jscale_f, v);
#pragma unroll
                for (int w = 0; w < W; ++w) smem_add_u64(myjw + (size_t)w * L + (m.nx0 - base), (unsigned long long)v[w]);
                Fix<T>::split(m.jx1, a.jscale, a.jscale_f, v);
#pragma unroll
                for (int w = 0; w < W; ++w) smem_add_u64(myjw + (size_t)w * L + (m.nx0 + 1 - base), (unsigned long long)v[w]);
                if (last) {  // Jz (a diagnostic) only on the call's last step
                    const MovedJz<T> z = particle_jz<T>(c, f, m, a.kJz);
                    Fix<T>::split(z.jzA, a.jscale, a.jscale_f, v);
#pragma unroll
                    for (int w = 0; w < W; ++w) smem_add_u64(myjw + (size_t)(W + w) * L + (z.nzA - base), (unsigned long long)v[w]);
                    if (z.nzB >= 0) {
                        Fix<T>::split(z.jzB, a.jscale, a.jscale_f, v);
#pragma unroll
                        for (int w = 0; w < W; ++w) smem_add_u64(myjw + (size_t)(W + w) * L + (z.nzB - base), (unsigned long long)v[w]);
                    }
                }
                cn = m.c1;
                if (cn >= a.chi) cn -= Lc;
                else if (cn < a.clo) cn += Lc;
                dir = -1;
                if (cn < c0 || cn >= c1) {
                    const int dt_ = tile_of(cn, a.G, n);
                    if (dt_ == b + 1) dir = 0;
                    else if (dt_ == b - 1) dir = 1;
                    else if (dt_ == partner) dir = 2;
                    else { atomicCAS(&s_err, 0, FDTDPIC_ERR_ARG); dir = -2; }
                }
                pid = idU[u];
            }
            // stayers: one ballot and one shared atomic per warp; movers (a few per step) take
            // the general per-direction loop
            const unsigned stay_mk = __ballot_sync(0xffffffffu, dir == -1);
            const unsigned move_mk = __ballot_sync(0xffffffffu, dir >= 0);
            if (stay_mk) {
                const int leader = __ffs(stay_mk) - 1;
                int slot0 = 0;
                if (lane == leader) slot0 = atomicAdd(&s_nstay, __popc(stay_mk));
                slot0 = __shfl_sync(0xffffffffu, slot0, leader);
                if (dir == -1) {
                    const int o = slot0 + __popc(stay_mk & lt_mask);
                    if (o < a.cap) {
                        const size_t r = seg + o;
                        cellN[r] = cn; fracN[r] = m.f1; uxN[r] = m.ux; uzN[r] = m.uz; idN[r] = pid;
                    } else {
                        atomicCAS(&s_err, 0, FDTDPIC_ERR_OOM);
                    }
                }
            }
            if (move_mk) {
                for (int d = 0; d < MIG_DIRS; ++d) {
                    const unsigned mk = __ballot_sync(0xffffffffu, dir == d);
                    if (mk == 0u) continue;
                    const int leader = __ffs(mk) - 1;
                    int slot0 = 0;
                    if (lane == leader) slot0 = atomicAdd(&s_nout[d], __popc(mk));
                    slot0 = __shfl_sync(0xffffffffu, slot0, leader);
                    if (dir != d) continue;
                    const int o = slot0 + __popc(mk & lt_mask);
                    if (o >= a.mig_cap) { atomicCAS(&s_err, 0, FDTDPIC_ERR_OOM); continue; }
                    const size_t r = (((size_t)par * a.G + b) * MIG_DIRS + d) * a.mig_cap + o;
                    a.mcell[r] = cn; a.mfrac[r] = m.f1; a.mux[r] = m.ux; a.muz[r] = m.uz;
                    a.mid[r] = pid;
                }
            }
            }  // u
        }
        __syncthreads();
        // tile sums of the per-warp deposits (exact, any order), then clear the warp copies
        for (int i = tid; i < 2 * W * L; i += nt) {
            unsigned long long acc = 0ull;
            for (int wp = 0; wp < TILE_WARPS; ++wp) {
                acc += jw[(size_t)wp * 2 * W * L + i];
                jw[(size_t)wp * 2 * W * L + i] = 0ull;
            }
            jt[i] = acc;
        }
        __syncthreads();
        // ---------------- round A: halo deposits and migrant counts ----------------
        if (tid < W) {
            unsigned long long *h = a.jhalo + (size_t)b * 5 * W;
            h[0 * W + tid] = jt[(size_t)tid * L + 0];                  // Jx at c0-1 (left)
            h[1 * W + tid] = jt[(size_t)(W + tid) * L + 0];            // Jz at c0-1 (left)
            h[2 * W + tid] = jt[(size_t)tid * L + (c1 - base)];        // Jx at c1 (right)
            h[3 * W + tid] = jt[(size_t)tid * L + (c1 + 1 - base)];    // Jx at c1+1 (right)
            h[4 * W + tid] = jt[(size_t)(W + tid) * L + (c1 - base)];  // Jz at c1 (right)
        }
        if (tid < MIG_DIRS)
            a.migcount[((size_t)par * a.G + b) * MIG_DIRS + tid] = min(s_nout[tid], a.mig_cap);
        if (tid == 0 && s_err) atomicCAS(a.abort, 0, s_err);
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            st_release(myflags + 0, target);
            bool ok = true;
            if (has_left) ok = ok && tile_wait(a.flags + (size_t)(b - 1) * 64, target, a.abort, deadline);
            if (has_right) ok = ok && tile_wait(a.flags + (size_t)(b + 1) * 64, target, a.abort, deadline);
            if (partner >= 0) ok = ok && tile_wait(a.flags + (size_t)partner * 64, target, a.abort, deadline);
            if (!ok || *(volatile int32_t *)a.abort) s_err = max(1, s_err);
        }
        __syncthreads();
        if (s_err) break;
        // neighbours' deposits on my nodes
        if (tid < W) {
            if (has_left) {
                const unsigned long long *h = a.jhalo + (size_t)(b - 1) * 5 * W;
                jt[(size_t)tid * L + (c0 - base)] += h[2 * W + tid];
                jt[(size_t)tid * L + (c0 + 1 - base)] += h[3 * W + tid];
                jt[(size_t)(W + tid) * L + (c0 - base)] += h[4 * W + tid];
            }
            if (has_right) {
                const unsigned long long *h = a.jhalo + (size_t)(b + 1) * 5 * W;
                jt[(size_t)tid * L + (c1 - 1 - base)] += h[0 * W + tid];
                jt[(size_t)(W + tid) * L + (c1 - 1 - base)] += h[1 * W + tid];
            }
        }
        // adopt migrants into the next segment after the stayers
        {
            const int nst = min(s_nstay, a.cap);
            const int srcs[3] = {has_left ? b - 1 : -1, has_right ? b + 1 : -1, partner};
            const int dirs[3] = {0, 1, 2};
            int off = nst;
            for (int s3 = 0; s3 < 3; ++s3) {
                const int src = srcs[s3];
                if (src < 0) continue;
                const int cnt = a.migcount[((size_t)par * a.G + src) * MIG_DIRS + dirs[s3]];
                for (int i = tid; i < cnt; i += nt) {
                    const int o = off + i;
                    if (o >= a.cap) { atomicCAS(&s_err, 0, FDTDPIC_ERR_OOM); break; }
                    const size_t r = (((size_t)par * a.G + src) * MIG_DIRS + dirs[s3]) * a.mig_cap + i;
                    const size_t d = seg + o;
                    cellN[d] = a.mcell[r]; fracN[d] = a.mfrac[r];
                    uxN[d] = a.mux[r]; uzN[d] = a.muz[r]; idN[d] = a.mid[r];
                }
                off += cnt;
            }
            if (tid == 0) a.count[nxt * a.G + b] = min(off, a.cap);
        }
        __syncthreads();
        // ---------------- E phase ----------------
        if (tid == 0) {
            const bool src_here = I.nzsrc >= c0 - 1 && I.nzsrc <= c1 + 1;
            s_src[0] = src_here ? src_e_at<T>(I, a.f.src, t) : T(0);
            s_src[1] = src_here ? src_h_at<T>(I, a.f.src, t) : T(0);
        }
        for (int l = tid; l < L; l += nt) {
            hyp[l] = hy[l];
            const int k = base + l;
            if (k >= c0 && k < c1) jloc[l] = Fix<T>::join2(jt, (size_t)L, l, a.jinv, a.jinv_f);
        }
        __syncthreads();
        const T src_e = s_src[0], src_h = s_src[1];
        for (int k = max(c0, 1) + tid; k < c1; k += nt)
            e_cell<T>(I, sc, kr, s, k, src_e, src_h, true, jloc[k - base], gA, &nfb, true);
        __syncthreads();
        // ---------------- round B: boundary Ex ----------------
        if (tid == 0) {
            if (s_err) atomicCAS(a.abort, 0, s_err);  // e.g. a segment overflow while adopting
            T *e = a.exhalo + (size_t)b * 3;
            e[0] = ex[c0 - base];
            e[1] = (c0 + 1 < c1) ? ex[c0 + 1 - base] : T(0);
            e[2] = ex[c1 - 1 - base];
            __threadfence();
            st_release(myflags + 32, target);
            bool ok = true;
            if (has_left) ok = ok && tile_wait(a.flags + (size_t)(b - 1) * 64 + 32, target, a.abort, deadline);
            if (has_right) ok = ok && tile_wait(a.flags + (size_t)(b + 1) * 64 + 32, target, a.abort, deadline);
            if (!ok) s_err = max(1, s_err);
            if (ok && has_left) ex[c0 - 1 - base] = a.exhalo[(size_t)(b - 1) * 3 + 2];
            if (ok && has_right) {
                ex[c1 - base] = a.exhalo[(size_t)(b + 1) * 3 + 0];
                ex[c1 + 1 - base] = a.exhalo[(size_t)(b + 1) * 3 + 1];
            }
        }
        __syncthreads();
        if (s_err) break;
        // ---------------- H phase (own cells and the two halo cells) ----------------
        {
            const int klo = max(has_left ? c0 - 1 : c0, 1);
            const int khi = min(has_right ? c1 + 1 : c1, n - 1);
            for (int k = klo + tid; k < khi; k += nt) h_cell<T>(I, sc, s, k, src_h);
            if (tid == 0) {
                const int jt_ = I.nzsrc - 1;
                if (I.tfsf && (jt_ <= 0 || jt_ >= I.nz) && jt_ >= c0 - 1 && jt_ <= c1) tfsf_edge<T>(I, s, src_h);
            }
        }
        // probes and snapshots of my cells (Ex is final for the step)
        if (tid < 2 && t >= I.probe_lo[tid] && t <= I.probe_hi[tid] && I.probe_cell[tid] >= c0 &&
            I.probe_cell[tid] < c1)
            a.f.probe[I.probe_offset + (int64_t)t * 2 + tid] = ex[I.probe_cell[tid] - base];
        if (a.f.hist && I.hist_interval > 0 && t > 0 && (t % I.hist_interval) == 0) {
            const int row = t / I.hist_interval;
            if (row < I.hist_rows)
                for (int k = c0 + tid; k < c1; k += nt) a.f.hist[I.hist_offset + (int64_t)row * n + k] = ex[k - base];
        }
        if (t == I.step_end - 1) {
            for (int l = tid; l < L; l += nt) {
                const int k = base + l;
                if (k >= c0 && k < c1) {
                    a.jx_out[k] = jloc[l];
                    a.jz_out[k] = Fix<T>::join2(jt + (size_t)W * L, (size_t)L, l, a.jinv, a.jinv_f);
                }
            }
        }
        cur = nxt;
        __syncthreads();
    }

    // ---- write back my cells
    T *gw = a.f.state + I.state_offset;
    bool bad = false;
    for (int k = c0 + tid; k < c1; k += nt) {
        const int l = k - base, i = k - c0;
        gw[(int64_t)FDTD_ST_EX * n + k] = ex[l];
        gw[(int64_t)FDTD_ST_HY * n + k] = hy[l];
        a.hyp_out[k] = hyp[l];
        gw[(int64_t)FDTD_ST_DX * n + k] = dx[i];
        gw[(int64_t)FDTD_ST_P * n + k] = pc[i];
        gw[(int64_t)FDTD_ST_PPREV * n + k] = pp[i];
        gw[(int64_t)FDTD_ST_PSIE * n + k] = psie[i];
        gw[(int64_t)FDTD_ST_PSIH * n + k] = psih[i];
        bad |= !(isfinite((double)ex[l]) && isfinite((double)hy[l]));
    }
    if (bad) atomicOr(a.status + 1, FDTD_STATUS_NONFINITE);
    if (tid == 0) {
        if (s_lost) atomicAdd(a.status, s_lost);
        if (b == 0) *a.final_seg = cur;
    }
    if (nfb && a.f.fallbacks) atomicAdd(a.f.fallbacks, nfb);
}

// Bin the caller's particles into tile segments (segment 0) and back out.
template <typename T>
__global__ void tile_bin_kernel(int n_part, int G, int n, int cap, const int32_t *cell, const T *frac,
                                const T *ux, const T *uz, const int32_t *id, int32_t *count,
                                int32_t *scell, T *sfrac, T *sux, T *suz, int32_t *sid,
                                int32_t *status)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n_part; p += gridDim.x * blockDim.x) {
        const int c = cell[p];
        if (c < 0 || c >= n) { atomicCAS(status, 0, FDTDPIC_ERR_ARG); continue; }
        const int tb = tile_of(c, G, n);
        const int o = atomicAdd(count + tb, 1);
        if (o >= cap) { atomicCAS(status, 0, FDTDPIC_ERR_OOM); continue; }
        const size_t r = (size_t)tb * cap + o;
        scell[r] = cell[p]; sfrac[r] = frac[p]; sux[r] = ux[p]; suz[r] = uz[p]; sid[r] = id[p];
    }
}

static __global__ void tile_offsets_kernel2(const int32_t *count, const int32_t *final_seg, int G,
                                            int cap, int32_t *offs)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const int32_t *cnt = count + (size_t)(*final_seg) * G;
        int s = 0;
        for (int b = 0; b < G; ++b) { offs[b] = s; s += min(cnt[b], cap); }
        offs[G] = s;
    }
}

template <typename T>
struct TileSegs {
    int32_t *cell[2];
    T *frac[2], *ux[2], *uz[2];
    int32_t *id[2];
};

template <typename T>
__global__ void tile_unbin_kernel(int G, int cap, const int32_t *count, const int32_t *final_seg,
                                  const int32_t *offs, TileSegs<T> sg, int32_t *cell, T *frac,
                                  T *ux, T *uz, int32_t *id, int n_part, int32_t *status)
{
    const int b = blockIdx.x;
    if (b >= G) return;
    const int sgi = *final_seg;
    const int cnt = min(count[(size_t)sgi * G + b], cap), o = offs[b];
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const size_t r = (size_t)b * cap + i;
        const int d = o + i;
        if (d >= n_part) break;
        cell[d] = sg.cell[sgi][r]; frac[d] = sg.frac[sgi][r]; ux[d] = sg.ux[sgi][r];
        uz[d] = sg.uz[sgi][r]; id[d] = sg.id[sgi][r];
    }
    if (b == 0 && threadIdx.x == 0 && offs[G] != n_part) atomicAdd(status, n_part - offs[G]);
}

// abort code -> status bits (the tiled path's status word reports a timeout or an overflow)
static __global__ void tile_status_kernel(const int32_t *abort, int32_t *status)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const int e = *abort;
        if (e == FDTDPIC_ERR_TIMEOUT) atomicOr(status + 1, FDTD_STATUS_TIMEOUT);
        else if (e != 0) atomicOr(status + 1, FDTD_STATUS_OVERFLOW);
    }
}

// ---- scratch layout and launcher ---------------------------------------------------------
struct TileScratch {
    size_t count, flags, jhalo, exhalo, migcount, mcell, mfrac, mux, muz, mid;
    size_t scell[2], sfrac[2], sux[2], suz[2], sid[2], offs, abort, final_seg, total;
};

struct TileGeom {
    int G, wmax, cap, mig_cap, wrap_lo, wrap_hi;
    bool ok;
};

// Tiling for one device: one CTA per SM at most, tiles at least pml+2 cells wide (so the halo
// cells the H phase recomputes are never PML cells) and at least 8.
inline TileGeom tile_geometry(const FdtdInstance &h, const PicBeam &bm, int sms)
{
    TileGeom g{};
    const int n = h.nz + 1;
    const int wmin = (h.pml + 2 > 8) ? h.pml + 2 : 8;
    int G = n / wmin;
    if (G > sms) G = sms;
    g.ok = G >= 2 && bm.n_part >= 0 && bm.chi > bm.clo;
    if (!g.ok) return g;
    g.G = G;
    g.wmax = (n + G - 1) / G;
    const int wlo = n / G;
    const double per_cell = (double)bm.n_part / (double)(bm.chi - bm.clo);
    // segment capacities within the int arithmetic (such a beam takes the streaming path)
    const double int_room = (double)(1 << 30);
    if (2.0 * per_cell * g.wmax + 1024 > int_room || 4.0 * per_cell + 256 > int_room) {
        g.ok = false;
        return g;
    }
    g.cap = (int)(2.0 * per_cell * g.wmax) + 1024;
    g.mig_cap = (int)(4.0 * per_cell) + 256;
    g.wrap_lo = tile_of(bm.clo, G, n);
    g.wrap_hi = tile_of(bm.chi - 1, G, n);
    g.ok = wlo >= wmin;
    return g;
}

inline TileScratch tile_scratch_layout(int tsize, const TileGeom &g)
{
    TileScratch L{};
    const int W = (tsize == 8) ? 2 : 1;
    size_t o = 0;
    const size_t G = (size_t)g.G, mc = (size_t)g.mig_cap, cap = (size_t)g.cap;
    L.count = o; o = align256(o + 2 * G * 4);
    L.flags = o; o = align256(o + G * 64 * 4);
    L.jhalo = o; o = align256(o + G * 5 * W * 8);
    L.exhalo = o; o = align256(o + G * 3 * tsize);
    L.migcount = o; o = align256(o + 2 * G * MIG_DIRS * 4);
    L.mcell = o; o = align256(o + 2 * G * MIG_DIRS * mc * 4);
    L.mfrac = o; o = align256(o + 2 * G * MIG_DIRS * mc * tsize);
    L.mux = o; o = align256(o + 2 * G * MIG_DIRS * mc * tsize);
    L.muz = o; o = align256(o + 2 * G * MIG_DIRS * mc * tsize);
    L.mid = o; o = align256(o + 2 * G * MIG_DIRS * mc * 4);
    for (int sgi = 0; sgi < 2; ++sgi) {
        L.scell[sgi] = o; o = align256(o + G * cap * 4);
        L.sfrac[sgi] = o; o = align256(o + G * cap * tsize);
        L.sux[sgi] = o; o = align256(o + G * cap * tsize);
        L.suz[sgi] = o; o = align256(o + G * cap * tsize);
        L.sid[sgi] = o; o = align256(o + G * cap * 4);
    }
    L.offs = o; o = align256(o + (G + 1) * 4);
    L.abort = o; o = align256(o + 4);
    L.final_seg = o; o = align256(o + 4);
    L.total = o;
    return L;
}

template <typename T>
int launch_pic_tiled(int tsize, const FdtdInstance &h, const BatchArgs<T> &fa, const PicBeam &bm,
                     const TileGeom &g, int32_t *cell, T *frac, T *ux, T *uz, int32_t *id, T *jx,
                     T *jz, T *hyp, unsigned char *scratch, int32_t *status, FdtdPicTiming *timing,
                     cudaStream_t st)
{
    const TileScratch S = tile_scratch_layout(tsize, g);
    TileArgs<T> a;
    a.f = fa;
    a.G = g.G; a.w = g.wmax; a.clo = bm.clo; a.chi = bm.chi;
    a.wrap_lo = g.wrap_lo; a.wrap_hi = g.wrap_hi; a.cap = g.cap; a.mig_cap = g.mig_cap;
    a.kE = (T)bm.kE; a.kH = (T)bm.kH; a.sc = (T)bm.sc; a.kJ = (T)bm.kJ; a.kJz = (T)bm.kJz;
    a.jscale = bm.jscale; a.jinv = 1.0 / bm.jscale;
    a.jscale_f = (float)bm.jscale; a.jinv_f = (float)(1.0 / bm.jscale);
    TileSegs<T> sg;
    for (int i = 0; i < 2; ++i) {
        a.cell[i] = sg.cell[i] = (int32_t *)(scratch + S.scell[i]);
        a.frac[i] = sg.frac[i] = (T *)(scratch + S.sfrac[i]);
        a.ux[i] = sg.ux[i] = (T *)(scratch + S.sux[i]);
        a.uz[i] = sg.uz[i] = (T *)(scratch + S.suz[i]);
        a.id[i] = sg.id[i] = (int32_t *)(scratch + S.sid[i]);
    }
    a.count = (int32_t *)(scratch + S.count);
    a.flags = (int32_t *)(scratch + S.flags);
    a.jhalo = (unsigned long long *)(scratch + S.jhalo);
    a.exhalo = (T *)(scratch + S.exhalo);
    a.migcount = (int32_t *)(scratch + S.migcount);
    a.mcell = (int32_t *)(scratch + S.mcell);
    a.mfrac = (T *)(scratch + S.mfrac);
    a.mux = (T *)(scratch + S.mux);
    a.muz = (T *)(scratch + S.muz);
    a.mid = (int32_t *)(scratch + S.mid);
    a.jx_out = jx; a.jz_out = jz; a.hyp_out = hyp;
    a.status = status;
    a.abort = (int32_t *)(scratch + S.abort);
    a.final_seg = (int32_t *)(scratch + S.final_seg);
    // deadline for the whole run: 20 s plus 1 ms per step, far above any healthy run (a test
    // may set a shorter one, fdtdpic_set_run_deadline)
    a.timeout_ns = 20LL * 1000 * 1000 * 1000 + 1000000LL * (h.step_end - h.step_begin);
    const long long test_ns = tiled_deadline_override_ns();
    if (test_ns > 0) a.timeout_ns = test_ns;

    const int threads = 256;
    const int nz1 = h.nz + 1;
    int fblocks = (nz1 + threads - 1) / threads;
    cudaError_t e = cudaMemsetAsync(scratch + S.count, 0, S.jhalo - S.count, st);  // count + flags
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch + S.migcount, 0, S.mcell - S.migcount, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch + S.abort, 0, S.total - S.abort, st);
    if (e != cudaSuccess) return cuda_status(e);
    if (!h.resume) fdtd_global_init_kernel<T><<<fblocks, threads, 0, st>>>(fa);
    const int sblocks = bm.n_part > 0 ? (bm.n_part + threads - 1) / threads : 1;
    if (bm.n_part > 0)
        tile_bin_kernel<T><<<sblocks < 4096 ? sblocks : 4096, threads, 0, st>>>(
            bm.n_part, g.G, nz1, g.cap, cell, frac, ux, uz, id, a.count, a.cell[0], a.frac[0],
            a.ux[0], a.uz[0], a.id[0], a.abort);
    const int64_t smem = tile_smem_bytes(tsize, g.wmax);
    auto kern = pic_tiled_kernel<T>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (timing) {
        *timing = FdtdPicTiming{};
        cudaEventCreate(&ev[0]);
        cudaEventCreate(&ev[1]);
        cudaEventRecord(ev[0], st);
    }
    void *params[] = {&a};
    e = cudaLaunchCooperativeKernel((const void *)kern, dim3(g.G), dim3(TILE_THREADS), params,
                                    (size_t)smem, st);
    if (e != cudaSuccess) return cuda_status(e);
    if (timing) {
        cudaEventRecord(ev[1], st);
        cudaEventSynchronize(ev[1]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[0], ev[1]);
        timing->push_ms = ms;
        timing->steps = h.step_end - h.step_begin;
        timing->path = 2;
        cudaEventDestroy(ev[0]);
        cudaEventDestroy(ev[1]);
    }
    if (bm.n_part > 0) {
        int32_t *offs = (int32_t *)(scratch + S.offs);
        tile_offsets_kernel2<<<1, 1, 0, st>>>(a.count, a.final_seg, g.G, g.cap, offs);
        tile_unbin_kernel<T><<<g.G, 256, 0, st>>>(g.G, g.cap, a.count, a.final_seg, offs, sg, cell,
                                                   frac, ux, uz, id, bm.n_part, status);
    }
    tile_status_kernel<<<1, 1, 0, st>>>(a.abort, status);
    return cuda_status(cudaGetLastError());
}

}  // namespace fdtdpic
