// Temporally blocked beam path for long grids: S whole steps per launch (a "pass"), each tile's
// fields and particles held in shared memory for the whole pass.
//
// The CTA of tile b owns the cells [c0, c1) and loads [c0 - H, c1 + H) (clipped to the grid),
// H = 3 S + 4: those cells' fields from the pass's input state, its own particles, and its
// neighbours' particles within H cells of its edges.  It then runs S steps -- push with deposits
// into shared-memory currents, E phase, H phase, probes -- over everything it loaded.  Near the
// ends of the loaded range the results go wrong step by step (a cell's update reads its
// neighbours, a particle gathers from and deposits on c-1 .. c+2, particles outside the range
// are missing), but the wrong zone advances at most 3 cells a step (E reads Hy[k-1], the
// currents at k come from particles at k-2 .. k+1, H reads Ex[k+1]; particles move less than one
// cell a step), so [c0, c1) is exact after S steps: the same operations as the streaming
// kernels', hence the same bits (deposits are exact integer sums in any order).
//
// At the pass's end the CTA writes its own cells' fields to the other state buffer (double
// buffered: the neighbours still read the input state) and the particles whose cell lies in
// [c0, c1) to its segment of the other particle buffer, grouped L (cells below c0 + H), M, R
// (cells from c1 - H): a neighbour's ghosts are one group.
//
// Periodic beams: a particle that wraps at chi continues next to clo.  The tiles holding clo and
// chi - 1 are run by one CTA holding both ranges (a second launch, with twice the shared
// memory); the host takes this path only when no other tile's loaded range reaches a wrap point.
//
// HBM traffic per step: the fields and particles, read and written once a pass, over S.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_tiled.cuh"

namespace fdtdpic {

constexpr int PASS_THREADS = 512;
constexpr int PASS_GROUPS = 3;  // L, M, R
constexpr int PASS_MAX_STEPS = 32;

template <typename T>
struct PassArgs {
    BatchArgs<T> f;                 // instance, tables, source, probe, hist
    const T *st_in;                 // the instance's state block read by this pass
    T *st_out;                      // ... and the one it writes (own cells)
    const T *hyp_in;
    T *hyp_out;
    T *gA;                          // Acubic of the caller's state (the call's last step)
    int n, G, H, S, t0;
    int clo, chi;
    int wrap_lo, wrap_hi;           // tiles holding clo and chi - 1 (wrap_lo < wrap_hi)
    int capE, capM, stride;         // group capacities; segment stride = 2 capE + capM
    int pcap;                       // particles one region holds in shared memory
    int Lmax;                       // loaded cells of one region (shared-memory array length)
    T kE, kH, sc, kJ, kJz;
    double jscale, jinv;
    float jscale_f, jinv_f;
    const int32_t *cell_in;
    const T *frac_in, *ux_in, *uz_in;
    const int32_t *id_in;
    int32_t *cell_out;
    T *frac_out, *ux_out, *uz_out;
    int32_t *id_out;
    const int32_t *count_in;        // [G][3]
    int32_t *count_out;
    T *jx_out, *jz_out;
    int last_pass;                  // the call's last step ends this pass
    int32_t *status;                // [0] lost, [1] status bits
};

__host__ __device__ inline int pass_group_off(int g, int capE, int capM)
{
    return g == 0 ? 0 : (g == 1 ? capE : capE + capM);
}

// Shared-memory bytes of one CTA holding NR regions: currents (Jx, Jz words), Ex, Hy, Hyp, Dx
// per loaded cell, P and P one step back per loaded cell on Lorentz grids (lin), both psi arrays
// by PML table column (pw = 2 pml + 1 columns), the particles.
__host__ __device__ inline int64_t pass_smem_bytes(int tsize, int NR, int Lmax, int pcap, int lin,
                                                   int pw)
{
    const int W = (tsize == 8) ? 2 : 1;
    const int64_t LL = (int64_t)NR * Lmax;
    int64_t b = 2LL * W * LL * 8 + (4LL + 2 * lin) * LL * tsize + ((2LL * pw * tsize + 7) & ~7LL);
    b += (int64_t)NR * pcap * (8 + 3 * tsize);
    return (b + 15) & ~15LL;
}

// The fields of the loaded cells (cell k of region r at k - base[r]); psi by PML table column.
template <typename T, int NR>
struct PassStore {
    T *ex, *hy, *dx, *p, *pp, *psie, *psih;
    const double *tab;
    int W;
    int lo0, lo1, Lmax;
    __device__ int loc(int k) const { return (NR == 2 && k >= lo1) ? k - lo1 + Lmax : k - lo0; }
    __device__ T &Ex(int k) { return ex[loc(k)]; }
    __device__ T &Hy(int k) { return hy[loc(k)]; }
    __device__ T ExR(int k) { return ex[loc(k)]; }
    __device__ T HyR(int k) { return hy[loc(k)]; }
    __device__ T &Dx(int k) { return dx[loc(k)]; }
    __device__ T &P(int k) { return p[loc(k)]; }
    __device__ T &Pp(int k) { return pp[loc(k)]; }
    __device__ T &PsiE(int col, int) { return psie[col]; }
    __device__ T &PsiH(int col, int) { return psih[col]; }
    __device__ T tab_at(int row, int col) const { return (T)tab[row * W + col]; }
};

// NR = 1: the CTAs of every tile but the two wrap tiles; NR = 2: one CTA for both wrap tiles.
template <typename T, int NR>
__global__ void __launch_bounds__(PASS_THREADS, 2) pic_pass_kernel(PassArgs<T> a)
{
    constexpr int W = Fix<T>::W;
    extern __shared__ __align__(16) unsigned char sm_raw[];
    __shared__ int s_np, s_err, s_lost, s_nsrc;
    __shared__ int s_cnt[NR][PASS_GROUPS];
    __shared__ int s_src_off[2 * 5 + 1];
    __shared__ long long s_src_at[2 * 5];
    __shared__ T s_src[2];
    const int tid = threadIdx.x, nt = blockDim.x;
    const FdtdInstance &I = instance_block(a.f.inst[0]);
    const int n = a.n;
    const int lane = tid & 31;

    // this CTA's tiles and ranges
    int tile[2], olo[2], ohi[2], llo[2], lhi[2], base[2];
    if (NR == 2) {
        tile[0] = a.wrap_lo;
        tile[1] = a.wrap_hi;
    } else {
        int b = blockIdx.x;  // every tile but wrap_lo and wrap_hi, in order
        if (b >= a.wrap_lo) ++b;
        if (b >= a.wrap_hi) ++b;
        tile[0] = b;
        tile[1] = -1;
    }
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        olo[r] = tile_begin(tile[r], a.G, n);
        ohi[r] = tile_begin(tile[r] + 1, a.G, n);
        llo[r] = max(olo[r] - a.H, 0);
        lhi[r] = min(ohi[r] + a.H, n);
        base[r] = llo[r] - r * a.Lmax;  // local index of cell k in region r: k - base[r]
    }
    const int LL = NR * a.Lmax;

    // shared memory: currents [2W][LL] (Jx words, then Jz words), Ex, Hy, Hyp, Dx [LL] each,
    // P and P one step back [LL] each on Lorentz grids, psi_e and psi_h by PML column, particles
    unsigned long long *jw = reinterpret_cast<unsigned long long *>(sm_raw);
    T *fl = reinterpret_cast<T *>(jw + (size_t)2 * W * LL);
    T *ex = fl, *hy = fl + LL, *hyp = fl + 2 * LL, *dx = fl + 3 * LL;
    const int lin = I.mode == FDTD_MODE_LINLOR ? 1 : 0;
    T *pc = lin ? fl + 4 * LL : ex;  // (never read or written on other grids)
    T *pp = lin ? fl + 5 * LL : ex;
    const int pw = 2 * I.pml + 1;
    T *psie = fl + (4 + 2 * lin) * LL, *psih = psie + pw;
    const int pcap = NR * a.pcap;
    T *pfrac = reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(fl) +
                                     (((4LL + 2 * lin) * LL * sizeof(T) + 2LL * pw * sizeof(T) + 7) & ~7LL));
    T *pux = pfrac + pcap, *puz = pux + pcap;
    int32_t *pcell = reinterpret_cast<int32_t *>(puz + pcap);
    int32_t *pid = pcell + pcap;

    PassStore<T, NR> s;
    s.ex = ex; s.hy = hy; s.dx = dx; s.p = pc; s.pp = pp; s.psie = psie; s.psih = psih;
    s.tab = a.f.pml_tab + I.pml_offset;
    s.W = 2 * I.pml + 1;
    s.lo0 = llo[0];
    s.lo1 = NR == 2 ? llo[1] : INT_MAX;
    s.Lmax = a.Lmax;

    // ---- load: fields of the loaded cells (the arrays each cell's updates use)
    const T *gi = a.st_in;
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        for (int k = llo[r] + tid; k < lhi[r]; k += nt) {
            const int l = k - base[r];
            const CellUse u = cell_use(I, k);
            ex[l] = gi[(int64_t)FDTD_ST_EX * n + k];
            hy[l] = gi[(int64_t)FDTD_ST_HY * n + k];
            hyp[l] = a.hyp_in[k];
            dx[l] = u.dx ? gi[(int64_t)FDTD_ST_DX * n + k] : T(0);
            if (lin) {
                pc[l] = u.p ? gi[(int64_t)FDTD_ST_P * n + k] : T(0);
                pp[l] = u.p ? gi[(int64_t)FDTD_ST_PPREV * n + k] : T(0);
            }
            if (u.psie) psie[pml_col(I, k)] = gi[(int64_t)FDTD_ST_PSIE * n + k];
            if (u.psih) psih[pml_col(I, k)] = gi[(int64_t)FDTD_ST_PSIH * n + k];
#pragma unroll
            for (int w = 0; w < 2 * W; ++w) jw[(size_t)w * LL + l] = 0ull;
        }
    }
    // ---- load: particles -- per region its own three groups and the adjacent group of each
    // neighbour tile that is not one of this CTA's tiles
    if (tid == 0) {
        int ns = 0, off = 0;
        s_err = 0;
        s_lost = 0;
        for (int r = 0; r < NR; ++r) {
            const int b = tile[r];
            for (int g = 0; g < PASS_GROUPS; ++g) {
                const int cap = g == 1 ? a.capM : a.capE;
                const int c = min(a.count_in[b * PASS_GROUPS + g], cap);
                s_src_at[ns] = (long long)b * a.stride + pass_group_off(g, a.capE, a.capM);
                s_src_off[ns++] = off;
                off += c;
            }
            const int nb[2] = {b - 1, b + 1};
            const int ng[2] = {2, 0};  // the left neighbour's R group, the right one's L group
            for (int q = 0; q < 2; ++q) {
                const int o = nb[q];
                if (o < 0 || o >= a.G || o == tile[0] || (NR == 2 && o == tile[1])) continue;
                const int c = min(a.count_in[o * PASS_GROUPS + ng[q]], a.capE);
                s_src_at[ns] = (long long)o * a.stride + pass_group_off(ng[q], a.capE, a.capM);
                s_src_off[ns++] = off;
                off += c;
            }
        }
        s_src_off[ns] = off;
        s_nsrc = ns;
        if (off > pcap) {
            s_err = FDTD_STATUS_OVERFLOW;
            off = pcap;
        }
        s_np = off;
#pragma unroll
        for (int r = 0; r < NR; ++r)
            for (int g = 0; g < PASS_GROUPS; ++g) s_cnt[r][g] = 0;
        s_src[0] = T(0);
        s_src[1] = T(0);
    }
    __syncthreads();
    const int np = s_np;
    // four particles a thread per round, their loads issued before any store
    for (int q = 0; q < s_nsrc; ++q) {
        const int o0 = s_src_off[q], cnt = min(s_src_off[q + 1], pcap) - o0;
        const long long at = s_src_at[q];
        for (int i0 = 0; i0 < cnt; i0 += 4 * nt) {
            int c4[4], d4[4];
            T f4[4], x4[4], z4[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * nt + tid;
                const bool in = i < cnt;
                const long long g = at + (in ? i : 0);
                c4[u] = in ? a.cell_in[g] : 0;
                f4[u] = in ? a.frac_in[g] : T(0);
                x4[u] = in ? a.ux_in[g] : T(0);
                z4[u] = in ? a.uz_in[g] : T(0);
                d4[u] = in ? a.id_in[g] : 0;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * nt + tid;
                if (i < cnt) {
                    const int d = o0 + i;
                    pcell[d] = c4[u]; pfrac[d] = f4[u]; pux[d] = x4[u]; puz[d] = z4[u]; pid[d] = d4[u];
                }
            }
        }
    }
    const Scal<T> sc = scal_block<T>(I);
    Kerr<T> kr;
    kerr_setup_block<T>(kr, I);  // (both hold barriers: the loads above are complete)
    const int Lc = a.chi - a.clo;
    int nfb = 0, lost = 0;

    for (int st = 0; st < a.S; ++st) {
        const int t = a.t0 + st;
        const bool last = a.last_pass && st == a.S - 1;
        if (tid == 0) {
            s_src[0] = src_e_at<T>(I, a.f.src, t);
            s_src[1] = src_h_at<T>(I, a.f.src, t);
        }
        // the exact zone at the start of this step: the loaded range less 3 cells a step at each
        // end that is not a grid end (nothing is missing beyond a grid end); work outside it
        // cannot reach the own cells, so it is skipped
        int zlo[2], zhi[2];
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            zlo[r] = llo[r] == 0 ? 0 : llo[r] + 3 * st;
            zhi[r] = lhi[r] == n ? n : lhi[r] - 3 * st;
        }
        // ---------------- push ----------------
        for (int i = tid; i < np; i += nt) {
            const int c = pcell[i];
            if (c < 0) continue;
            // the region holding c (selected, not indexed: a dynamic index into the per-region
            // arrays would go through local memory)
            const bool r1 = NR == 2 && c >= llo[NR - 1];
            const int rlo = r1 ? zlo[NR - 1] : zlo[0], rhi = r1 ? zhi[NR - 1] : zhi[0];
            const int rb = r1 ? base[NR - 1] : base[0];
            // gathers read c-1 .. c+2 and deposits touch c-1 .. c+2: a particle whose cells are
            // not all in the exact zone is dropped (it can no longer reach an own cell; so are
            // particles that wrapped out of this CTA's ranges)
            if (c - 1 < rlo || c + 2 >= rhi) {
                pcell[i] = -1;
                continue;
            }
            if (c < 1 || c + 2 > I.nz) {  // off the grid (the streaming kernels skip it too)
                if (c >= (r1 ? olo[NR - 1] : olo[0]) && c < (r1 ? ohi[NR - 1] : ohi[0])) ++lost;
                pcell[i] = -1;
                continue;
            }
            const T f = pfrac[i];
            int j;
            T fh;
            if (f >= T(0.5)) { j = c; fh = f - T(0.5); } else { j = c - 1; fh = f + T(0.5); }
            const int lc = c - rb, lj = j - rb;
            const T E = (T(1) - f) * ex[lc] + f * ex[lc + 1];
            const T H = (T(1) - fh) * (T(0.5) * (hy[lj] + hyp[lj])) +
                        fh * (T(0.5) * (hy[lj + 1] + hyp[lj + 1]));
            Moved<T> m;
            particle_step<T>(E, H, c, f, pux[i], puz[i], a.kE, a.kH, a.sc, a.kJ, m);
            long long v[W];
            Fix<T>::split(m.jx0, a.jscale, a.jscale_f, v);
#pragma unroll
            for (int w = 0; w < W; ++w)
                if (v[w] != 0) smem_add_u64(jw + (size_t)w * LL + (m.nx0 - rb), (unsigned long long)v[w]);
            Fix<T>::split(m.jx1, a.jscale, a.jscale_f, v);
#pragma unroll
            for (int w = 0; w < W; ++w)
                if (v[w] != 0) smem_add_u64(jw + (size_t)w * LL + (m.nx0 + 1 - rb), (unsigned long long)v[w]);
            if (last) {  // Jz (a diagnostic) only on the call's last step
                const MovedJz<T> z = particle_jz<T>(c, f, m, a.kJz);
                Fix<T>::split(z.jzA, a.jscale, a.jscale_f, v);
#pragma unroll
                for (int w = 0; w < W; ++w)
                    if (v[w] != 0) smem_add_u64(jw + (size_t)(W + w) * LL + (z.nzA - rb), (unsigned long long)v[w]);
                if (z.nzB >= 0) {
                    Fix<T>::split(z.jzB, a.jscale, a.jscale_f, v);
#pragma unroll
                    for (int w = 0; w < W; ++w)
                        if (v[w] != 0) smem_add_u64(jw + (size_t)(W + w) * LL + (z.nzB - rb), (unsigned long long)v[w]);
                }
            }
            int cn = m.c1;
            if (cn >= a.chi) cn -= Lc;
            else if (cn < a.clo) cn += Lc;
            pcell[i] = cn;
            pfrac[i] = m.f1;
            pux[i] = m.ux;
            puz[i] = m.uz;
        }
        __syncthreads();
        const T src_e = s_src[0], src_h = s_src[1];
        // ---------------- E phase: Hyp <- Hy, currents out of the words (cleared), e_cell ----
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            for (int k = zlo[r] + tid; k < zhi[r]; k += nt) {
                const int l = k - base[r];
                hyp[l] = hy[l];
                const T jxk = Fix<T>::join2(jw, (size_t)LL, l, a.jinv, a.jinv_f);
#pragma unroll
                for (int w = 0; w < W; ++w) jw[(size_t)w * LL + l] = 0ull;
                const bool own = k >= olo[r] && k < ohi[r];
                if (k >= 1 && k > zlo[r]) {  // Ex over [1, nz]; cell k reads Hy[k-1]
                    // interior cells take e_cell's operations without its terms that vanish
                    // there (the streaming E kernel's forms: the same bits)
                    const int kd = cell_kind(I, k);
                    if (kd == CELL_VACUUM) {
                        ex[l] = ex[l] + mul_c((hy[l] - hy[l - 1]) - jxk, sc.ue, sc.ue_lo);
                    } else if (kd == CELL_KERR) {
                        const T d = dx[l] + mul_c((hy[l] - hy[l - 1]) - jxk, sc.dtdz, sc.dtdz_lo);
                        const T A = kr.root(d, sc.eps0, &nfb);
                        if (last && own) a.gA[k] = A;
                        dx[l] = d;
                        ex[l] = div_c(d, sc.e0r + sc.e0chi * A, sc.e0r_rel);
                    } else {
                        e_cell<T>(I, sc, kr, s, k, src_e, src_h, true, jxk,
                                  (last && own) ? a.gA : nullptr, &nfb, true);
                    }
                }
                if (last && own) {
                    a.jx_out[k] = jxk;
                    a.jz_out[k] = Fix<T>::join2(jw + (size_t)W * LL, (size_t)LL, l, a.jinv, a.jinv_f);
                }
            }
        }
        __syncthreads();
        // ---------------- H phase ----------------
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            const int khi = min(zhi[r] - 1, n - 1);  // Hy over [1, nz-1]; cell k reads Ex[k+1]
            for (int k = max(zlo[r], 1) + tid; k < khi; k += nt) {
                const int l = k - base[r];
                if (cell_kind(I, k) != CELL_GENERIC)  // interior: h_cell with den = 1
                    hy[l] = hy[l] + mul_c(ex[l + 1] - ex[l], sc.uh, sc.uh_lo);
                else
                    h_cell<T>(I, sc, s, k, src_h);
            }
        }
        if (tid == 0) {
            const int jt = I.nzsrc - 1;
#pragma unroll
            for (int r = 0; r < NR; ++r)
                if (I.tfsf && (jt <= 0 || jt >= I.nz) && jt >= llo[r] && jt < lhi[r])
                    tfsf_edge<T>(I, s, src_h);
        }
        __syncthreads();
        // probes and snapshots of the own cells (Ex is final for the step)
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            if (tid < 2 && t >= I.probe_lo[tid] && t <= I.probe_hi[tid] &&
                I.probe_cell[tid] >= olo[r] && I.probe_cell[tid] < ohi[r])
                a.f.probe[I.probe_offset + (int64_t)t * 2 + tid] = ex[I.probe_cell[tid] - base[r]];
            if (a.f.hist && I.hist_interval > 0 && t > 0 && (t % I.hist_interval) == 0) {
                const int row = t / I.hist_interval;
                if (row < I.hist_rows)
                    for (int k = olo[r] + tid; k < ohi[r]; k += nt)
                        a.f.hist[I.hist_offset + (int64_t)row * n + k] = ex[k - base[r]];
            }
        }
    }

    // ---- write back: own cells' fields
    T *go = a.st_out;
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        for (int k = olo[r] + tid; k < ohi[r]; k += nt) {
            const int l = k - base[r];
            const CellUse u = cell_use(I, k);
            go[(int64_t)FDTD_ST_EX * n + k] = ex[l];
            go[(int64_t)FDTD_ST_HY * n + k] = hy[l];
            a.hyp_out[k] = hyp[l];
            if (u.dx) go[(int64_t)FDTD_ST_DX * n + k] = dx[l];
            if (u.p) {
                go[(int64_t)FDTD_ST_P * n + k] = pc[l];
                go[(int64_t)FDTD_ST_PPREV * n + k] = pp[l];
            }
            if (u.psie) go[(int64_t)FDTD_ST_PSIE * n + k] = psie[pml_col(I, k)];
            if (u.psih) go[(int64_t)FDTD_ST_PSIH * n + k] = psih[pml_col(I, k)];
        }
    }
    // ---- write back: particles whose cell lies in an own range, by group; one shared atomic
    // per warp and group
    const unsigned lt_mask = (1u << lane) - 1u;
    const int iters = (np + nt - 1) / nt;
    for (int it = 0; it < iters; ++it) {
        const int i = it * nt + tid;
        int code = -1, c = -1;
        if (i < np) {
            c = pcell[i];
#pragma unroll
            for (int r = 0; r < NR; ++r)
                if (c >= olo[r] && c < ohi[r])
                    code = r * PASS_GROUPS + (c < olo[r] + a.H ? 0 : (c >= ohi[r] - a.H ? 2 : 1));
        }
#pragma unroll
        for (int q = 0; q < NR * PASS_GROUPS; ++q) {
            const unsigned mk = __ballot_sync(0xffffffffu, code == q);
            if (mk == 0u) continue;
            const int leader = __ffs(mk) - 1;
            int slot0 = 0;
            if (lane == leader) slot0 = atomicAdd(&s_cnt[q / PASS_GROUPS][q % PASS_GROUPS], __popc(mk));
            slot0 = __shfl_sync(0xffffffffu, slot0, leader);
            if (code != q) continue;
            const int g = q % PASS_GROUPS;
            const int o = slot0 + __popc(mk & lt_mask);
            const int cap = g == 1 ? a.capM : a.capE;
            if (o >= cap) {
                atomicOr(&s_err, FDTD_STATUS_OVERFLOW);
                continue;
            }
            const size_t d = (size_t)tile[q / PASS_GROUPS] * a.stride + pass_group_off(g, a.capE, a.capM) + o;
            a.cell_out[d] = c;
            a.frac_out[d] = pfrac[i];
            a.ux_out[d] = pux[i];
            a.uz_out[d] = puz[i];
            a.id_out[d] = pid[i];
        }
    }
    if (lost) atomicAdd(&s_lost, lost);
    __syncthreads();
    if (tid < NR * PASS_GROUPS) {
        const int r = tid / PASS_GROUPS, g = tid % PASS_GROUPS;
        a.count_out[tile[r] * PASS_GROUPS + g] = min(s_cnt[r][g], g == 1 ? a.capM : a.capE);
    }
    if (tid == 0) {
        if (s_err) atomicOr(a.status + 1, s_err);
        if (s_lost) atomicAdd(a.status, s_lost);
    }
    if (nfb && a.f.fallbacks) atomicAdd(a.f.fallbacks, nfb);
}

// The caller's particles into the segments (parity 0), grouped by cell; a particle outside the
// beam domain or beyond a group's capacity is counted in status[0] (the host takes this path
// only for beams inside their domain).
template <typename T>
__global__ void pass_bin_kernel(int n_part, int G, int n, int H, int capE, int capM, int stride,
                                const int32_t *cell, const T *frac, const T *ux, const T *uz,
                                const int32_t *id, int32_t *count, int32_t *scell, T *sfrac,
                                T *sux, T *suz, int32_t *sid, int32_t *status)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n_part; p += gridDim.x * blockDim.x) {
        const int c = cell[p];
        if (c < 0 || c >= n) { atomicAdd(status, 1); continue; }
        const int b = tile_of(c, G, n);
        const int c0 = tile_begin(b, G, n), c1 = tile_begin(b + 1, G, n);
        const int g = c < c0 + H ? 0 : (c >= c1 - H ? 2 : 1);
        const int o = atomicAdd(count + b * PASS_GROUPS + g, 1);
        if (o >= (g == 1 ? capM : capE)) { atomicOr(status + 1, FDTD_STATUS_OVERFLOW); continue; }
        const size_t r = (size_t)b * stride + pass_group_off(g, capE, capM) + o;
        scell[r] = c; sfrac[r] = frac[p]; sux[r] = ux[p]; suz[r] = uz[p]; sid[r] = id[p];
    }
}

// Exclusive scan of the clamped group counts (G x 3, one CTA) into offs[0 .. 3G].
static __global__ void pass_offsets_kernel(const int32_t *count, int ng, int capE, int capM,
                                           int32_t *offs)
{
    __shared__ int s_part[1024];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int per = (ng + nt - 1) / nt;
    const int i0 = tid * per, i1 = min(ng, i0 + per);
    int sum = 0;
    for (int i = i0; i < i1; ++i) sum += min(count[i], (i % PASS_GROUPS) == 1 ? capM : capE);
    s_part[tid] = sum;
    __syncthreads();
    if (tid == 0) {
        int acc = 0;
        for (int q = 0; q < nt; ++q) {
            const int v = s_part[q];
            s_part[q] = acc;
            acc += v;
        }
        offs[ng] = acc;
    }
    __syncthreads();
    int acc = s_part[tid];
    for (int i = i0; i < i1; ++i) {
        offs[i] = acc;
        acc += min(count[i], (i % PASS_GROUPS) == 1 ? capM : capE);
    }
}

// Segments back into the caller's arrays, tile by tile and group by group; a shortfall (particles
// dropped by an overflow) is counted in status[0].
template <typename T>
__global__ void pass_unbin_kernel(int G, int capE, int capM, int stride, const int32_t *count,
                                  const int32_t *offs, const int32_t *scell, const T *sfrac,
                                  const T *sux, const T *suz, const int32_t *sid, int32_t *cell,
                                  T *frac, T *ux, T *uz, int32_t *id, int n_part, int32_t *status)
{
    const int q = blockIdx.x;  // tile * 3 + group
    if (q >= G * PASS_GROUPS) return;
    const int g = q % PASS_GROUPS;
    const int cnt = min(count[q], g == 1 ? capM : capE), o = offs[q];
    const size_t at = (size_t)(q / PASS_GROUPS) * stride + pass_group_off(g, capE, capM);
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const int d = o + i;
        if (d >= n_part) break;
        cell[d] = scell[at + i]; frac[d] = sfrac[at + i]; ux[d] = sux[at + i];
        uz[d] = suz[at + i]; id[d] = sid[at + i];
    }
    if (q == 0 && threadIdx.x == 0 && offs[G * PASS_GROUPS] != n_part)
        atomicAdd(status, n_part - offs[G * PASS_GROUPS]);
}

// ---- geometry, scratch layout and launcher ------------------------------------------------
struct PassGeom {
    int G, S, H, wmin, wmax, Lmax, capE, capM, stride, pcap, wrap_lo, wrap_hi;
    int64_t smem1, smem2;
    bool ok;
};

// Tiles of about bm.chunk cells (0: 512) and bm.sort_every steps a pass (0: 8); ok=false when
// the path does not apply: a tile narrower than 2H, the wrap tiles too close to each other or
// to the wrap points, no beam, or shared memory too small.
inline PassGeom pass_geometry(int tsize, const FdtdInstance &h, const PicBeam &bm,
                              int64_t smem_optin)
{
    PassGeom g{};
    const int n = h.nz + 1;
    g.S = bm.sort_every > 0 ? bm.sort_every : 8;
    if (g.S > PASS_MAX_STEPS) g.S = PASS_MAX_STEPS;
    g.H = 3 * g.S + 4;
    const int w = bm.chunk > 0 ? bm.chunk : 512;
    g.G = n / w;
    g.ok = bm.n_part > 0 && bm.chi > bm.clo && g.G >= 5;
    if (!g.ok) return g;
    g.wmin = n / g.G;
    g.wmax = (n + g.G - 1) / g.G;
    g.Lmax = g.wmax + 2 * g.H;
    g.wrap_lo = tile_of(bm.clo, g.G, n);
    g.wrap_hi = tile_of(bm.chi - 1, g.G, n);
    const int lo0 = tile_begin(g.wrap_lo, g.G, n), lo1 = tile_begin(g.wrap_lo + 1, g.G, n);
    const int hi0 = tile_begin(g.wrap_hi, g.G, n), hi1 = tile_begin(g.wrap_hi + 1, g.G, n);
    // the wrap points sit at least H inside their tiles' own ranges (so no other tile's loaded
    // range reaches them), and the two tiles' loaded ranges are apart
    const bool lo_ok = (bm.clo - lo0 >= g.H || g.wrap_lo == 0) && lo1 - bm.clo >= g.H;
    const bool hi_ok = (hi1 - bm.chi >= g.H || g.wrap_hi == g.G - 1) && bm.chi - hi0 >= g.H;
    g.ok = g.wmin >= 2 * g.H && lo_ok && hi_ok && lo1 + g.H <= hi0 - g.H;
    if (!g.ok) return g;
    const double ppc = (double)bm.n_part / (double)(bm.chi - bm.clo);
    // capacities within the int arithmetic (far beyond what shared memory holds: such a beam
    // takes another path); H < wmax and Lmax <= 2 wmax, so these two bound all three
    const double int_room = (double)(1 << 30);
    if (2.0 * ppc * g.wmax + 1024 > int_room || 1.25 * ppc * g.Lmax + 1024 > int_room) {
        g.ok = false;
        return g;
    }
    g.capE = ((int)(2.0 * ppc * g.H) + 256 + 3) & ~3;
    g.capM = ((int)(2.0 * ppc * g.wmax) + 512 + 3) & ~3;
    g.stride = 2 * g.capE + g.capM;
    // a loaded range holds ~ppc Lmax particles; a quarter more and 256 cover the fluctuations
    // of a beam of even density (a shortfall is reported, FDTD_STATUS_OVERFLOW)
    g.pcap = ((int)(1.25 * ppc * g.Lmax) + 256 + 3) & ~3;
    const int lin = h.mode == FDTD_MODE_LINLOR ? 1 : 0;
    g.smem1 = pass_smem_bytes(tsize, 1, g.Lmax, g.pcap, lin, 2 * h.pml + 1);
    g.smem2 = pass_smem_bytes(tsize, 2, g.Lmax, g.pcap, lin, 2 * h.pml + 1);
    // 1 KiB stays for the kernel's static shared variables
    g.ok = g.smem2 <= smem_optin - 1024;
    return g;
}

struct PassScratch {
    size_t count[2], cell[2], frac[2], ux[2], uz[2], id[2], state, hyp, offs, total;
};

inline PassScratch pass_scratch_layout(int tsize, int nz, const PassGeom &g)
{
    PassScratch L{};
    const size_t G = (size_t)g.G, n = (size_t)nz + 1, seg = G * (size_t)g.stride;
    size_t o = 0;
    for (int q = 0; q < 2; ++q) {
        L.count[q] = o; o = align256(o + G * PASS_GROUPS * 4);
        L.cell[q] = o; o = align256(o + seg * 4);
        L.frac[q] = o; o = align256(o + seg * tsize);
        L.ux[q] = o; o = align256(o + seg * tsize);
        L.uz[q] = o; o = align256(o + seg * tsize);
        L.id[q] = o; o = align256(o + seg * 4);
    }
    L.state = o; o = align256(o + (size_t)FDTD_STATE_ARRAYS * n * tsize);
    L.hyp = o; o = align256(o + n * tsize);
    L.offs = o; o = align256(o + (G * PASS_GROUPS + 1) * 4);
    L.total = o;
    return L;
}

template <typename T>
int launch_pic_pass(int tsize, const FdtdInstance &h, const BatchArgs<T> &fa, const PicBeam &bm,
                    const PassGeom &g, int32_t *cell, T *frac, T *ux, T *uz, int32_t *id, T *jx,
                    T *jz, T *hyp, unsigned char *scratch, int32_t *status, FdtdPicTiming *timing,
                    cudaStream_t st)
{
    const PassScratch S = pass_scratch_layout(tsize, h.nz, g);
    const int n = h.nz + 1;
    T *stA = fa.state + h.state_offset;
    T *stB = (T *)(scratch + S.state);
    T *hypB = (T *)(scratch + S.hyp);
    PassArgs<T> a;
    a.f = fa;
    a.gA = stA + (int64_t)FDTD_ST_A * n;
    a.n = n; a.G = g.G; a.H = g.H;
    a.clo = bm.clo; a.chi = bm.chi; a.wrap_lo = g.wrap_lo; a.wrap_hi = g.wrap_hi;
    a.capE = g.capE; a.capM = g.capM; a.stride = g.stride; a.pcap = g.pcap; a.Lmax = g.Lmax;
    a.kE = (T)bm.kE; a.kH = (T)bm.kH; a.sc = (T)bm.sc; a.kJ = (T)bm.kJ; a.kJz = (T)bm.kJz;
    a.jscale = bm.jscale; a.jinv = 1.0 / bm.jscale;
    a.jscale_f = (float)bm.jscale; a.jinv_f = (float)(1.0 / bm.jscale);
    a.jx_out = jx; a.jz_out = jz;
    a.status = status;

    cudaError_t e = cudaMemsetAsync(scratch + S.count[0], 0, (size_t)g.G * PASS_GROUPS * 4, st);
    if (e != cudaSuccess) return cuda_status(e);
    const int threads = 256;
    int fblocks = (n + threads - 1) / threads;
    if (!h.resume) fdtd_global_init_kernel<T><<<fblocks, threads, 0, st>>>(fa);
    {
        const int sblocks = (bm.n_part + threads - 1) / threads;
        pass_bin_kernel<T><<<sblocks < 8192 ? sblocks : 8192, threads, 0, st>>>(
            bm.n_part, g.G, n, g.H, g.capE, g.capM, g.stride, cell, frac, ux, uz, id,
            (int32_t *)(scratch + S.count[0]), (int32_t *)(scratch + S.cell[0]),
            (T *)(scratch + S.frac[0]), (T *)(scratch + S.ux[0]), (T *)(scratch + S.uz[0]),
            (int32_t *)(scratch + S.id[0]), status);
    }
    e = cudaFuncSetAttribute(pic_pass_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)g.smem1);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(pic_pass_kernel<T, 2>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem2);
    if (e != cudaSuccess) return cuda_status(e);
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (timing) {
        *timing = FdtdPicTiming{};
        cudaEventCreate(&ev[0]);
        cudaEventCreate(&ev[1]);
        cudaEventRecord(ev[0], st);
    }
    int q = 0;  // the parity holding the current particles and state (0: caller's state)
    for (int t0 = h.step_begin; t0 < h.step_end; t0 += g.S) {
        a.t0 = t0;
        a.S = (h.step_end - t0) < g.S ? (h.step_end - t0) : g.S;
        a.last_pass = t0 + a.S == h.step_end;
        a.st_in = q ? stB : stA;
        a.st_out = q ? stA : stB;
        a.hyp_in = q ? hypB : hyp;
        a.hyp_out = q ? hyp : hypB;
        a.cell_in = (const int32_t *)(scratch + S.cell[q]);
        a.frac_in = (const T *)(scratch + S.frac[q]);
        a.ux_in = (const T *)(scratch + S.ux[q]);
        a.uz_in = (const T *)(scratch + S.uz[q]);
        a.id_in = (const int32_t *)(scratch + S.id[q]);
        a.count_in = (const int32_t *)(scratch + S.count[q]);
        a.cell_out = (int32_t *)(scratch + S.cell[q ^ 1]);
        a.frac_out = (T *)(scratch + S.frac[q ^ 1]);
        a.ux_out = (T *)(scratch + S.ux[q ^ 1]);
        a.uz_out = (T *)(scratch + S.uz[q ^ 1]);
        a.id_out = (int32_t *)(scratch + S.id[q ^ 1]);
        a.count_out = (int32_t *)(scratch + S.count[q ^ 1]);
        pic_pass_kernel<T, 1><<<g.G - 2, PASS_THREADS, (size_t)g.smem1, st>>>(a);
        pic_pass_kernel<T, 2><<<1, PASS_THREADS, (size_t)g.smem2, st>>>(a);
        q ^= 1;
    }
    if (q) {  // the run ended in the scratch buffers: copy the fields back (Acubic is in place)
        for (int arr = 0; arr < FDTD_STATE_ARRAYS && e == cudaSuccess; ++arr)
            if (arr != FDTD_ST_A)
                e = cudaMemcpyAsync(stA + (int64_t)arr * n, stB + (int64_t)arr * n,
                                    (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hyp, hypB, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_status(e);
    }
    if (timing) {
        cudaEventRecord(ev[1], st);
        cudaEventSynchronize(ev[1]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[0], ev[1]);
        timing->push_ms = ms;
        timing->steps = h.step_end - h.step_begin;
        timing->path = 4;
        cudaEventDestroy(ev[0]);
        cudaEventDestroy(ev[1]);
    }
    int32_t *offs = (int32_t *)(scratch + S.offs);
    const int32_t *cnt = (const int32_t *)(scratch + S.count[q]);
    pass_offsets_kernel<<<1, 1024, 0, st>>>(cnt, g.G * PASS_GROUPS, g.capE, g.capM, offs);
    pass_unbin_kernel<T><<<g.G * PASS_GROUPS, 256, 0, st>>>(
        g.G, g.capE, g.capM, g.stride, cnt, offs, (const int32_t *)(scratch + S.cell[q]),
        (const T *)(scratch + S.frac[q]), (const T *)(scratch + S.ux[q]),
        (const T *)(scratch + S.uz[q]), (const int32_t *)(scratch + S.id[q]), cell, frac, ux, uz,
        id, bm.n_part, status);
    pic_finish_kernel<T><<<fblocks < 1024 ? fblocks : 1024, threads, 0, st>>>(stA, n, status);
    return cuda_status(cudaGetLastError());
}

}  // namespace fdtdpic
