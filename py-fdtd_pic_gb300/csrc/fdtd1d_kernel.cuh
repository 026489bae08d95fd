// 1D FDTD time stepping for one grid ("instance"), templated on the state type T.
//
// Step order (one step t), exactly the reference's (Solver_Engine.py:236-267 for the Kerr
// integrator, :294-370 for the Lorentz one, :167-211 for free space):
//   E phase (cell-local given the old Hy):
//     [LinLor, pol_active] P <- A*P + B*P_prev + C*Ex          ADE_PolarisationCurrent_Ex :610
//     Ex <- Ex + (Hy[k]-Hy[k-1]-Jx)*UpExMat*den_Exdz            ADE_ExUpdate :664
//     PML: psi_e <- beX*psi_e + ceX*dHy ; Ex <- Ex - Cb*psi_e     CPML_Psi_e_Update :365
//     Ex[nzsrc] += Exs[t]/Sc ; TF/SF: Hy[nzsrc-1] -= Hys[t]/Sc   Solver_Engine.py:249-252
//     slab: Dx <- Dx + dHy'*(dt/dz)*den_Exdz  (dHy' sees the TF/SF-corrected Hy)  :751
//       Kerr:   A = roots[0] of cub A^3 + qua A^2 + one A - |Dx/eps0|^2 (0 if |d|<=1e-8)
//               Ex = Dx/(eps0 Re(sqrt 1.2) + eps0 chi3 A)          :803-877
//       LinLor: Ex = (Dx - P)/eps0                                 ADE_ExCreate :713
//   H phase (cell-local given the new Ex):
//     Hy <- Hy + (Ex[k+1]-Ex[k])*UpHyMat*den_Hydz                 ADE_HyUpdate :641
//     PML: psi_h <- bmY*psi_h + cmY*dEx ; Hy <- Hy + C2*psi_h      CPML_Psi_m_Update :382
//     snapshot (vidMake) and probes (probeSim) read the final Ex of the step.
// Index ranges: Ex over [1, nz], Hy over [1, nz-1], psi_e over [1,pml) U [nz+1-pml, nz],
// psi_h over [1,pml) U [nz+1-pml, nz-1], slab [front, rear).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fdtdpic.h"
#include "cubic.cuh"

namespace fdtdpic {

// The update coefficients in the state type.  In FP32 a coefficient rounded once is the same
// error at every cell and every step: a curl coefficient off by up to 2^-24 is a wave speed off
// by as much, whose phase error grows with the distance a pulse travels (2e-5 relative on a
// pulse after 8192 steps, 90% of it a shift of the whole pulse); the Lorentz recursion's A and
// B sit within 1e-4 of 2 and -1, so their rounding moves the resonance.  The FP32 forms
// therefore keep what FP32 drops: *_lo, the rest of the curl coefficients' FP64 values (mul_c
// multiplies by the pair); e0r_rel / eps0_rel, the divisors' relative rounding; pa_m2 = A - 2
// and pb_p1 = B + 1 in FP32 (pol_next).  In FP64 they are unused and every update keeps the
// reference's operation order.
template <typename T>
struct Scal {
    T ue, ue_slab, uh, uh_slab, dtdz, eps0, pa, pb, pc, e0r, e0chi;
    T ue_lo, ue_slab_lo, uh_lo, uh_slab_lo, dtdz_lo, e0r_rel, eps0_rel, pa_m2, pb_p1;
};

template <typename T>
__device__ inline Scal<T> make_scal(const FdtdInstance &I)
{
    Scal<T> s;
    s.ue = (T)I.ue; s.ue_slab = (T)I.ue_slab; s.uh = (T)I.uh; s.uh_slab = (T)I.uh_slab;
    s.dtdz = (T)I.dtdz; s.eps0 = (T)I.eps0; s.pa = (T)I.pol_a; s.pb = (T)I.pol_b;
    s.pc = (T)I.pol_c; s.e0r = (T)I.nl_e0; s.e0chi = (T)I.nl_e0chi;
    s.ue_lo = (T)(I.ue - (double)s.ue);
    s.ue_slab_lo = (T)(I.ue_slab - (double)s.ue_slab);
    s.uh_lo = (T)(I.uh - (double)s.uh);
    s.uh_slab_lo = (T)(I.uh_slab - (double)s.uh_slab);
    s.dtdz_lo = (T)(I.dtdz - (double)s.dtdz);
    s.e0r_rel = (T)((I.nl_e0 - (double)s.e0r) / (double)s.e0r);
    s.eps0_rel = (T)((I.eps0 - (double)s.eps0) / (double)s.eps0);
    s.pa_m2 = (T)(I.pol_a - 2.0);
    s.pb_p1 = (T)(I.pol_b + 1.0);
    return s;
}

// x times a curl coefficient (hi, lo).  FP64: x * hi, the reference's product.  FP32: the fused
// x * hi + (x * lo), one rounding of the product with the coefficient's ~48-bit value.  (The
// other grouping, fl(x * hi) + x * lo, rounds back to fl(x * hi): the correction is below half
// a unit in its last place.)
__device__ __forceinline__ double mul_c(double x, double hi, double) { return x * hi; }
__device__ __forceinline__ float mul_c(float x, float hi, float lo) { return fmaf(x, hi, x * lo); }

// num / den where den is a constant of the instance plus a per-cell term: FP64 the plain
// quotient; FP32 the quotient corrected by the constant's relative rounding rel (exact to first
// order in rel, where rel <= 2^-24).
__device__ __forceinline__ double div_c(double num, double den, double) { return num / den; }
__device__ __forceinline__ float div_c(float num, float den, float rel)
{
    const float q = num / den;
    return fmaf(-q, rel, q);
}

// The Lorentz recursion P_(n+1) = A P_n + B P_(n-1) + C E_n.  FP64 in the reference's order;
// FP32 as (P_n + (P_n - P_(n-1))) + ((A - 2) P_n + (B + 1) P_(n-1) + C E_n), where A - 2 and
// B + 1 are small and carry their own FP32 precision.
template <typename T>
__device__ __forceinline__ T pol_next(const Scal<T> &c, T p, T pm2, T ex);
template <>
__device__ __forceinline__ double pol_next(const Scal<double> &c, double p, double pm2, double ex)
{
    return c.pa * p + c.pb * pm2 + c.pc * ex;
}
template <>
__device__ __forceinline__ float pol_next(const Scal<float> &c, float p, float pm2, float ex)
{
    const float small = fmaf(c.pa_m2, p, fmaf(c.pb_p1, pm2, c.pc * ex));
    return (p + (p - pm2)) + small;
}

// PML table column of cell k, or -1.
__device__ __forceinline__ int pml_col(const FdtdInstance &I, int k)
{
    if (k <= I.pml) return k;
    const int r0 = I.nz + 1 - I.pml;
    if (k >= r0) return I.pml + 1 + (k - r0);
    return -1;
}

// Kerr root in the state precision.
template <typename T>
struct Kerr;
template <>
struct Kerr<double> {
    double a, b, c;
    __device__ void setup(const FdtdInstance &I) { a = I.kerr_a; b = I.kerr_b; c = I.kerr_c; }
    __device__ double root(double dx, double eps0, int *nfb) const
    {
        const double q = fabs(dx / eps0);
        const double d = -(q * q);
        return (fabs(d) > 1e-8) ? cubic_root0_f64(a, b, c, d) : 0.0;
    }
};
template <>
struct Kerr<float> {
    KerrF32 k;
    __device__ void setup(const FdtdInstance &I) { k = kerr_f32_setup(I.kerr_a, I.kerr_b, I.kerr_c); }
    __device__ float root(float dx, float eps0, int *nfb) const
    {
        const float q = dx / eps0;
        const float d = -(q * q);
        return (fabsf(d) > 1e-8f) ? cubic_root0_f32(k, d, nfb) : 0.f;
    }
};

// The instance descriptor, copied once per CTA into shared memory.  Kernels read its fields in
// every cell update; from shared memory those reads neither travel to L2 nor alias the state
// stores (a per-thread copy would live in local memory, a reference to global memory would be
// re-read after every store).  Every thread must call it (it holds barriers).
__device__ inline void copy_instance_block(FdtdInstance &dst, const FdtdInstance &src)
{
    static_assert(sizeof(FdtdInstance) % 4 == 0, "FdtdInstance is copied as 32-bit words");
    __syncthreads();  // an earlier use of dst by this CTA is finished
    const int *s = reinterpret_cast<const int *>(&src);
    int *d = reinterpret_cast<int *>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(FdtdInstance) / 4); i += blockDim.x) d[i] = s[i];
    __syncthreads();
}

__device__ inline const FdtdInstance &instance_block(const FdtdInstance &src)
{
    __shared__ FdtdInstance s_inst;
    copy_instance_block(s_inst, src);
    return s_inst;
}

// Per-launch set-up done once per CTA instead of once per thread: the Kerr constants (folded in
// FP64, whose pipe is narrow) and the step's source values.  Every thread of the CTA must call
// these (they hold a barrier).
template <typename T>
__device__ inline void kerr_setup_block(Kerr<T> &kr, const FdtdInstance &I)
{
    __shared__ Kerr<T> s_kr;
    __syncthreads();  // an earlier use of s_kr by this CTA is finished
    if (threadIdx.x == 0) s_kr.setup(I);
    __syncthreads();
    kr = s_kr;
}

// make_scal's FP64 -> T conversions also run on the FP64 pipe: once per CTA.
template <typename T>
__device__ inline Scal<T> scal_block(const FdtdInstance &I)
{
    __shared__ Scal<T> s_c;
    __syncthreads();
    if (threadIdx.x == 0) s_c = make_scal<T>(I);
    __syncthreads();
    return s_c;
}

// Source values of step t in T, (T)(Exs[t]/Sc) and (T)(Hys[t]/Sc) (TF/SF only), from the
// precomputed quotients when the descriptor has them (srcs_offset >= 0), else divided here.
// pool: the source pool (the instance's offsets index it).
template <typename T>
__device__ __forceinline__ T src_e_at(const FdtdInstance &I, const double *pool, int t)
{
    return I.srcs_offset >= 0 ? (T)pool[I.srcs_offset + t] : (T)(pool[I.src_offset + t] / I.sc);
}

template <typename T>
__device__ __forceinline__ T src_h_at(const FdtdInstance &I, const double *pool, int t)
{
    if (!I.tfsf) return T(0);
    return I.srcs_offset >= 0 ? (T)pool[I.srcs_offset + I.n_steps + t]
                              : (T)(pool[I.src_offset + I.n_steps + t] / I.sc);
}

template <typename T>
__device__ inline void source_block(const FdtdInstance &I, const double *pool, int t, T &src_e,
                                    T &src_h)
{
    __shared__ T s_v[2];
    __syncthreads();
    if (threadIdx.x == 0) {
        s_v[0] = src_e_at<T>(I, pool, t);
        s_v[1] = src_h_at<T>(I, pool, t);
    }
    __syncthreads();
    src_e = s_v[0];
    src_h = s_v[1];
}

// ---------------------------------------------------------------------------------------
// storage back ends: shared-memory resident (compact) and global (full-length arrays)
// ---------------------------------------------------------------------------------------
template <typename T>
struct SmemStore {
    T *ex, *hy, *dx, *p, *pp, *psie, *psih, *tab;
    int front, W;
    __device__ T &Ex(int k) { return ex[k]; }
    __device__ T &Hy(int k) { return hy[k]; }
    __device__ T ExR(int k) { return ex[k]; }  // reads of the field the phase does not write
    __device__ T HyR(int k) { return hy[k]; }
    __device__ T &Dx(int k) { return dx[k - front]; }
    __device__ T &P(int k) { return p[k - front]; }
    __device__ T &Pp(int k) { return pp[k - front]; }
    __device__ T &PsiE(int col, int) { return psie[col]; }
    __device__ T &PsiH(int col, int) { return psih[col]; }
    __device__ T tab_at(int row, int col) const { return tab[row * W + col]; }
};

// NC: the kernel holding this store runs one phase only, so the field it reads with ExR/HyR
// (Ex in the H phase, Hy in the E phase) is read-only for the whole launch and may go through
// the non-coherent path; such loads also need not wait behind the phase's own stores.
template <typename T, bool NC = false>
struct GlobalStore {
    T *ex, *hy, *dx, *p, *pp, *psie, *psih;
    const double *tab;
    int W;
    __device__ T &Ex(int k) { return ex[k]; }
    __device__ T &Hy(int k) { return hy[k]; }
    __device__ T ExR(int k) const { return NC ? __ldg(ex + k) : ex[k]; }
    __device__ T HyR(int k) const { return NC ? __ldg(hy + k) : hy[k]; }
    __device__ T &Dx(int k) { return dx[k]; }
    __device__ T &P(int k) { return p[k]; }
    __device__ T &Pp(int k) { return pp[k]; }
    __device__ T &PsiE(int, int k) { return psie[k]; }
    __device__ T &PsiH(int, int k) { return psih[k]; }
    __device__ T tab_at(int row, int col) const { return (T)tab[row * W + col]; }
};

// One cell's state in registers, for the grid-stride field kernels: a thread issues the loads
// of several cells (FIELD_UE in the E phase, FIELD_U in the H phase) before it updates any of
// them (the loads are in flight together), then runs
// e_cell / h_cell on the register copies and stores what the update changed.  The same e_cell /
// h_cell arithmetic as the global-memory store.
constexpr int FIELD_U = 8;   // H phase
constexpr int FIELD_UE = 2;  // E phase (the Kerr solve holds more registers)
template <typename T>
struct RegE {
    T ex, hk, hkm, dx, p, pp, psi;
    const double *tab;
    int k, W;
    __device__ T &Ex(int) { return ex; }
    __device__ T HyR(int kk) const { return kk == k ? hk : hkm; }
    __device__ T &Dx(int) { return dx; }
    __device__ T &P(int) { return p; }
    __device__ T &Pp(int) { return pp; }
    __device__ T &PsiE(int, int) { return psi; }
    __device__ T tab_at(int row, int col) const { return (T)tab[row * W + col]; }
};
template <typename T>
struct RegH {
    T hy, exk, exk1, psi;
    const double *tab;
    int k, W;
    __device__ T &Hy(int) { return hy; }
    __device__ T ExR(int kk) const { return kk == k ? exk : exk1; }
    __device__ T &PsiH(int, int) { return psi; }
    __device__ T tab_at(int row, int col) const { return (T)tab[row * W + col]; }
};
// Which state cell k's updates touch besides Ex and Hy (e_cell / h_cell's conditions).
struct CellUse {
    bool dx, p, pp_w, psie, psih;
};
__device__ __forceinline__ CellUse cell_use(const FdtdInstance &I, int k)
{
    const int n = I.nz + 1;
    const bool slab = k >= I.front && k < I.rear;
    CellUse u;
    u.dx = slab && I.mode != FDTD_MODE_FREESPACE;
    u.p = slab && I.mode == FDTD_MODE_LINLOR;       // P read (both passes), P_prev too
    u.pp_w = u.p && I.pol_active;                    // P and P_prev written
    u.psie = (I.cpml_lo && k < I.pml) || (I.cpml_hi && k >= n - I.pml);
    u.psih = (I.cpml_lo && k < I.pml) || (I.cpml_hi && k >= n - I.pml && k < n - 1);
    return u;
}

// Interior cells -- outside the PML columns of the table (pml < k < nz + 1 - pml) and not the
// source cells nzsrc - 1, nzsrc -- have den = 1 and none of the PML, source or TF/SF terms, so
// their E and H updates reduce to a few operations (the same operations, in the same order, as
// e_cell / h_cell: the factor den = 1 is exact).  CELL_KERR: a Kerr slab cell; CELL_VACUUM: outside
// the slab; CELL_GENERIC: anything else (e_cell / h_cell).
enum { CELL_GENERIC = 0, CELL_VACUUM = 1, CELL_KERR = 2 };
__device__ __forceinline__ int cell_kind(const FdtdInstance &I, int k)
{
    if (k <= I.pml || k >= I.nz + 1 - I.pml || k == I.nzsrc || k == I.nzsrc - 1) return CELL_GENERIC;
    if (k < I.front || k >= I.rear) return CELL_VACUUM;
    return I.mode == FDTD_MODE_KERR ? CELL_KERR : CELL_GENERIC;
}

// E phase for cell k in [1, nz].  src_e = Exs[t]/Sc, src_h = Hys[t]/Sc in T.
// has_jx/jxv: the beam's grid current at cell k, entering the Ex update as the reference's -Jx
// term and, with the beam on, the slab's Dx update too (dx_jx).
template <typename T, class S>
__device__ __forceinline__ void e_cell(const FdtdInstance &I, const Scal<T> &c, const Kerr<T> &kr,
                                       S &s, int k, T src_e, T src_h, bool has_jx, T jxv,
                                       T *a_out, int *nfb, bool dx_jx = false)
{
    const int n = I.nz + 1;
    const T hk = s.HyR(k), hkm = s.HyR(k - 1);
    T ex = s.Ex(k);
    const bool slab = (k >= I.front) && (k < I.rear);
    if (I.mode == FDTD_MODE_LINLOR && I.pol_active && slab) {
        const T pm2 = s.Pp(k);
        const T pcur = s.P(k);
        s.Pp(k) = pcur;
        s.P(k) = pol_next<T>(c, pcur, pm2, ex);
    }
    const int col = pml_col(I, k);
    const T den = (col >= 0) ? s.tab_at(FDTD_TAB_DENE, col) : T(1);
    const bool fs_slab = I.mode == FDTD_MODE_FREESPACE && slab;
    const T up = fs_slab ? c.ue_slab : c.ue;
    const T up_lo = fs_slab ? c.ue_slab_lo : c.ue_lo;
    T dh = hk - hkm;
    if (has_jx) dh = dh - jxv;
    ex = ex + mul_c(dh, up, up_lo) * den;
    if ((I.cpml_lo && k < I.pml) || (I.cpml_hi && k >= n - I.pml)) {
        T &psi = s.PsiE(col, k);
        psi = s.tab_at(FDTD_TAB_BEX, col) * psi + s.tab_at(FDTD_TAB_CEX, col) * (hk - hkm);
        ex = ex - s.tab_at(FDTD_TAB_CB, col) * psi;
    }
    if (k == I.nzsrc) ex += src_e;
    if (I.mode != FDTD_MODE_FREESPACE && slab) {
        T hk_d = hk, hkm_d = hkm;
        if (I.tfsf) {
            if (k == I.nzsrc - 1) hk_d = hk - src_h;
            if (k == I.nzsrc) hkm_d = hkm - src_h;
        }
        T dhd = hk_d - hkm_d;
        if (dx_jx && has_jx) dhd = dhd - jxv;
        const T dx = s.Dx(k) + mul_c(dhd, c.dtdz, c.dtdz_lo) * den;
        s.Dx(k) = dx;
        if (I.mode == FDTD_MODE_KERR) {
            const T A = kr.root(dx, c.eps0, nfb);
            if (a_out) a_out[k] = A;
            ex = div_c(dx, c.e0r + c.e0chi * A, c.e0r_rel);
        } else {
            ex = div_c(dx - s.P(k), c.eps0, c.eps0_rel);
        }
    }
    s.Ex(k) = ex;
}

// H phase for cell k in [1, nz-1].
template <typename T, class S>
__device__ __forceinline__ void h_cell(const FdtdInstance &I, const Scal<T> &c, S &s, int k,
                                       T src_h)
{
    const int n = I.nz + 1;
    T hy = s.Hy(k);
    if (I.tfsf && k == I.nzsrc - 1) hy = hy - src_h;
    const T exk = s.ExR(k), exk1 = s.ExR(k + 1);
    const bool slab = (k >= I.front) && (k < I.rear);
    const int col = pml_col(I, k);
    const T den = (col >= 0) ? s.tab_at(FDTD_TAB_DENH, col) : T(1);
    const bool fs_slab = I.mode == FDTD_MODE_FREESPACE && slab;
    const T uh = fs_slab ? c.uh_slab : c.uh;
    const T uh_lo = fs_slab ? c.uh_slab_lo : c.uh_lo;
    hy = hy + mul_c(exk1 - exk, uh, uh_lo) * den;
    if ((I.cpml_lo && k < I.pml) || (I.cpml_hi && k >= n - I.pml && k < n - 1)) {
        T &psi = s.PsiH(col, k);
        psi = s.tab_at(FDTD_TAB_BMY, col) * psi + s.tab_at(FDTD_TAB_CMY, col) * (exk1 - exk);
        hy = hy + s.tab_at(FDTD_TAB_C2, col) * psi;
    }
    s.Hy(k) = hy;
}

// The TF/SF correction for a cell the H loop does not visit (nzsrc-1 == 0 or >= nz).
template <typename T, class S>
__device__ __forceinline__ void tfsf_edge(const FdtdInstance &I, S &s, T src_h)
{
    const int j = I.nzsrc - 1;
    if (I.tfsf && (j <= 0 || j >= I.nz) && j >= 0 && j <= I.nz) s.Hy(j) = s.Hy(j) - src_h;
}

template <typename T>
struct BatchArgs {
    int n_inst;
    const FdtdInstance *inst;
    const int32_t *order;
    const double *pml_tab;
    const double *src;
    T *state;
    T *probe;
    T *hist;
    int32_t *queue;
    int32_t *status;
    int32_t *fallbacks;
    int64_t smem_bytes;
};

template <typename T>
__host__ __device__ inline int64_t resident_elems(const FdtdInstance &I)
{
    const int64_t n = (int64_t)I.nz + 1;
    const int64_t S = (I.mode == FDTD_MODE_FREESPACE) ? 0 : (int64_t)(I.rear - I.front);
    const int64_t nslab = (I.mode == FDTD_MODE_LINLOR) ? 3 : (I.mode == FDTD_MODE_KERR ? 1 : 0);
    const int64_t W = 2 * (int64_t)I.pml + 1;
    return 2 * n + nslab * (S > 0 ? S : 0) + 2 * W + FDTD_TAB_ROWS * W;
}

// One instance, all requested steps, fields resident in shared memory.  I is the instance's
// descriptor (offsets into the args' buffers); idx indexes the status/fallback words.
template <typename T>
__device__ void run_instance_resident(const BatchArgs<T> &args, const FdtdInstance &I, int idx,
                                      T *smem)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    const int n = I.nz + 1;
    const int W = 2 * I.pml + 1;
    const int S = (I.mode == FDTD_MODE_FREESPACE) ? 0 : (I.rear - I.front);
    T *gst = args.state + I.state_offset;
    T *gEx = gst + (int64_t)FDTD_ST_EX * n, *gHy = gst + (int64_t)FDTD_ST_HY * n;
    T *gDx = gst + (int64_t)FDTD_ST_DX * n, *gP = gst + (int64_t)FDTD_ST_P * n;
    T *gPp = gst + (int64_t)FDTD_ST_PPREV * n, *gPsiE = gst + (int64_t)FDTD_ST_PSIE * n;
    T *gPsiH = gst + (int64_t)FDTD_ST_PSIH * n, *gA = gst + (int64_t)FDTD_ST_A * n;

    SmemStore<T> s;
    T *q = smem;
    s.ex = q; q += n;
    s.hy = q; q += n;
    s.dx = q; q += (I.mode != FDTD_MODE_FREESPACE) ? S : 0;
    s.p = q; q += (I.mode == FDTD_MODE_LINLOR) ? S : 0;
    s.pp = q; q += (I.mode == FDTD_MODE_LINLOR) ? S : 0;
    s.psie = q; q += W;
    s.psih = q; q += W;
    s.tab = q;
    s.front = I.front;
    s.W = W;

    const double *tab = args.pml_tab + I.pml_offset;
    for (int i = tid; i < FDTD_TAB_ROWS * W; i += nt) s.tab[i] = (T)tab[i];
    // initial state
    if (I.resume) {
        for (int k = tid; k < n; k += nt) { s.ex[k] = gEx[k]; s.hy[k] = gHy[k]; }
        for (int j = tid; j < S; j += nt) {
            s.dx[j] = gDx[I.front + j];
            if (I.mode == FDTD_MODE_LINLOR) { s.p[j] = gP[I.front + j]; s.pp[j] = gPp[I.front + j]; }
        }
        for (int cidx = tid; cidx < W; cidx += nt) {
            const int k = (cidx <= I.pml) ? cidx : (n - I.pml + (cidx - I.pml - 1));
            s.psie[cidx] = gPsiE[k];
            s.psih[cidx] = gPsiH[k];
        }
    } else {
        for (int k = tid; k < n; k += nt) { s.ex[k] = T(0); s.hy[k] = T(0); }
        for (int j = tid; j < S; j += nt) {
            s.dx[j] = T(0);
            if (I.mode == FDTD_MODE_LINLOR) { s.p[j] = T(0); s.pp[j] = T(0); }
        }
        for (int cidx = tid; cidx < W; cidx += nt) { s.psie[cidx] = T(0); s.psih[cidx] = T(0); }
        if (I.mode == FDTD_MODE_KERR)
            for (int k = tid; k < n; k += nt) gA[k] = T(0);
    }
    __syncthreads();

    const Scal<T> c = make_scal<T>(I);
    Kerr<T> kr;
    kr.setup(I);
    T *probe = args.probe + I.probe_offset;
    T *hist = args.hist ? args.hist + I.hist_offset : nullptr;
    int nfb = 0;
    // Source values of step t, (T)(Exs[t]/Sc) and (T)(Hys[t]/Sc): one thread divides (in FP64)
    // one step ahead into a double buffer that the step-closing barrier publishes.
    __shared__ T s_src[2][2];
    __syncthreads();  // a previous instance of this CTA may still read s_src
    if (tid == 0 && I.step_begin < I.step_end) {
        s_src[I.step_begin & 1][0] = src_e_at<T>(I, args.src, I.step_begin);
        s_src[I.step_begin & 1][1] = src_h_at<T>(I, args.src, I.step_begin);
    }
    __syncthreads();

    for (int t = I.step_begin; t < I.step_end; ++t) {
        const T src_e = s_src[t & 1][0];
        const T src_h = s_src[t & 1][1];
        T *a_out = (t == I.step_end - 1) ? gA : nullptr;
        for (int k = 1 + tid; k < n; k += nt)
            e_cell<T>(I, c, kr, s, k, src_e, src_h, false, T(0), a_out, &nfb);
        __syncthreads();
        for (int k = 1 + tid; k < n - 1; k += nt) h_cell<T>(I, c, s, k, src_h);
        if (tid == 0) tfsf_edge<T>(I, s, src_h);
        // probes and snapshots read Ex, which the H phase does not write
        if (tid < 2 && t >= I.probe_lo[tid] && t <= I.probe_hi[tid])
            probe[(int64_t)t * 2 + tid] = s.ex[I.probe_cell[tid]];
        if (hist && I.hist_interval > 0 && t > 0 && (t % I.hist_interval) == 0) {
            const int row = t / I.hist_interval;
            if (row < I.hist_rows)
                for (int k = tid; k < n; k += nt) hist[(int64_t)row * n + k] = s.ex[k];
        }
        if (tid == nt - 1 && t + 1 < I.step_end) {
            s_src[(t + 1) & 1][0] = src_e_at<T>(I, args.src, t + 1);
            s_src[(t + 1) & 1][1] = src_h_at<T>(I, args.src, t + 1);
        }
        __syncthreads();
    }

    // write back the full-length state
    bool bad = false;
    for (int k = tid; k < n; k += nt) {
        const T e = s.ex[k], h = s.hy[k];
        gEx[k] = e;
        gHy[k] = h;
        bad |= !(isfinite((double)e) && isfinite((double)h));
        const bool in_slab = (k >= I.front && k < I.rear);
        gDx[k] = (I.mode != FDTD_MODE_FREESPACE && in_slab) ? s.dx[k - I.front] : T(0);
        gP[k] = (I.mode == FDTD_MODE_LINLOR && in_slab) ? s.p[k - I.front] : T(0);
        gPp[k] = (I.mode == FDTD_MODE_LINLOR && in_slab) ? s.pp[k - I.front] : T(0);
        const int col = pml_col(I, k);
        gPsiE[k] = (col >= 0) ? s.psie[col] : T(0);
        gPsiH[k] = (col >= 0) ? s.psih[col] : T(0);
        if (I.mode != FDTD_MODE_KERR) gA[k] = T(0);
    }
    if (bad && args.status) atomicOr(args.status + idx, FDTD_STATUS_NONFINITE);
    if (nfb && args.fallbacks) atomicAdd(args.fallbacks + idx, nfb);
}

template <typename T>
__global__ void __launch_bounds__(1024) fdtd_batch_kernel(BatchArgs<T> args)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int next;
    T *smem = reinterpret_cast<T *>(smem_raw);
    while (true) {
        if (threadIdx.x == 0) next = atomicAdd(args.queue, 1);
        __syncthreads();
        const int q = next;
        __syncthreads();
        if (q >= args.n_inst) break;
        const int idx = args.order ? args.order[q] : q;
        const FdtdInstance &I = instance_block(args.inst[idx]);
        if (resident_elems<T>(I) * (int64_t)sizeof(T) > args.smem_bytes) {
            if (threadIdx.x == 0 && args.status) atomicOr(args.status + idx, FDTD_STATUS_SKIPPED);
            continue;
        }
        run_instance_resident<T>(args, I, idx, smem);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// global-memory path: one instance of any size, two launches per step
// ---------------------------------------------------------------------------------------
template <typename T, bool NC = false>
__device__ inline GlobalStore<T, NC> global_store(const FdtdInstance &I, const BatchArgs<T> &args)
{
    const int n = I.nz + 1;
    T *gst = args.state + I.state_offset;
    GlobalStore<T, NC> s;
    s.ex = gst + (int64_t)FDTD_ST_EX * n;
    s.hy = gst + (int64_t)FDTD_ST_HY * n;
    s.dx = gst + (int64_t)FDTD_ST_DX * n;
    s.p = gst + (int64_t)FDTD_ST_P * n;
    s.pp = gst + (int64_t)FDTD_ST_PPREV * n;
    s.psie = gst + (int64_t)FDTD_ST_PSIE * n;
    s.psih = gst + (int64_t)FDTD_ST_PSIH * n;
    s.tab = args.pml_tab + I.pml_offset;
    s.W = 2 * I.pml + 1;
    return s;
}

// Register copies of cell k (k < kend) for e_cell / h_cell, and the stores of what they changed.
template <typename T>
__device__ __forceinline__ void e_cell_load(const FdtdInstance &I, const GlobalStore<T, true> &s,
                                            int k, int kend, RegE<T> &r)
{
    r.tab = s.tab;
    r.W = s.W;
    r.k = k;
    const bool in = k < kend;
    const CellUse u = cell_use(I, k);
    r.hk = in ? __ldg(s.hy + k) : T(0);
    r.hkm = (in && k >= 1) ? __ldg(s.hy + k - 1) : T(0);
    r.ex = in ? s.ex[k] : T(0);
    r.dx = (in && u.dx) ? s.dx[k] : T(0);
    r.p = (in && u.p) ? s.p[k] : T(0);
    r.pp = (in && u.p) ? s.pp[k] : T(0);
    r.psi = (in && u.psie) ? s.psie[k] : T(0);
}
template <typename T>
__device__ __forceinline__ void e_cell_store(const FdtdInstance &I, GlobalStore<T, true> &s, int k,
                                             const RegE<T> &r)
{
    const CellUse u = cell_use(I, k);
    s.ex[k] = r.ex;
    if (u.dx) s.dx[k] = r.dx;
    if (u.pp_w) { s.p[k] = r.p; s.pp[k] = r.pp; }
    if (u.psie) s.psie[k] = r.psi;
}
template <typename T>
__device__ __forceinline__ void h_cell_load(const FdtdInstance &I, const GlobalStore<T, true> &s,
                                            int k, int kend, RegH<T> &r)
{
    r.tab = s.tab;
    r.W = s.W;
    r.k = k;
    const bool in = k < kend;
    r.hy = in ? s.hy[k] : T(0);
    r.exk = in ? __ldg(s.ex + k) : T(0);
    r.exk1 = in ? __ldg(s.ex + k + 1) : T(0);
    r.psi = (in && cell_use(I, k).psih) ? s.psih[k] : T(0);
}
template <typename T>
__device__ __forceinline__ void h_cell_store(const FdtdInstance &I, GlobalStore<T, true> &s, int k,
                                             const RegH<T> &r)
{
    s.hy[k] = r.hy;
    if (cell_use(I, k).psih) s.psih[k] = r.psi;
}

template <typename T>
__global__ void __launch_bounds__(256, 4) fdtd_global_e_kernel(BatchArgs<T> args, int t)
{
    const FdtdInstance &I = instance_block(args.inst[0]);
    GlobalStore<T, true> s = global_store<T, true>(I, args);
    const Scal<T> c = scal_block<T>(I);
    Kerr<T> kr;
    kerr_setup_block<T>(kr, I);
    T src_e, src_h;
    source_block<T>(I, args.src, t, src_e, src_h);
    const int n = I.nz + 1;
    T *gA = args.state + I.state_offset + (int64_t)FDTD_ST_A * n;
    const int stride = gridDim.x * blockDim.x;
    int nfb = 0;
    for (int k0 = 1 + blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += FIELD_UE * stride) {
        RegE<T> r[FIELD_UE];
#pragma unroll
        for (int u = 0; u < FIELD_UE; ++u) e_cell_load<T>(I, s, k0 + u * stride, n, r[u]);
#pragma unroll
        for (int u = 0; u < FIELD_UE; ++u) {
            const int k = k0 + u * stride;
            if (k >= n) break;
            e_cell<T>(I, c, kr, r[u], k, src_e, src_h, false, T(0), gA, &nfb);
            e_cell_store<T>(I, s, k, r[u]);
        }
    }
    if (nfb && args.fallbacks) atomicAdd(args.fallbacks, nfb);
}

template <typename T>
__global__ void __launch_bounds__(256, 4) fdtd_global_h_kernel(BatchArgs<T> args, int t)
{
    const FdtdInstance &I = instance_block(args.inst[0]);
    GlobalStore<T, true> s = global_store<T, true>(I, args);
    const Scal<T> c = scal_block<T>(I);
    const T src_h = src_h_at<T>(I, args.src, t);
    const int n = I.nz + 1;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    for (int k0 = 1 + gt; k0 < n - 1; k0 += FIELD_U * stride) {
        RegH<T> r[FIELD_U];
#pragma unroll
        for (int u = 0; u < FIELD_U; ++u) h_cell_load<T>(I, s, k0 + u * stride, n - 1, r[u]);
#pragma unroll
        for (int u = 0; u < FIELD_U; ++u) {
            const int k = k0 + u * stride;
            if (k >= n - 1) break;
            h_cell<T>(I, c, r[u], k, src_h);
            h_cell_store<T>(I, s, k, r[u]);
        }
    }
    if (gt == 0) tfsf_edge<T>(I, s, src_h);
}

// Probes and snapshots after the H phase (they read Ex only).
template <typename T>
__global__ void fdtd_global_probe_kernel(BatchArgs<T> args, int t)
{
    const FdtdInstance &I = instance_block(args.inst[0]);
    const int n = I.nz + 1;
    const T *ex = args.state + I.state_offset + (int64_t)FDTD_ST_EX * n;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    if (gt < 2 && t >= I.probe_lo[gt] && t <= I.probe_hi[gt])
        args.probe[I.probe_offset + (int64_t)t * 2 + gt] = ex[I.probe_cell[gt]];
    if (args.hist && I.hist_interval > 0 && t > 0 && (t % I.hist_interval) == 0) {
        const int row = t / I.hist_interval;
        if (row < I.hist_rows)
            for (int k = gt; k < n; k += gridDim.x * blockDim.x)
                args.hist[I.hist_offset + (int64_t)row * n + k] = ex[k];
    }
}

template <typename T>
__global__ void fdtd_global_init_kernel(BatchArgs<T> args)
{
    const FdtdInstance &I = instance_block(args.inst[0]);
    const int64_t n = (int64_t)I.nz + 1;
    T *gst = args.state + I.state_offset;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < FDTD_STATE_ARRAYS * n;
         i += (int64_t)gridDim.x * blockDim.x)
        gst[i] = T(0);
}

template <typename T>
__global__ void fdtd_global_finish_kernel(BatchArgs<T> args)
{
    const FdtdInstance &I = instance_block(args.inst[0]);
    const int n = I.nz + 1;
    const T *gst = args.state + I.state_offset;
    bool bad = false;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        bad |= !(isfinite((double)gst[k]) && isfinite((double)gst[n + k]));
    if (bad && args.status) atomicOr(args.status, FDTD_STATUS_NONFINITE);
}

}  // namespace fdtdpic
