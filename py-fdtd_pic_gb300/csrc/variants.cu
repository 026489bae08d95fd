// The reference's uncalled per-step variants (fdtdpic_variant_run): the first-order Mur edge
// update, the JEC polarisation current and Varin's explicit nonlinear ADE, over rows of device
// arrays.  Each cell's arithmetic is the reference function's, in its operation order (Python
// evaluates a * b * c as (a * b) * c and a + b + c as (a + b) + c); the unit is built with
// -fmad=false so each product and sum rounds on its own, as the reference's do.  The functions:
//
//   MUR1DEx                     BaseFDTD11.py:769-788
//   ADE_JxUpdate                BaseFDTD11.py:543-563
//   ADE_NonLin_Pol_Ex_Pbar      BaseFDTD11.py:567-576
//   ADE_Lin_Curr_And_Pol_Varin  BaseFDTD11.py:579-593
//   ADE_Nonlin_Q_and_G          BaseFDTD11.py:596-607
//
// Every operation but the Mur update is elementwise over a cell range: CTAs take chunks of
// VAR_SPAN cells of a row (grid x over chunks, y over rows), threads consecutive cells, so loads
// and stores are coalesced, a few long rows still spread over every SM, and the kernels run at
// the memory's pace.  Cell indices are 64-bit, so an empty range far out
// (front near INT32_MAX, which the host check lets through) cannot wrap into the row.  The Mur
// update reads and writes nine cells in the order of the reference's two loops, so one thread
// of the row's CTA does it.
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "fdtdpic.h"

namespace fdtdpic {

int cuda_status(cudaError_t e);

namespace {

constexpr int VAR_THREADS = 256;
constexpr int VAR_MAX_ARRAYS = 6;
constexpr int VAR_SPAN = 4096;  // cells per CTA chunk: a row's range spreads over many CTAs

template <typename T>
struct VarArrays {
    T *a[VAR_MAX_ARRAYS];
};

// First-order Mur update of a row (MUR1DEx).  Left loop k = 1..4 ascending reads Ex[k+1]
// before it is rewritten; the right loop k = Nz-1 down to Nz-5 reads Ex[k-1] likewise, and
// after the left loop (on grids so short that the two bands overlap it reads values the left
// loop wrote), so the row runs as the reference's loops do.
template <typename T>
__device__ void mur_row(const FdtdVariantRow &r, T *ex, const T *e2)
{
    const double m64 = (r.c0 * r.dt - r.dz) / (r.c0 * r.dt + r.dz);
    const T m = (T)m64;
    for (int k = 1; k < 5; ++k) ex[k] = e2[k + 1] + m * (ex[k + 1] - e2[k]);
    for (int k = r.nz - 1; k > r.nz - 6; --k) ex[k] = e2[k - 1] + m * (ex[k - 1] - e2[k]);
}

template <typename T>
__global__ void __launch_bounds__(VAR_THREADS) variant_kernel(int op, int n_rows,
                                                              const FdtdVariantRow *rows,
                                                              int64_t stride, VarArrays<T> v)
{
    for (int row = blockIdx.y; row < n_rows; row += gridDim.y) {
        const FdtdVariantRow r = rows[row];
        const int64_t o = (int64_t)row * stride;
        if (op == FDTD_VAR_MUR_EX) {
            if (blockIdx.x == 0 && threadIdx.x == 0) mur_row<T>(r, v.a[0] + o, v.a[1] + o);
            continue;
        }
        // this CTA's chunks of VAR_SPAN cells of the row's range, grid-stride over blockIdx.x
        const int64_t lo = (int64_t)r.front - (op == FDTD_VAR_ADE_JX ? 1 : 0), hi = r.rear;
        const int64_t first = lo + (int64_t)blockIdx.x * VAR_SPAN;
        const int64_t step = (int64_t)gridDim.x * VAR_SPAN;
        if (first >= hi) continue;
        if (op == FDTD_VAR_ADE_JX) {
            // coef = 1/(permit_0 * plasmaFreqE * omega_0E * omega_0)
            const T coef = (T)(1.0 / (((r.eps0 * r.plasma_freq) * r.omega0) * r.omega0_j));
            const T w0sq = (T)(r.omega0 * r.omega0);
            const T g_dt = (T)(r.gamma / r.dt);
            const T dt2 = (T)(r.dt * r.dt);
            T *jx = v.a[0] + o;
            const T *pc = v.a[1] + o, *p1 = v.a[2] + o, *p2 = v.a[3] + o;
            for (int64_t c0 = first; c0 < hi; c0 += step) {
                const int64_t c1 = c0 + VAR_SPAN < hi ? c0 + VAR_SPAN : hi;
                for (int64_t k = c0 + threadIdx.x; k < c1; k += blockDim.x) {
                    const T P = pc[k], P1 = p1[k], P2 = p2[k];
                    jx[k] = coef * ((w0sq * P1 + g_dt * (P - P1)) + ((P - T(2) * P1) + P2) / dt2);
                }
            }
            continue;
        }
        // Varin's constants (formed in FP64 as the reference does, then in the state type)
        const double a3 = r.alpha3;
        const T eps0 = (T)r.eps0, tchi1 = (T)r.chi1, tchi3 = (T)r.chi3, ta3 = (T)a3;
        const T one_a3 = (T)(1.0 - a3);
        const double G = (r.gamma * r.dt) / 2.0;
        const T AD = (T)((1.0 - G) / (1.0 + G));
        const T BD = (T)(((r.omega0 * r.omega0) * r.dt) / (1.0 + G));
        const double g = (r.nl_gamma * r.dt) / 2.0;
        const T ef = (T)((1.0 - g) / (1.0 + g));
        const T hf = (T)(((r.nl_omega0 * r.nl_omega0) * r.dt) / (1.0 + g));
        const T dt = (T)r.dt;
        T *a0 = v.a[0] + o, *a1 = v.a[1] + o, *a2 = v.a[2] + o;
        for (int64_t c0 = first; c0 < hi; c0 += step) {
            const int64_t c1 = c0 + VAR_SPAN < hi ? c0 + VAR_SPAN : hi;
            if (op == FDTD_VAR_VARIN_PBAR) {  // a0 Pbar3, a1 Ex, a2 Qx3
                for (int64_t k = c0 + threadIdx.x; k < c1; k += blockDim.x) {
                    const T E = a1[k], Q = a2[k];
                    a0[k] = eps0 * (tchi1 * E + tchi3 * (((ta3 * E) * E) * E + (one_a3 * Q) * E));
                }
            } else if (op == FDTD_VAR_VARIN_JP) {  // a0 Jx, a1 P, a2 Pbar3
                for (int64_t k = c0 + threadIdx.x; k < c1; k += blockDim.x) {
                    const T P = a1[k];
                    const T J = AD * a0[k] + BD * (a2[k] - P);
                    a0[k] = J;
                    a1[k] = P + dt * J;
                }
            } else if (op == FDTD_VAR_VARIN_QG) {  // a0 Gx3, a1 Qx3, a2 Ex
                for (int64_t k = c0 + threadIdx.x; k < c1; k += blockDim.x) {
                    const T E = a2[k], Q = a1[k];
                    const T Gn = ef * a0[k] + hf * (E * E - Q);
                    a0[k] = Gn;
                    a1[k] = Q + dt * Gn;
                }
            } else {  // FDTD_VAR_VARIN_STEP: a0 Pbar3, a1 Jx, a2 P, a3 Gx3, a4 Qx3, a5 Ex
                T *a3p = v.a[3] + o, *a4 = v.a[4] + o;
                const T *a5 = v.a[5] + o;
                for (int64_t k = c0 + threadIdx.x; k < c1; k += blockDim.x) {
                    const T E = a5[k], Q = a4[k], P = a2[k];
                    const T pb =
                        eps0 * (tchi1 * E + tchi3 * (((ta3 * E) * E) * E + (one_a3 * Q) * E));
                    const T J = AD * a1[k] + BD * (pb - P);
                    const T Gn = ef * a3p[k] + hf * (E * E - Q);
                    a0[k] = pb;
                    a1[k] = J;
                    a2[k] = P + dt * J;
                    a3p[k] = Gn;
                    a4[k] = Q + dt * Gn;
                }
            }
        }
    }
}

int n_arrays(int op)
{
    switch (op) {
    case FDTD_VAR_MUR_EX: return 2;
    case FDTD_VAR_ADE_JX: return 4;
    case FDTD_VAR_VARIN_PBAR:
    case FDTD_VAR_VARIN_JP:
    case FDTD_VAR_VARIN_QG: return 3;
    case FDTD_VAR_VARIN_STEP: return 6;
    default: return 0;
    }
}

// Grid: x over VAR_SPAN-cell chunks of the longest row, y over rows (both grid-stride).
template <typename T>
int launch(int op, int n_rows, const FdtdVariantRow *d_rows, int64_t stride, int64_t max_n,
           void *const *arrays, cudaStream_t st)
{
    VarArrays<T> v{};
    for (int i = 0; i < n_arrays(op); ++i) v.a[i] = static_cast<T *>(arrays[i]);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FDTDPIC_ERR_NODEV;
    const int64_t chunks = op == FDTD_VAR_MUR_EX ? 1 : (max_n + VAR_SPAN - 1) / VAR_SPAN;
    const dim3 grid((unsigned)(chunks < 65535 ? (chunks > 0 ? chunks : 1) : 65535),
                    (unsigned)(n_rows < 65535 ? n_rows : 65535));
    variant_kernel<T><<<grid, VAR_THREADS, 0, st>>>(op, n_rows, d_rows, stride, v);
    return cuda_status(cudaGetLastError());
}

}  // namespace

}  // namespace fdtdpic

using namespace fdtdpic;

extern "C" int fdtdpic_variant_layout(int64_t *out, int n)
{
    const int64_t v[] = {
        (int64_t)sizeof(FdtdVariantRow),
        offsetof(FdtdVariantRow, n), offsetof(FdtdVariantRow, nz),
        offsetof(FdtdVariantRow, front), offsetof(FdtdVariantRow, rear),
        offsetof(FdtdVariantRow, c0), offsetof(FdtdVariantRow, dt), offsetof(FdtdVariantRow, dz),
        offsetof(FdtdVariantRow, eps0), offsetof(FdtdVariantRow, plasma_freq),
        offsetof(FdtdVariantRow, omega0), offsetof(FdtdVariantRow, gamma),
        offsetof(FdtdVariantRow, omega0_j), offsetof(FdtdVariantRow, chi1),
        offsetof(FdtdVariantRow, chi3), offsetof(FdtdVariantRow, alpha3),
        offsetof(FdtdVariantRow, nl_gamma), offsetof(FdtdVariantRow, nl_omega0)};
    const int m = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n && i < m; ++i) out[i] = v[i];
    return m;
}

extern "C" int fdtdpic_variant_check(int op, int n_rows, const FdtdVariantRow *h_rows,
                                     int64_t stride)
{
    if (n_arrays(op) == 0 || n_rows < 0 || (n_rows > 0 && !h_rows)) return FDTDPIC_ERR_ARG;
    for (int i = 0; i < n_rows; ++i) {
        const FdtdVariantRow &r = h_rows[i];
        if (r.n < 1 || (int64_t)r.n > stride) return FDTDPIC_ERR_ARG;
        if (op == FDTD_VAR_MUR_EX) {
            if (r.nz < 6 || r.nz > r.n) return FDTDPIC_ERR_ARG;
        } else if (op == FDTD_VAR_ADE_JX) {
            if ((int64_t)r.front - 1 < r.rear && (r.front < 1 || r.rear > r.n))
                return FDTDPIC_ERR_ARG;
        } else {
            if (r.front < r.rear && (r.front < 0 || r.rear > r.n)) return FDTDPIC_ERR_ARG;
        }
    }
    return FDTDPIC_OK;
}

extern "C" int fdtdpic_variant_run(int op, int precision, int n_rows, const FdtdVariantRow *h_rows,
                                   const FdtdVariantRow *d_rows, int64_t stride,
                                   void *const *arrays, fdtdpic_stream_t stream)
{
    if (precision != FDTDPIC_F32 && precision != FDTDPIC_F64) return FDTDPIC_ERR_ARG;
    const int rc = fdtdpic_variant_check(op, n_rows, h_rows, stride);
    if (rc != FDTDPIC_OK) return rc;
    if (n_rows == 0) return FDTDPIC_OK;
    if (!d_rows || !arrays) return FDTDPIC_ERR_ARG;
    for (int i = 0; i < n_arrays(op); ++i)
        if (!arrays[i]) return FDTDPIC_ERR_ARG;
    int64_t max_n = 0;
    for (int i = 0; i < n_rows; ++i)
        if (h_rows[i].n > max_n) max_n = h_rows[i].n;
    const cudaStream_t st = (cudaStream_t)stream;
    return precision == FDTDPIC_F64
               ? launch<double>(op, n_rows, d_rows, stride, max_n, arrays, st)
               : launch<float>(op, n_rows, d_rows, stride, max_n, arrays, st);
}
