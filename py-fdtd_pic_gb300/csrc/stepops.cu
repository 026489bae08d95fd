// Per-step updates of the reference's BaseFDTD11 and legacy BaseFDTD modules, one launch each.
//
// The integrators of this library fuse whole runs into a few launches; these entry points keep
// the reference's finer unit of work for callers that build their own time loop out of the
// module functions (ADE_ExUpdate, CPML_Psi_e_Update, ADE_DxUpdate, AcubicFinder,
// NonLinExUpdate, ADE_HyUpdate, CPML_Psi_m_Update, ADE_PolarisationCurrent_Ex, ADE_ExCreate
// and their legacy forms).  Each operation updates cells [lo, hi) of FP64 device arrays with the
// reference function's arithmetic in its operation order (built with -fmad=false, so products
// and sums round one by one as the reference's scalar loops do).  Every cell of a range is
// independent of the others (a cell writes only its own elements and reads neighbours of
// arrays the operation does not write), so the launch's order of cells does not matter.
#include <cuda_runtime.h>

#include "cubic.cuh"
#include "fdtdpic.h"

namespace fdtdpic {
int cuda_status(cudaError_t e);
}

namespace {

struct OpArgs {
    FdtdStepOp op;
    double *a[FDTD_STEP_OP_ARRAYS];
};

__device__ __forceinline__ double factor(const OpArgs &g, int k, int cell, double t)
{
    const int mode = g.op.fmode[k];
    if (mode == 0) return t;
    const double *arr = g.a[4 + k];
    const double v = arr ? arr[cell] : g.op.fval[k];
    return mode == 2 ? t / v : t * v;
}

__global__ void step_op_kernel(OpArgs g)
{
    const FdtdStepOp &o = g.op;
    const int k = o.lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= o.hi) return;
    double *const *a = g.a;
    switch (o.op) {
    case FDTD_OP_CURL: {
        // y = y*s + ((x[k+xa] - x[k+xb]) - j) (*|/) f0 (*|/) f1 (*|/) f2
        double t = a[1][k + o.xa] - a[1][k + o.xb];
        if (a[3]) t = t - a[3][k];
        t = factor(g, 0, k, t);
        t = factor(g, 1, k, t);
        t = factor(g, 2, k, t);
        const double y = a[2] ? a[0][k] * a[2][k] : a[0][k];
        a[0][k] = y + t;
        break;
    }
    case FDTD_OP_PSI: {
        // psi = b*psi + c*(x[k+xa] - x[k+xb]); y = y + sgn*(C*psi)
        const double psi = a[3][k] * a[0][k] + a[4][k] * (a[2][k + o.xa] - a[2][k + o.xb]);
        a[0][k] = psi;
        const double corr = a[5][k] * psi;
        a[1][k] = a[1][k] + (o.s[0] < 0.0 ? -corr : corr);
        break;
    }
    case FDTD_OP_POL:
        // y = (A*p1 + B*p2) + C*x
        a[0][k] = (o.s[0] * a[1][k] + o.s[1] * a[2][k]) + o.s[2] * a[3][k];
        break;
    case FDTD_OP_EXCREATE:
        // y = (u - v) / s
        a[0][k] = (a[1][k] - a[2][k]) / o.s[0];
        break;
    case FDTD_OP_NONLIN_EX:
        // y = Dx / (e0r + e0chi*A)
        a[0][k] = a[1][k] / (o.s[0] + o.s[1] * a[2][k]);
        break;
    case FDTD_OP_ACUBIC: {
        // d = -|Dx/eps0|^2; A = Re(roots[0]) of cub A^3 + qua A^2 + one A + d when |d| > 1e-8
        const double q = fabs(a[1][k] / o.s[0]);
        const double d = -(q * q);
        a[0][k] = (fabs(d) > 1e-8) ? fdtdpic::cubic_root0_f64(o.s[1], o.s[2], o.s[3], d) : 0.0;
        if (a[2]) a[2][k] = d;
        break;
    }
    default:
        break;
    }
}

// Arrays each operation reads or writes (bit i: slot i must be non-NULL).
unsigned required_slots(int op)
{
    switch (op) {
    case FDTD_OP_CURL: return 0x3u;
    case FDTD_OP_PSI: return 0x3Fu;
    case FDTD_OP_POL: return 0xFu;
    case FDTD_OP_EXCREATE: return 0x7u;
    case FDTD_OP_NONLIN_EX: return 0x7u;
    case FDTD_OP_ACUBIC: return 0x3u;
    default: return 0u;
    }
}

}  // namespace

extern "C" int fdtdpic_step_op_check(const FdtdStepOp *op, double *const *arrays, int64_t n)
{
    if (!op || !arrays || n < 1 || n > INT32_MAX) return FDTDPIC_ERR_ARG;
    const FdtdStepOp &o = *op;
    const unsigned need = required_slots(o.op);
    if (!need) return FDTDPIC_ERR_ARG;
    for (int i = 0; i < FDTD_STEP_OP_ARRAYS; ++i)
        if (((need >> i) & 1u) && !arrays[i]) return FDTDPIC_ERR_ARG;
    if (o.lo < 0 || o.hi > n || o.lo > o.hi) return FDTDPIC_ERR_ARG;
    if (o.op == FDTD_OP_CURL || o.op == FDTD_OP_PSI) {
        // every stencil read x[k+xa], x[k+xb] of the range stays inside the array
        const int lo_off = o.xa < o.xb ? o.xa : o.xb, hi_off = o.xa > o.xb ? o.xa : o.xb;
        if (o.xa < -1 || o.xa > 1 || o.xb < -1 || o.xb > 1) return FDTDPIC_ERR_ARG;
        if (o.hi > o.lo && ((int64_t)o.lo + lo_off < 0 || (int64_t)o.hi - 1 + hi_off >= n))
            return FDTDPIC_ERR_ARG;
    }
    if (o.op == FDTD_OP_CURL)
        for (int k = 0; k < 3; ++k)
            if (o.fmode[k] < 0 || o.fmode[k] > 2) return FDTDPIC_ERR_ARG;
    return FDTDPIC_OK;
}

extern "C" int fdtdpic_step_op(const FdtdStepOp *op, double *const *arrays, int64_t n,
                               fdtdpic_stream_t stream)
{
    const int rc = fdtdpic_step_op_check(op, arrays, n);
    if (rc != FDTDPIC_OK) return rc;
    if (op->hi == op->lo) return FDTDPIC_OK;
    OpArgs g;
    g.op = *op;
    for (int i = 0; i < FDTD_STEP_OP_ARRAYS; ++i) g.a[i] = arrays[i];
    const int threads = 256;
    const int blocks = (op->hi - op->lo + threads - 1) / threads;
    step_op_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(g);
    return fdtdpic::cuda_status(cudaGetLastError());
}

extern "C" int fdtdpic_step_op_layout(int64_t *out, int n)
{
    const int64_t v[] = {(int64_t)sizeof(FdtdStepOp),
                         (int64_t)offsetof(FdtdStepOp, op),
                         (int64_t)offsetof(FdtdStepOp, lo),
                         (int64_t)offsetof(FdtdStepOp, hi),
                         (int64_t)offsetof(FdtdStepOp, xa),
                         (int64_t)offsetof(FdtdStepOp, xb),
                         (int64_t)offsetof(FdtdStepOp, fmode),
                         (int64_t)offsetof(FdtdStepOp, fval),
                         (int64_t)offsetof(FdtdStepOp, s)};
    const int m = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n && i < m; ++i) out[i] = v[i];
    return m;
}
