// Per-grid set-up on the device (fdtdpic_setup_batch): the CPML table and the update, Kerr and
// Lorentz coefficients of every instance of a ragged batch, in FP64, in the operation order of
// the host restatement (fdtdpic/physics_setup.py), which follows the reference:
//
//   UpExMat = CharImp * courantNo, UpHyMat = (1/CharImp) * courantNo; the free-space integrator
//     divides the slab's by epsRe / muRe                    (BaseFDTD11.py:124-182)
//   CPML profiles over i = 0..pml-1, mirrored on the right   (CPML_ScalingCalc, :223-272)
//     kappa = 1 + (kappaMax - 1) ((pml - i)/pml)^m,  sigma = sigmaOpt ((pml - i)/pml)^m,
//     alpha = alphaMax ((i + 1)/pml)^ma
//   beX = bmY = exp(-(sigma dt/(kappa eps0) + alpha dt/eps0))              (:275-296)
//   ceX = (beX - 1) sigma / (sigma kappa + alpha kappa^2), cmY the same / dz
//   Cb = UpExMat, C2 = dt/mu0 on [0, pml) and [Nz+2-pml, Nz] (the right loops stop one short)
//   den = 1/kappa, the right side walking kappa with its own counter  (:299-357)
//   Kerr: eps = 1 + wp^2 / (w0^2 - (2 pi f)^2 + i gamma 2 pi f), cub = (alpha3 chi3)^2,
//     qua = 2 Re(alpha3 eps chi3), one = |eps|^2                        (:795-820)
//   Lorentz ADE: D = 1/dt^2 + gamma/(2 dt), A = (2/dt^2 - w0^2)/D, B = (gamma/(2 dt) - 1/dt^2)/D,
//     C = eps0 wp^2 / D                                                (:487-538)
// Built with -fmad=false so each product and sum rounds on its own, as numpy's do.  The pow and
// exp of the profiles may differ from the host library's in the last place.
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "fdtdpic.h"

namespace fdtdpic {

int cuda_status(cudaError_t e);

namespace {

constexpr double kPi = 3.141592653589793;

// kappa, sigma, alpha of cell j (0 <= j <= nz) of a grid with n = nz + 1 cells; the right
// profile is the left one reversed and overwrites it where they overlap (tiny grids).
struct Profile {
    double kappa, sigma, alpha;
};
__device__ Profile profile(const FdtdSetup &s, int pml, int n, int j)
{
    Profile p{1.0, 0.0, 0.0};
    int i = -1;
    if (j >= n - pml) i = n - 1 - j;
    else if (j < pml) i = j;
    if (i < 0) return p;
    const double ramp = pow((double)(pml - i) / (double)pml, s.r_scale);
    p.kappa = 1.0 + (s.kappa_max - 1.0) * ramp;
    p.sigma = s.sigma_opt * ramp;
    p.alpha = s.alpha_max * pow((double)(i + 1) / (double)pml, s.r_a_scale);
    return p;
}

__global__ void setup_kernel(int n_inst, const FdtdSetup *setup, FdtdInstance *inst, double *tab)
{
    for (int g = blockIdx.x; g < n_inst; g += gridDim.x) {
        const FdtdSetup s = setup[g];
        FdtdInstance &I = inst[g];
        const int nz = I.nz, pml = I.pml, n = nz + 1;
        const bool lo = I.cpml_lo != 0, hi = I.cpml_hi != 0;
        const double ue = s.char_imp * s.courant;
        const double uh = (1.0 / s.char_imp) * s.courant;
        if (threadIdx.x == 0) {
            I.ue = ue;
            I.uh = uh;
            I.ue_slab = s.free_space ? ue / s.eps_re : ue;
            I.uh_slab = s.free_space ? uh / s.mu_re : uh;
            I.dtdz = s.dt / s.dz;
            I.eps0 = s.eps0;
            I.sc = s.courant;
            // Lorentz ADE
            const double dt = s.dt;
            const double D = (1.0 / (dt * dt)) + (s.gamma / (2.0 * dt));
            I.pol_a = ((2.0 / (dt * dt)) - s.omega0 * s.omega0) / D;
            I.pol_b = ((s.gamma / (2.0 * dt)) - 1.0 / (dt * dt)) / D;
            I.pol_c = (s.eps0 * (s.plasma_freq * s.plasma_freq)) / D;
            // Kerr cubic: eps = 1 + wp^2 / den (complex division, Smith's form)
            const double w = 2.0 * kPi * s.freq_in * 2.0 * kPi * s.freq_in;
            const double dr = s.omega0 * s.omega0 - w;
            const double di = s.gamma * 2.0 * kPi * s.freq_in;
            const double num = s.plasma_freq * s.plasma_freq;
            double qr, qi;
            if (fabs(dr) >= fabs(di)) {
                const double rat = di / dr, scl = 1.0 / (dr + di * rat);
                qr = (num + 0.0 * rat) * scl;
                qi = (0.0 - num * rat) * scl;
            } else {
                const double rat = dr / di, scl = 1.0 / (di + dr * rat);
                qr = (num * rat + 0.0) * scl;
                qi = (0.0 * rat - num) * scl;
            }
            const double er = 1.0 + qr, ei = qi;
            const double ac = s.alpha3 * s.chi3;
            I.kerr_a = ac * ac;
            I.kerr_b = 2.0 * ((s.alpha3 * er) * s.chi3);
            const double mag = hypot(er, ei);
            I.kerr_c = mag * mag;
            I.nl_e0 = s.eps0 * sqrt(1.2);
            I.nl_e0chi = s.eps0 * s.chi3;
        }
        // the PML table: columns 0..pml are cells 0..pml, columns pml+1..2 pml are cells
        // n - pml .. n - 1
        const int W = 2 * pml + 1;
        double *t = tab + I.pml_offset;
        const bool any = (lo || hi) && pml > 0;
        // the right-hand denominators walk kappa from index pml down over the cells
        // [rstart, n); rstart skips cells the left loop already took
        const int rstart = (lo && pml + 1 > n - pml) ? pml + 1 : n - pml;
        for (int col = threadIdx.x; col < W; col += blockDim.x) {
            const int j = col <= pml ? col : n - pml + (col - pml - 1);
            double be = 0.0, ce = 0.0, cb = 0.0, cm = 0.0, c2 = 0.0, dene = 1.0, denh = 1.0;
            if (any) {
                if (j < pml || j >= n - pml) {
                    const Profile p = profile(s, pml, n, j);
                    be = exp(-((p.sigma * s.dt / (p.kappa * s.eps0)) + ((p.alpha * s.dt) / s.eps0)));
                    const double q = p.sigma * p.kappa + p.alpha * p.kappa * p.kappa;
                    ce = (be - 1.0) * p.sigma / q;
                    cm = (be - 1.0) * p.sigma / (q * s.dz);
                }
                if (j < pml || j >= n - pml + 1) {
                    cb = 1.0 * ue;
                    c2 = s.dt / s.mu0;
                }
                if (lo && j <= pml) {
                    const double inv = 1.0 / profile(s, pml, n, j).kappa;
                    dene = inv;
                    denh = inv;
                }
                if (hi && j >= n - pml && !(j <= pml && lo)) {
                    const int w = j - rstart;
                    denh = 1.0 / profile(s, pml, n, pml - w).kappa;
                    dene = 1.0 / profile(s, pml, n, pml - 1 - w).kappa;
                }
            }
            t[FDTD_TAB_BEX * W + col] = be;
            t[FDTD_TAB_CEX * W + col] = ce;
            t[FDTD_TAB_CB * W + col] = cb;
            t[FDTD_TAB_BMY * W + col] = be;
            t[FDTD_TAB_CMY * W + col] = cm;
            t[FDTD_TAB_C2 * W + col] = c2;
            t[FDTD_TAB_DENE * W + col] = dene;
            t[FDTD_TAB_DENH * W + col] = denh;
        }
    }
}

}  // namespace

}  // namespace fdtdpic

using namespace fdtdpic;

extern "C" int fdtdpic_setup_layout(int64_t *out, int n)
{
    const int64_t v[] = {
        (int64_t)sizeof(FdtdSetup),
        offsetof(FdtdSetup, dz), offsetof(FdtdSetup, dt), offsetof(FdtdSetup, courant),
        offsetof(FdtdSetup, eps0), offsetof(FdtdSetup, mu0), offsetof(FdtdSetup, char_imp),
        offsetof(FdtdSetup, eps_re), offsetof(FdtdSetup, mu_re), offsetof(FdtdSetup, kappa_max),
        offsetof(FdtdSetup, sigma_opt), offsetof(FdtdSetup, alpha_max),
        offsetof(FdtdSetup, r_scale), offsetof(FdtdSetup, r_a_scale),
        offsetof(FdtdSetup, plasma_freq), offsetof(FdtdSetup, omega0), offsetof(FdtdSetup, gamma),
        offsetof(FdtdSetup, chi3), offsetof(FdtdSetup, alpha3), offsetof(FdtdSetup, freq_in),
        offsetof(FdtdSetup, free_space), offsetof(FdtdSetup, reserved)};
    const int m = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n && i < m; ++i) out[i] = v[i];
    return m;
}

extern "C" int fdtdpic_setup_batch(int n_inst, const FdtdSetup *d_setup, FdtdInstance *d_inst,
                                   double *d_pml_tab, fdtdpic_stream_t stream)
{
    if (n_inst < 0) return FDTDPIC_ERR_ARG;
    if (n_inst == 0) return FDTDPIC_OK;
    if (!d_setup || !d_inst || !d_pml_tab) return FDTDPIC_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FDTDPIC_ERR_NODEV;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = n_inst < 16 * sms ? n_inst : 16 * sms;
    if (grid < 1) grid = 1;
    setup_kernel<<<grid, 64, 0, (cudaStream_t)stream>>>(n_inst, d_setup, d_inst, d_pml_tab);
    return cuda_status(cudaGetLastError());
}
