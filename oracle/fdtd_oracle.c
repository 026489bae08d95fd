/*
 * CPU oracle for the 1D FDTD/PIC time-stepping path.  TEST INFRASTRUCTURE ONLY: the tests, the
 * smoke check and the CPU-baseline leg of bench.py call it as the checker; the product never
 * links or calls it.
 *
 * FP64, compiled with -O2 -ffp-contract=off so every expression rounds in the order written,
 * which is the order of the reference's Python/numba loops:
 *   ADE_ExUpdate          BaseFDTD11.py:664-669
 *   CPML_Psi_e_Update     BaseFDTD11.py:365-376
 *   soft source / TF-SF   Solver_Engine.py:249-252 (NL), 307-310 (LinLor), 177-179 (free space)
 *   ADE_DxUpdate          BaseFDTD11.py:751-760
 *   AcubicFinder +
 *   Nonlin_Cubic_Solver   BaseFDTD11.py:803-853, root from CubicEquationSolver.py:29-90
 *   NonLinExUpdate        BaseFDTD11.py:859-877
 *   ADE_TempPolCurr +
 *   ADE_PolarisationCurrent_Ex  BaseFDTD11.py:487-538, 610-633
 *   ADE_ExCreate          BaseFDTD11.py:713-725
 *   ADE_HyUpdate          BaseFDTD11.py:641-656
 *   CPML_Psi_m_Update     BaseFDTD11.py:382-393
 *   vidMake / probeSim    Solver_Engine.py:57-68, 16-54
 * The per-cell coefficient arrays come from oracle.py, which restates the set-up functions.
 *
 * The PIC part (or_pic_run) has no counterpart in the reference: it is the FP64 restatement of the
 * beam model this repository specifies (relativistic Boris push, CIC gather/deposit, periodic wrap).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

enum { OR_FREESPACE = 0, OR_LINLOR = 1, OR_KERR = 2 };

/* CubicEquationSolver.solve(a, b, c, d) (CubicEquationSolver.py:29-90), all roots.
 * Real inputs; roots returned as (re, im) pairs, count in *n. */
void or_cubic_solve(double a, double b, double c, double d, double *re, double *im, int *n)
{
    const double third = 1.0 / 3.0;
    im[0] = im[1] = im[2] = 0.0;
    re[0] = re[1] = re[2] = 0.0;
    if (a == 0.0 && b == 0.0) {           /* linear, :30-31 */
        re[0] = (-d * 1.0) / c;
        *n = 1;
        return;
    }
    if (a == 0.0) {                       /* quadratic, :33-45 */
        double D = c * c - 4.0 * b * d;
        if (D >= 0) {
            D = sqrt(D);
            re[0] = (-c + D) / (2.0 * b);
            re[1] = (-c - D) / (2.0 * b);
        } else {
            D = sqrt(-D);
            re[0] = -c / (2.0 * b); im[0] = D / (2.0 * b);
            re[1] = -c / (2.0 * b); im[1] = -D / (2.0 * b);
        }
        *n = 2;
        return;
    }
    /* findF/findG/findH, :94-105 */
    double f = ((3.0 * c / a) - (pow(b, 2.0) / pow(a, 2.0))) / 3.0;
    double g = (((2.0 * pow(b, 3.0)) / pow(a, 3.0)) - ((9.0 * b * c) / pow(a, 2.0)) + (27.0 * d / a)) / 27.0;
    double h = (pow(g, 2.0) / 4.0 + pow(f, 3.0) / 27.0);
    *n = 3;
    if (f == 0 && g == 0 && h == 0) {     /* triple root, :51-56 */
        double x;
        if ((d / a) >= 0) x = pow(d / (1.0 * a), third) * -1;
        else x = pow(-d / (1.0 * a), third);
        re[0] = re[1] = re[2] = x;
    } else if (h <= 0) {                  /* three real roots, :58-72 */
        double i = sqrt((pow(g, 2.0) / 4.0) - h);
        double j = pow(i, third);
        double k = acos(-(g / (2 * i)));
        double L = j * -1;
        double M = cos(k / 3.0);
        double N = sqrt(3) * sin(k / 3.0);
        double P = (b / (3.0 * a)) * -1;
        re[0] = 2 * j * cos(k / 3.0) - (b / (3.0 * a));
        re[1] = L * (M + N) + P;
        re[2] = L * (M - N) + P;
    } else {                              /* one real root, :74-90 */
        double R = -(g / 2.0) + sqrt(h), S, U;
        if (R >= 0) S = pow(R, third);
        else S = pow(-R, third) * -1;
        double T = -(g / 2.0) - sqrt(h);
        if (T >= 0) U = pow(T, third);
        else U = pow(-T, third) * -1;
        re[0] = (S + U) - (b / (3.0 * a));
        re[1] = -(S + U) / 2 - (b / (3.0 * a)); im[1] = (S - U) * sqrt(3) * 0.5;
        re[2] = -(S + U) / 2 - (b / (3.0 * a)); im[2] = -(S - U) * sqrt(3) * 0.5;
    }
}

/* Re(roots[0]), the value Nonlin_Cubic_Solver keeps (BaseFDTD11.py:838). */
double or_cubic_root0(double a, double b, double c, double d)
{
    double re[3], im[3];
    int n;
    or_cubic_solve(a, b, c, d, re, im, &n);
    return re[0];
}

/* One integrator pass.  Arrays are length nz+1 unless noted; state arrays are read and written
 * in place, so a caller may continue a run.  Returns 0, or -1 on bad arguments.
 *   mode         OR_FREESPACE / OR_LINLOR / OR_KERR
 *   pol_active   LinLor only: 1 runs the polarisation update (pass i==1), 0 leaves P at zero
 *   coef[10]     upEx upHy denE denH beX ceX Cb bmY cmY C2 (each nz+1)
 *   scal[8]      dtdz eps0 polA polB polC kerr_a kerr_b kerr_c ; scal2[2] nl_e0 nl_e0chi
 *   src          Exs, Hys (n_steps each), sc = courant number used as the divisor
 *   probes       n_probe cells; probe_lo/probe_hi the inclusive step window in which sample
 *                k is written to probe_out[k*n_probe + p] (other rows untouched)
 *   hist         every hist_interval steps (k>0, k%hist_interval==0, k/hist_interval<hist_rows)
 *                Ex is copied to hist_out[(k/hist_interval)*(nz+1)]
 */
int or_run_pass(int mode, int pol_active, int nz, int t0, int n_steps, int pml, int cpml_lo,
                int cpml_hi, int front, int rear, int nzsrc, int tfsf, int dx_jx,
                const double *const *coef, const double *scal, const double *scal2,
                const double *Exs, const double *Hys, double sc,
                double *Ex, double *Hy, double *Dx, double *P, double *Pprev, double *psiE,
                double *psiH, double *Acub, const double *Jx,
                int n_probe, const int *probe_cells, int probe_lo, int probe_hi, double *probe_out,
                int hist_interval, int hist_rows, double *hist_out)
{
    if (nz < 2 || n_steps < 0 || pml < 0) return -1;
    const double *upEx = coef[0], *upHy = coef[1], *denE = coef[2], *denH = coef[3];
    const double *beX = coef[4], *ceX = coef[5], *Cb = coef[6], *bmY = coef[7], *cmY = coef[8],
                 *C2 = coef[9];
    const double dtdz = scal[0], eps0 = scal[1], pA = scal[2], pB = scal[3], pC = scal[4];
    const double ka = scal[5], kb = scal[6], kc = scal[7];
    const double e0r = scal2[0], e0chi = scal2[1];
    const int len = nz + 1;
    const int cpml = cpml_lo || cpml_hi;

    for (int t = t0; t < t0 + n_steps; ++t) {
        if (mode == OR_LINLOR && pol_active) {
            for (int k = front; k < rear; ++k) {
                double pm2 = Pprev[k];      /* tempTempVarPol after ADE_TempPolCurr */
                Pprev[k] = P[k];
                P[k] = pA * P[k] + pB * pm2 + pC * Ex[k];
            }
        }
        for (int k = 1; k < len; ++k)
            Ex[k] = Ex[k] + (Hy[k] - Hy[k - 1] - Jx[k]) * upEx[k] * denE[k];
        if (cpml) {
            if (cpml_lo)
                for (int k = 1; k < pml; ++k) {
                    psiE[k] = beX[k] * psiE[k] + ceX[k] * (Hy[k] - Hy[k - 1]);
                    Ex[k] = Ex[k] - Cb[k] * psiE[k];
                }
            if (cpml_hi)
                for (int k = len - pml; k < len; ++k) {
                    psiE[k] = beX[k] * psiE[k] + ceX[k] * (Hy[k] - Hy[k - 1]);
                    Ex[k] = Ex[k] - Cb[k] * psiE[k];
                }
        }
        Ex[nzsrc] += Exs[t] / sc;
        if (tfsf) Hy[nzsrc - 1] -= Hys[t] / sc;
        if (mode == OR_LINLOR || mode == OR_KERR) {
            if (dx_jx)
                for (int k = front; k < rear; ++k)
                    Dx[k] = Dx[k] + (Hy[k] - Hy[k - 1] - Jx[k]) * (dtdz) * denE[k];
            else
                for (int k = front; k < rear; ++k)
                    Dx[k] = Dx[k] + (Hy[k] - Hy[k - 1]) * (dtdz) * denE[k];
        }
        if (mode == OR_KERR) {
            for (int k = front; k < rear; ++k) {
                double q = fabs(Dx[k] / eps0);
                double d = -pow(q, 2.0);
                Acub[k] = (fabs(d) > 1e-8) ? or_cubic_root0(ka, kb, kc, d) : 0.0;
            }
            for (int k = front; k < rear; ++k)
                Ex[k] = Dx[k] / (e0r + e0chi * Acub[k]);
        } else if (mode == OR_LINLOR) {
            for (int k = front; k < rear; ++k)
                Ex[k] = (Dx[k] - P[k]) / (eps0);
        }
        for (int k = 1; k < nz; ++k)
            Hy[k] = Hy[k] * 1.0 + (Ex[k + 1] - Ex[k]) * upHy[k] * denH[k];
        if (cpml) {
            if (cpml_lo)
                for (int k = 1; k < pml; ++k) {
                    psiH[k] = bmY[k] * psiH[k] + cmY[k] * (Ex[k + 1] - Ex[k]);
                    Hy[k] = Hy[k] + C2[k] * psiH[k];
                }
            if (cpml_hi)
                for (int k = len - pml; k < len - 1; ++k) {
                    psiH[k] = bmY[k] * psiH[k] + cmY[k] * (Ex[k + 1] - Ex[k]);
                    Hy[k] = Hy[k] + C2[k] * psiH[k];
                }
        }
        if (hist_out && hist_interval > 0 && t > 0 && t % hist_interval == 0) {
            int row = t / hist_interval;
            if (row < hist_rows) memcpy(hist_out + (size_t)row * len, Ex, sizeof(double) * len);
        }
        if (probe_out && t >= probe_lo && t <= probe_hi)
            for (int p = 0; p < n_probe; ++p) probe_out[(size_t)t * n_probe + p] = Ex[probe_cells[p]];
    }
    return 0;
}
