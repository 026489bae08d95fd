/*
 * CPU oracle for the electron-beam PIC step.  TEST INFRASTRUCTURE ONLY (checker and CPU
 * baseline); the product never links or calls it.
 *
 * The reference has no particle code: its only hooks are the Jx array (MasterController.py:93,
 * :159) and the -Jx term of ADE_ExUpdate (BaseFDTD11.py:667).  This file is the FP64 statement of
 * the beam model this repository specifies; the GPU kernels implement the same model.
 *
 * Units and staggering.  Positions are zeta = z/dz (cells), held as an integer cell and a
 * fraction in [0, 1); Ex lives on nodes zeta = k, Hy on half nodes zeta = k + 1/2.  Momenta are u/c = gamma*v/c (x and z components).  In the
 * reference's sign convention Hy is minus the physical H_y (its Ex and Hy updates both carry the
 * opposite sign of Maxwell's curl equations), so B_y = -mu0 * Hy.  At the start of step t the
 * grid holds E^t and H^(t+1/2); the caller keeps H^(t-1/2) as Hyp, so B^t uses the average.
 *
 * One step for every particle (relativistic Boris):
 *   E  = CIC(Ex, zeta)            H = CIC((Hy + Hyp)/2, zeta - 1/2)
 *   u- = u + kE*E x_hat           (kE = q dt / (2 m c))
 *   g- = sqrt(1 + |u-|^2)         ty = kH*H/g-   (kH = -q mu0 dt / (2 m): ty = q dt B_y/(2 m g))
 *   u' = u- + u- x t ; u+ = u- + u' x s,  s = 2t/(1+t^2)
 *   u  = u+ + kE*E x_hat ; g = sqrt(1 + |u|^2)
 *   zeta1 = zeta + sc*uz/g        (sc = c dt / dz)
 *   Jx: CIC of kJ*ux/g at the midpoint zeta + sc*uz/(2g)    (kJ = q w c)
 *   Jz: charge-conserving at half nodes h+1/2:
 *       kJz*(W_h(zeta) - W_h(zeta1)),  W_h(z) = clamp(h + 1 - z, 0, 1)   (kJz = q w dz/dt)
 *       (|zeta1 - zeta| < 1, so at most the two half nodes around the crossed node)
 *   periodic wrap of the cell into [clo, chi)
 * Jx/Jz are "grid" currents (physical current density times dz), the units of the reference's
 * -Jx term: Ex += (dHy - Jx) * CharImp * Sc.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* scal: clo chi kE kH sc kJ kJz (clo/chi integral).  Positions are (cell, frac) with frac in
 * [0, 1): zeta = cell + frac, exact in the cell index.  Jx/Jz (nz+1) are overwritten with this
 * step's deposit.  Returns the number of particles that left the grid (0 expected). */
int or_pic_step(int n_part, int *cell, double *frac, double *ux, double *uz, const double *Ex,
                const double *Hy, const double *Hyp, double *Jx, double *Jz, int nz,
                const double *scal, int n_threads)
{
    const int clo = (int)scal[0], chi = (int)scal[1];
    const double kE = scal[2], kH = scal[3], sc = scal[4], kJ = scal[5], kJz = scal[6];
    const int Lc = chi - clo;
    const int len = nz + 1;
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n_part) n_threads = n_part > 0 ? n_part : 1;
    /* Thread t takes particles [n_part t / T, n_part (t+1) / T) and deposits into a private
     * window of cells [lo_t, hi_t] covering every node its particles can reach (c-1 .. c+2):
     * sorted beams need windows a fraction of the grid long, so large grids stay cheap.  The
     * windows are summed in thread order below. */
    int *win = (int *)malloc((size_t)n_threads * 2 * sizeof(int));
    size_t *off = (size_t *)malloc((size_t)(n_threads + 1) * sizeof(size_t));
    if (!win || !off) { free(win); free(off); return -1; }
    off[0] = 0;
    for (int t = 0; t < n_threads; ++t) {
        const int p0 = (int)((long long)n_part * t / n_threads);
        const int p1 = (int)((long long)n_part * (t + 1) / n_threads);
        int cmin = len, cmax = -1;
        for (int p = p0; p < p1; ++p) {
            if (cell[p] < cmin) cmin = cell[p];
            if (cell[p] > cmax) cmax = cell[p];
        }
        int lo = cmin - 1, hi = cmax + 2;
        if (lo < 0) lo = 0;
        if (hi > len - 1) hi = len - 1;
        if (hi < lo) { lo = 0; hi = -1; }
        win[2 * t] = lo;
        win[2 * t + 1] = hi;
        off[t + 1] = off[t] + 2 * (size_t)(hi - lo + 1);
    }
    double *bufs = (double *)calloc(off[n_threads] > 0 ? off[n_threads] : 1, sizeof(double));
    if (!bufs) { free(win); free(off); return -1; }
    int lost = 0;
    /* one partition per loop index, so the result does not depend on the team size */
#pragma omp parallel for num_threads(n_threads) schedule(static, 1) reduction(+ : lost)
    for (int t = 0; t < n_threads; ++t) {
        const int wlo = win[2 * t], wn = win[2 * t + 1] - wlo + 1;
        double *jx = bufs + off[t] - wlo; /* jx[k], jz[k] for k in [wlo, whi] */
        double *jz = jx + wn;
        const int p_begin = (int)((long long)n_part * t / n_threads);
        const int p_end = (int)((long long)n_part * (t + 1) / n_threads);
        for (int p = p_begin; p < p_end; ++p) {
            const int c = cell[p];
            const double f = frac[p];
            int j;
            double fh;
            if (f >= 0.5) { j = c; fh = f - 0.5; } else { j = c - 1; fh = f + 0.5; }
            if (c < 1 || c + 2 > nz) { ++lost; continue; }
            const double E = (1.0 - f) * Ex[c] + f * Ex[c + 1];
            const double H = (1.0 - fh) * (0.5 * (Hy[j] + Hyp[j])) + fh * (0.5 * (Hy[j + 1] + Hyp[j + 1]));
            const double uxm = ux[p] + kE * E;
            const double uzm = uz[p];
            const double gm = sqrt(1.0 + uxm * uxm + uzm * uzm);
            const double ty = kH * H / gm;
            const double sy = 2.0 * ty / (1.0 + ty * ty);
            const double uxp = uxm - uzm * ty;
            const double uzp = uzm + uxm * ty;
            const double uxn = (uxm - uzp * sy) + kE * E;
            const double uzn = uzm + uxp * sy;
            const double g = sqrt(1.0 + uxn * uxn + uzn * uzn);
            const double dz = sc * uzn / g;
            /* Jx at the half-step midpoint */
            double fm = f + 0.5 * dz;
            int cm = c;
            if (fm >= 1.0) { cm += 1; fm -= 1.0; } else if (fm < 0.0) { cm -= 1; fm += 1.0; }
            const double jxv = kJ * uxn / g;
            jx[cm] += jxv * (1.0 - fm);
            jx[cm + 1] += jxv * fm;
            /* new position and the charge-conserving Jz on half nodes */
            double f1 = f + dz;
            int c1 = c;
            if (f1 >= 1.0) { c1 += 1; f1 -= 1.0; } else if (f1 < 0.0) { c1 -= 1; f1 += 1.0; }
            if (c1 == c) {
                jz[c] += kJz * (f1 - f);
            } else if (c1 == c + 1) {
                jz[c] += kJz * (1.0 - f);
                jz[c + 1] += kJz * f1;
            } else {
                jz[c - 1] += -kJz * (1.0 - f1);
                jz[c] += -kJz * f;
            }
            if (c1 >= chi) c1 -= Lc;
            else if (c1 < clo) c1 += Lc;
            cell[p] = c1;
            frac[p] = f1;
            ux[p] = uxn;
            uz[p] = uzn;
        }
    }
#pragma omp parallel for num_threads(n_threads) schedule(static)
    for (int k = 0; k < len; ++k) {
        double sx = 0.0, sz = 0.0;
        for (int t = 0; t < n_threads; ++t) {
            const int wlo = win[2 * t];
            if (k < wlo || k > win[2 * t + 1]) continue;
            const int wn = win[2 * t + 1] - wlo + 1;
            sx += bufs[off[t] + (k - wlo)];
            sz += bufs[off[t] + wn + (k - wlo)];
        }
        Jx[k] = sx;
        Jz[k] = sz;
    }
    free(bufs);
    free(win);
    free(off);
    return lost;
}
