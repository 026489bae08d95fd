// Per-cell Kerr cubic: the root the reference keeps, Re(CubicEquationSolver.solve(a,b,c,d)[0])
// (CubicEquationSolver.py:29-90, called from Nonlin_Cubic_Solver, BaseFDTD11.py:824-853).
//
// In exact arithmetic roots[0] is the largest real root in every branch of the closed form:
// 2*j*cos(k/3) - b/3a is the top root when h <= 0, S+U-b/3a the only real root when h > 0.
//
// cubic_root0_f64: the reference's closed form, operation for operation, in FP64.
// cubic_root0_f32: FP32 path for the mixed-precision kernels.  The per-instance constants
//   (f, the d-independent part of g, f^3/27, b/3a) are folded once in FP64; per cell only
//   g = g0 + d/a and h = g^2/4 + f^3/27 remain.  The FP32 closed form seeds three Newton steps
//   on the cubic itself (well conditioned where the closed form loses digits to the b/3a shift).
//   Cells whose discriminant is within 1e-3 of zero (branch choice uncertain in FP32), whose
//   Newton residual stays large, or whose values are not finite are re-solved with the FP64
//   closed form and counted.
//   Monotone case first: with a >= 0, b >= 0, c > 0 and d < 0 the cubic rises on x > 0 from
//   p(0) = d < 0, so its largest real root is its only positive root, and it is simple.  The
//   positive root x_q of b x^2 + c x + d (stable form -2d / (c + sqrt(c^2 - 4bd))) has
//   p(x_q) = a x_q^3 >= 0, so x_q lies at or above the root, where p is convex; Newton from x_q
//   then falls monotonically onto the root.  Three steps, then the same residual test; a cell
//   that fails it takes the closed-form path.  This is the Kerr slab's usual case (a = chi3'^2,
//   b = 2 Re(alpha3 eps chi3), c = |eps|^2, d = -|Dx/eps0|^2).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace fdtdpic {

__host__ __device__ inline double cubic_root0_f64(double a, double b, double c, double d)
{
    const double third = 1.0 / 3.0;
    if (a == 0.0 && b == 0.0) return (-d * 1.0) / c;
    if (a == 0.0) {
        double D = c * c - 4.0 * b * d;
        if (D >= 0) {
            D = sqrt(D);
            return (-c + D) / (2.0 * b);
        }
        return -c / (2.0 * b);
    }
    const double f = ((3.0 * c / a) - (pow(b, 2.0) / pow(a, 2.0))) / 3.0;
    const double g =
        (((2.0 * pow(b, 3.0)) / pow(a, 3.0)) - ((9.0 * b * c) / pow(a, 2.0)) + (27.0 * d / a)) / 27.0;
    const double h = (pow(g, 2.0) / 4.0 + pow(f, 3.0) / 27.0);
    if (f == 0 && g == 0 && h == 0) {
        if ((d / a) >= 0) return pow(d / (1.0 * a), third) * -1;
        return pow(-d / (1.0 * a), third);
    }
    if (h <= 0) {
        const double i = sqrt((pow(g, 2.0) / 4.0) - h);
        const double j = pow(i, third);
        const double k = acos(-(g / (2 * i)));
        return 2 * j * cos(k / 3.0) - (b / (3.0 * a));
    }
    const double R = -(g / 2.0) + sqrt(h);
    const double S = (R >= 0) ? pow(R, third) : pow(-R, third) * -1;
    const double T = -(g / 2.0) - sqrt(h);
    const double U = (T >= 0) ? pow(T, third) : pow(-T, third) * -1;
    return (S + U) - (b / (3.0 * a));
}

// Per-instance constants of the FP32 path, folded in FP64 from (a, b, c).
struct KerrF32 {
    float a, b, c, ia, bo3a, g0, f3, j2, inv2i, a3, b2, b4, c2;
    double ad, bd, cd;
    int kind;  // 0: general cubic, 1: linear (a=b=0), 2: quadratic (a=0) -> FP64
    int mono;  // a >= 0, b >= 0, c > 0: the monotone case applies for every d < 0
};

__device__ inline KerrF32 kerr_f32_setup(double a, double b, double c)
{
    KerrF32 k;
    k.ad = a; k.bd = b; k.cd = c;
    k.a = (float)a; k.b = (float)b; k.c = (float)c;
    k.a3 = (float)(3.0 * a); k.b2 = (float)(2.0 * b);
    k.b4 = (float)(4.0 * b); k.c2 = (float)(c * c);
    k.mono = (a >= 0.0 && b >= 0.0 && c > 0.0 && !(a == 0.0 && b == 0.0)) ? 1 : 0;
    if (a == 0.0) {
        k.kind = (b == 0.0) ? 1 : 2;
        k.ia = k.bo3a = k.g0 = k.f3 = k.j2 = k.inv2i = 0.f;
        return k;
    }
    k.kind = 0;
    const double f = ((3.0 * c / a) - (b * b) / (a * a)) / 3.0;
    const double g0 = ((2.0 * b * b * b) / (a * a * a) - (9.0 * b * c) / (a * a)) / 27.0;
    const double f3 = f * f * f / 27.0;
    k.ia = (float)(1.0 / a);
    k.bo3a = (float)(b / (3.0 * a));
    k.g0 = (float)g0;
    k.f3 = (float)f3;
    if (f < 0.0) {
        const double i = sqrt(-f3);  // sqrt(g^2/4 - h) = sqrt(-f^3/27), independent of d
        k.j2 = (float)(2.0 * cbrt(i));
        k.inv2i = (float)(0.5 / i);
    } else {
        k.j2 = 0.f;
        k.inv2i = 0.f;
    }
    return k;
}

// The FP64 re-solve, out of line: it is rare, and inlined it would hold registers in every
// kernel that steps Kerr cells.
static __device__ __noinline__ float cubic_root0_f64_to_f32(double a, double b, double c, double d)
{
    return (float)cubic_root0_f64(a, b, c, d);
}

__device__ inline float cubic_root0_f32(const KerrF32 &k, float d, int *n_fallback)
{
    if (k.kind == 1) return -d / k.c;
    if (k.mono && d < 0.f) {
        float x = __fdividef(-2.f * d, k.c + sqrtf(fmaf(-k.b4, d, k.c2)));
#pragma unroll
        for (int it = 0; it < 3; ++it) {
            const float p = fmaf(fmaf(fmaf(k.a, x, k.b), x, k.c), x, d);
            const float dp = fmaf(fmaf(k.a3, x, k.b2), x, k.c);
            x -= __fdividef(p, dp);
        }
        const float p = fmaf(fmaf(fmaf(k.a, x, k.b), x, k.c), x, d);
        const float mag = fabsf(k.c * x) + fabsf(d) + fabsf(k.b * x * x) + fabsf(k.a * x * x * x);
        if (isfinite(x) && fabsf(p) <= 1e-5f * mag) return x;
    }
    bool fb = (k.kind != 0);
    float x = 0.f;
    if (!fb) {
        const float g = fmaf(d, k.ia, k.g0);
        const float g2 = 0.25f * g * g;
        const float h = g2 + k.f3;
        const float scale = g2 + fabsf(k.f3);
        if (!(fabsf(h) > 1e-3f * scale) || !isfinite(h)) {
            fb = true;
        } else if (h < 0.f) {
            float arg = -g * k.inv2i;
            arg = fminf(1.f, fmaxf(-1.f, arg));
            x = k.j2 * cosf(acosf(arg) * (1.f / 3.f)) - k.bo3a;
        } else {
            const float sh = sqrtf(h);
            x = cbrtf(-0.5f * g + sh) + cbrtf(-0.5f * g - sh) - k.bo3a;
        }
        if (!fb) {
#pragma unroll
            for (int it = 0; it < 3; ++it) {
                const float p = fmaf(fmaf(fmaf(k.a, x, k.b), x, k.c), x, d);
                const float dp = fmaf(fmaf(k.a3, x, k.b2), x, k.c);
                x -= p / dp;
            }
            const float p = fmaf(fmaf(fmaf(k.a, x, k.b), x, k.c), x, d);
            const float mag = fabsf(k.c * x) + fabsf(d) + fabsf(k.b * x * x) + fabsf(k.a * x * x * x);
            if (!isfinite(x) || fabsf(p) > 1e-4f * mag) fb = true;
        }
    }
    if (fb) {
        if (n_fallback) ++*n_fallback;
        x = cubic_root0_f64_to_f32(k.ad, k.bd, k.cd, (double)d);
    }
    return x;
}

}  // namespace fdtdpic
