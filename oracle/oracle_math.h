/* Host math helpers shared by the CPU oracles (test infrastructure only).
 *
 * glibc has no erfinv(); CUDA's device library does, and the reference calls it
 * in its VNDF slope sampler (CLARITAS/CLARITAS.py:2032, `double sy=erfinv(ey)`).
 * This file supplies a host erfinv built from the mathematics, not from any
 * vendor implementation:
 *   1. an initial guess from the closed-form approximation of S. Winitzki,
 *      "A handy approximation for the error function and its inverse" (2008),
 *      erfinv(y) ~ sgn(y) sqrt( sqrt(t^2 - ln(1-y^2)/a) - t ),
 *      t = 2/(pi a) + ln(1-y^2)/2, a = 0.147;
 *   2. three Halley iterations on f(x) = erf(x) - y (f' = 2/sqrt(pi) e^{-x^2},
 *      f''/f' = -2x), using erfc() for |y| > 0.5 so the tail keeps full relative
 *      accuracy.
 * The result is checked against scipy.special.erfinv in tests/test_oracle_cpu.py.
 * Host and device results are not expected to be bit-identical.
 */
#ifndef CLARITAS_ORACLE_MATH_H
#define CLARITAS_ORACLE_MATH_H

#include <math.h>

static inline double oracle_erfinv(double y) {
    if (!(y > -1.0 && y < 1.0)) {
        if (y == 1.0) return HUGE_VAL;
        if (y == -1.0) return -HUGE_VAL;
        return NAN;
    }
    if (y == 0.0) return y;
    const double a = 0.147;
    const double pi = 3.14159265358979323846;
    double l = log1p(-y * y);            /* ln(1-y^2) without cancellation */
    double t = 2.0 / (pi * a) + 0.5 * l;
    double x = sqrt(sqrt(t * t - l / a) - t);
    if (y < 0.0) x = -x;
    const double two_over_sqrt_pi = 1.12837916709551257390;
    for (int it = 0; it < 3; ++it) {
        double r; /* r = erf(x) - y, computed to keep relative precision in the tails */
        if (y > 0.5) r = (1.0 - y) - erfc(x);
        else if (y < -0.5) r = erfc(-x) - (1.0 + y);
        else r = erf(x) - y;
        double fp = two_over_sqrt_pi * exp(-x * x);
        if (!(fp > 0.0)) break;
        double step = r / fp;
        /* Halley: x -= step / (1 + x*step) since f''/f' = -2x */
        x -= step / (1.0 + x * step);
    }
    return x;
}

#endif
