// fquantile.h -- the quantile function of the F distribution, for the upper
// confidence bound of the potential scale reduction factor (gelman's
// qf(0.5 * (1 + conf), nchain - 1, 2 w^2 / var_w), R/model-class.R:1613).
//
// F = (d2 / d1) x / (1 - x) where x solves I_x(d1/2, d2/2) = p, I the
// regularized incomplete beta function.  I is evaluated by its continued
// fraction (DLMF 8.17.22, modified Lentz method) on either side of the
// symmetry I_x(a, b) = 1 - I_{1-x}(b, a), or by a series of positive terms
// where both fractions cancel (fq_ibeta); x and 1 - x are passed separately
// so that neither is formed by a cancelling subtraction.  log B(a, b) for a
// large b (the second degrees of freedom are often 10^4 - 10^7) is formed
// from the Stirling series of the difference lgamma(b) - lgamma(a + b)
// rather than from two nearly equal lgamma values.  The root is found by bisection on log F, which needs no
// derivative and is safe for every (p, d1, d2).  Host/device, so the CPU
// tests run the same code.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define GG_FQ __host__ __device__ inline
#else
#define GG_FQ inline
#endif

namespace ggdmc {

// lgamma(x) - ((x - 1/2) log x - x + log(2 pi) / 2), x >= 10, by the
// Stirling series to x^-9 (remainder below 1e-13 there)
GG_FQ double fq_stirling_rest(double x)
{
    const double r = 1.0 / x, r2 = r * r;
    return r * (1.0 / 12 - r2 * (1.0 / 360 - r2 * (1.0 / 1260 - r2 * (1.0 / 1680 - r2 / 1188))));
}

// log B(a, b) = lgamma(a) + lgamma(b) - lgamma(a + b)
GG_FQ double fq_log_beta(double a, double b)
{
    if (a > b) {
        const double t = a;
        a = b;
        b = t;
    }
    if (b < 10.0) return lgamma(a) + lgamma(b) - lgamma(a + b);
    // lgamma(b) - lgamma(a + b) = -(b - 1/2) log1p(a / b) - a log(a + b) + a
    //                             + rest(b) - rest(a + b)
    const double d = -(b - 0.5) * log1p(a / b) - a * log(a + b) + a + fq_stirling_rest(b) -
                     fq_stirling_rest(a + b);
    return lgamma(a) + d;
}

// 1 / (1 + d1 / (1 + d2 / (1 + ...))) of I_x(a, b) (DLMF 8.17.22), modified Lentz
GG_FQ double fq_beta_cf(double a, double b, double x)
{
    const double tiny = 1e-300, eps = 1e-16;
    double f = 1.0, C = 1.0, D = 0.0;
    for (int j = 1; j <= 2000; ++j) {
        const int m = j / 2;
        double dj;
        if (j & 1) dj = -(a + m) * (a + b + m) * x / ((a + 2 * m) * (a + 2 * m + 1));
        else dj = m * (b - m) * x / ((a + 2 * m - 1) * (a + 2 * m));
        // term j: a_j = dj over the previous level's 1 + ...
        D = 1.0 + dj * D;
        if (fabs(D) < tiny) D = tiny;
        C = 1.0 + dj / C;
        if (fabs(C) < tiny) C = tiny;
        D = 1.0 / D;
        const double delta = C * D;
        f *= delta;
        if (fabs(delta - 1.0) < eps) break;
    }
    return 1.0 / f;
}

// I_x(a, b) with y = 1 - x given separately; lx = log x, ly = log y.
// Three regions, each free of cancellation (checked against 40-digit values
// for a in [0.5, 300], b in [0.25, 1e12]):
//  * x < (a + 1) / (a + b + 2): the continued fraction of I_x(a, b);
//  * b <= a, or (a + b) y < (b + 1) / 2: 1 - the fraction of I_y(b, a);
//  * otherwise (b > a, x between the two): the series of positive terms
//    x^a y^b / (a B(a, b)) sum_j (a + b)_j / (a + 1)_j x^j (DLMF 8.17.8 with
//    8.17.4's symmetry), which needs about b x terms; beyond 60 standard
//    deviations above the mean a / (a + b), where 1 - I < 1e-17 for a >= 1/2,
//    the value is 1.
GG_FQ double fq_ibeta(double a, double b, double x, double y, double lx, double ly)
{
    if (x <= 0.0) return 0.0;
    if (y <= 0.0) return 1.0;
    const double pre = exp(a * lx + b * ly - fq_log_beta(a, b));
    if (x < (a + 1.0) / (a + b + 2.0)) return pre * fq_beta_cf(a, b, x) / a;
    if (b <= a || (a + b) * y < 0.5 * (b + 1.0)) return 1.0 - pre * fq_beta_cf(b, a, y) / b;
    const double ab = a + b, mu = a / ab, sd = sqrt(a * b / (ab * ab * (ab + 1.0)));
    if (x > mu + 60.0 * sd) return 1.0;
    double s = 1.0, t = 1.0;
    for (int j = 0; j < 10000000; ++j) {
        t *= x * (ab + j) / (a + j + 1.0);
        s += t;
        if (t < 1e-17 * s && x * (ab + j) < a + j + 1.0) break;
    }
    return fmin(1.0, pre * s / a);
}

// P(F(d1, d2) <= f)
GG_FQ double f_cdf(double f, double d1, double d2)
{
    if (!(f > 0.0)) return 0.0;
    const double u = d1 * f, s = u + d2;
    const double x = u / s, y = d2 / s;
    const double lx = log(u) - log(s), ly = -log1p(u / d2);
    return fq_ibeta(0.5 * d1, 0.5 * d2, x, y, lx, ly);
}

// qf(p, d1, d2) for 0 < p < 1, d1, d2 > 0 (d2 may be +inf: the chi-square
// limit is taken at d2 = 1e15, a relative change below 1e-14); NaN outside.
GG_FQ double f_quantile(double p, double d1, double d2)
{
    if (!(p > 0.0 && p < 1.0 && d1 > 0.0 && d2 > 0.0)) return NAN;
    if (d2 > 1e15) d2 = 1e15;
    double lo = -60.0, hi = 60.0;               // log F
    for (int it = 0; it < 200 && hi - lo > 1e-15 * (1.0 + fabs(lo)); ++it) {
        const double mid = 0.5 * (lo + hi);
        if (f_cdf(exp(mid), d1, d2) < p) lo = mid;
        else hi = mid;
    }
    return exp(0.5 * (lo + hi));
}

}  // namespace ggdmc
