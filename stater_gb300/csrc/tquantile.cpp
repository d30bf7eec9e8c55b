// Student-t quantiles (host). P(T > t) = I_x(df/2, 1/2) / 2 with
// x = df / (df + t^2), where the regularised incomplete beta function I_x(a, b)
// comes from its continued fraction (DLMF 8.17.22), evaluated with the modified
// Lentz method and used on the side of x where it converges quickly (swap via
// I_x(a, b) = 1 - I_{1-x}(b, a)). The quantile is the root of the tail equation,
// found by bracketing and bisection in t; the normal quantile (df <= 0) uses
// P(Z > z) = erfc(z / sqrt 2) / 2 in the same way.
#include "tquantile.h"

#include <cmath>

namespace stater {
namespace {

double guard(double v) { return std::fabs(v) < 1e-300 ? 1e-300 : v; }

// 1 / (1 + d1 / (1 + d2 / (1 + ...))) of DLMF 8.17.22.
double beta_fraction(double a, double b, double x) {
    double g = 1.0, C = 1.0, D = 0.0;
    for (int j = 1; j < 100000; j++) {
        double dj;
        const double m = (double)(j / 2);
        if ((j & 1) == 0)
            dj = m * (b - m) * x / ((a + 2.0 * m - 1.0) * (a + 2.0 * m));
        else
            dj = -(a + m) * (a + b + m) * x / ((a + 2.0 * m) * (a + 2.0 * m + 1.0));
        D = 1.0 / guard(1.0 + dj * D);
        C = guard(1.0 + dj / C);
        const double delta = C * D;
        g *= delta;
        if (std::fabs(delta - 1.0) < 1e-16) break;
    }
    return 1.0 / g;
}

double reg_inc_beta(double a, double b, double x) {
    if (x <= 0.0) return 0.0;
    if (x >= 1.0) return 1.0;
    const double front =
        std::exp(std::lgamma(a + b) - std::lgamma(a) - std::lgamma(b) + a * std::log(x) + b * std::log1p(-x));
    if (x < (a + 1.0) / (a + b + 2.0)) return front * beta_fraction(a, b, x) / a;
    return 1.0 - front * beta_fraction(b, a, 1.0 - x) / b;
}

double upper_tail(double t, double df) {
    if (df <= 0.0) return 0.5 * std::erfc(t / std::sqrt(2.0));
    return 0.5 * reg_inc_beta(0.5 * df, 0.5, df / (df + t * t));
}

}  // namespace

double t_quantile(double p, double df) {
    const double tail = 1.0 - p;
    double lo = 0.0, hi = 1.0;
    while (upper_tail(hi, df) > tail && hi < 1e12) hi *= 2.0;
    for (int it = 0; it < 400; it++) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (upper_tail(mid, df) > tail)
            lo = mid;
        else
            hi = mid;
    }
    return 0.5 * (lo + hi);
}

void tcrit2_table(double alpha, int N, double *table) {
    const double p = 1.0 - 0.5 * alpha;
    for (int m = 0; m <= N; m++) {
        const double t = m == 0 ? t_quantile(p, 0.0) : t_quantile(p, (double)N / (double)m);
        table[m] = t * t;
    }
}

}  // namespace stater
