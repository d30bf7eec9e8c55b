// Student-t quantiles for the Welch test's critical-value table (host code).
#pragma once

namespace stater {
// t with P(T <= t) = p for Student's t with df degrees of freedom (df <= 0:
// the standard normal quantile). p in (0.5, 1).
double t_quantile(double p, double df);
// table[m] = t_{1-alpha/2}(N/m)^2 for m = 1..N and table[0] = z_{1-alpha/2}^2.
void tcrit2_table(double alpha, int N, double *table);
}  // namespace stater
