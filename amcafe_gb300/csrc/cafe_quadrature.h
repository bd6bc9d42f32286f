// Fixed Gauss-Legendre rule for the EASM temperature.
//
// AMCAFE's Utilities::Integral (Utilities.C:105-124) integrates the moving
// Gaussian-source kernel with GSL's gsl_integration_fixed (25 Legendre nodes on
// [0, 8e-4 s]), whose result is sum_i w_i f(x_i) over the nodes in ascending
// order. This header computes that rule: the roots of P_n by Newton iteration
// from the asymptotic guess cos(pi (i + 3/4) / (n + 1/2)), refined by two
// Newton steps with P_n and P_n' evaluated in double-double, weights
// 2 / ((1 - x^2) P_n'(x)^2), and the map x -> (a + b)/2 + (b - a)/2 x,
// w -> (b - a)/2 w of GSL's scqf. Only IEEE operations and the correctly
// rounded cosine of cafe_crmath.h are used, so every machine gets the same
// bits.
#ifndef CAFE_QUADRATURE_H
#define CAFE_QUADRATURE_H

#include "cafe_crmath.h"

// P_n(x) and P_n'(x) in double-double by the three-term recurrence.
static inline void cafe_legendre_dd(int n, crm_dd x, crm_dd *p, crm_dd *dp) {
  crm_dd p0 = {1.0, 0.0}, p1 = x;
  for (int k = 2; k <= n; ++k) {
    // ((2k - 1) x p1 - (k - 1) p0) / k
    crm_dd a = crm_dd_mul_d(crm_dd_mul(x, p1), 2.0 * k - 1.0);
    crm_dd b = crm_dd_mul_d(p0, k - 1.0);
    crm_dd pk = crm_dd_div(crm_dd_add(a, crm_dd_neg(b)), crm_dd{(double)k, 0.0});
    p0 = p1;
    p1 = pk;
  }
  *p = p1;
  // n (x p1 - p0) / (x^2 - 1)
  crm_dd num = crm_dd_mul_d(crm_dd_add(crm_dd_mul(x, p1), crm_dd_neg(p0)), (double)n);
  crm_dd den = crm_dd_add(crm_dd_mul(x, x), crm_dd{-1.0, 0.0});
  *dp = crm_dd_div(num, den);
}

// n nodes x[] (ascending) and weights w[] of the Gauss-Legendre rule on [a, b].
static inline void cafe_gauss_legendre(int n, double a, double b, double *x, double *w) {
  const double pi = 3.141592653589793;
  const double slp = (b - a) / 2.0, shft = (a + b) / 2.0;
  for (int i = 0; i < n; ++i) {
    // the i-th root counted from +1, stored at n-1-i
    double t = crm_cos(pi * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      crm_dd p, dp;
      cafe_legendre_dd(n, crm_dd{t, 0.0}, &p, &dp);
      double dx = p.hi / dp.hi;
      t -= dx;
      if (fabs(dx) < 1e-15) break;
    }
    crm_dd td = {t, 0.0};
    for (int it = 0; it < 2; ++it) {
      crm_dd p, dp;
      cafe_legendre_dd(n, td, &p, &dp);
      td = crm_dd_add(td, crm_dd_neg(crm_dd_div(p, dp)));
    }
    crm_dd p, dp;
    cafe_legendre_dd(n, td, &p, &dp);
    crm_dd one_m = crm_dd_add(crm_dd{1.0, 0.0}, crm_dd_neg(crm_dd_mul(td, td)));
    crm_dd wt = crm_dd_div(crm_dd{2.0, 0.0}, crm_dd_mul(one_m, crm_dd_mul(dp, dp)));
    int k = n - 1 - i;
    x[k] = shft + slp * crm_dd_round(td);
    w[k] = crm_dd_round(wt) * slp;
  }
}

#endif
