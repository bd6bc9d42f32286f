// Out-of-line parts of the test-only shims in this folder: METIS stubs (never
// called on the single-rank path) and a Gauss-Legendre rule for the GSL shim.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include "gsl/gsl_integration.h"
#include "metis.h"

static const gsl_integration_fixed_type cafe_legendre_type = {1};
const gsl_integration_fixed_type *gsl_integration_fixed_legendre = &cafe_legendre_type;

// Legendre P_n and its derivative by the three-term recurrence.
static void legendre_eval(int n, double x, double *p, double *dp) {
  double p0 = 1.0, p1 = x;
  if (n == 0) { *p = 1.0; *dp = 0.0; return; }
  for (int k = 2; k <= n; ++k) {
    double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = pk;
  }
  *p = p1;
  *dp = n * (x * p1 - p0) / (x * x - 1.0);
}

gsl_integration_fixed_workspace *gsl_integration_fixed_alloc(const gsl_integration_fixed_type *,
                                                             size_t n, double a, double b, double,
                                                             double) {
  gsl_integration_fixed_workspace *w =
      (gsl_integration_fixed_workspace *)std::malloc(sizeof(gsl_integration_fixed_workspace));
  w->n = n;
  w->x = (double *)std::malloc(n * sizeof(double));
  w->w = (double *)std::malloc(n * sizeof(double));
  const double pi = 3.14159265358979323846;
  for (size_t i = 0; i < n; ++i) {
    // Newton iteration from the Chebyshev-like initial guess.
    double x = std::cos(pi * (i + 0.75) / (n + 0.5)), p, dp;
    for (int it = 0; it < 100; ++it) {
      legendre_eval((int)n, x, &p, &dp);
      double dx = p / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    legendre_eval((int)n, x, &p, &dp);
    double wt = 2.0 / ((1.0 - x * x) * dp * dp);
    w->x[i] = 0.5 * (b - a) * x + 0.5 * (b + a);
    w->w[i] = 0.5 * (b - a) * wt;
  }
  return w;
}

void gsl_integration_fixed_free(gsl_integration_fixed_workspace *w) {
  if (!w) return;
  std::free(w->x);
  std::free(w->w);
  std::free(w);
}

int gsl_integration_fixed(const gsl_function *f, double *result,
                          const gsl_integration_fixed_workspace *w) {
  double s = 0.0;
  for (size_t i = 0; i < w->n; ++i) s += w->w[i] * f->function(w->x[i], f->params);
  *result = s;
  return 0;
}

int METIS_PartGraphRecursive(idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *,
                             idx_t *, real_t *, real_t *, idx_t *, idx_t *, idx_t *) {
  std::fprintf(stderr, "metis shim: PartitionGraph is not available\n");
  std::abort();
}
int METIS_PartGraphKway(idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *,
                        real_t *, real_t *, idx_t *, idx_t *, idx_t *) {
  std::fprintf(stderr, "metis shim: PartitionGraph is not available\n");
  std::abort();
}
