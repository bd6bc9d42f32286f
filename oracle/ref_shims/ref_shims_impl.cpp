// Out-of-line parts of the test-only shims in this folder: METIS stubs (never
// called on the single-rank path) and a Gauss-Legendre rule for the GSL shim.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include "../../amcafe_gb300/csrc/cafe_quadrature.h"
#include "gsl/gsl_integration.h"
#include "metis.h"

static const gsl_integration_fixed_type cafe_legendre_type = {1};
const gsl_integration_fixed_type *gsl_integration_fixed_legendre = &cafe_legendre_type;

// The rule itself comes from amcafe_gb300/csrc/cafe_quadrature.h (ascending
// nodes, GSL's interval map), so the reference built here and the engine use
// the same nodes and weights.
gsl_integration_fixed_workspace *gsl_integration_fixed_alloc(const gsl_integration_fixed_type *,
                                                             size_t n, double a, double b, double,
                                                             double) {
  gsl_integration_fixed_workspace *w =
      (gsl_integration_fixed_workspace *)std::malloc(sizeof(gsl_integration_fixed_workspace));
  w->n = n;
  w->x = (double *)std::malloc(n * sizeof(double));
  w->w = (double *)std::malloc(n * sizeof(double));
  // the reference allocates the same rule at every call: keep the last one
  static size_t cn = 0;
  static double ca = 0, cb = 0, cx[64], cw[64];
  if (n <= 64 && n == cn && a == ca && b == cb) {
    for (size_t i = 0; i < n; ++i) {
      w->x[i] = cx[i];
      w->w[i] = cw[i];
    }
    return w;
  }
  cafe_gauss_legendre((int)n, a, b, w->x, w->w);
  if (n <= 64) {
    cn = n;
    ca = a;
    cb = b;
    for (size_t i = 0; i < n; ++i) {
      cx[i] = w->x[i];
      cw[i] = w->w[i];
    }
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
