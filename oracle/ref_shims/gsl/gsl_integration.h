/* Minimal stand-in for GSL 2.7.1's fixed-point Gauss-Legendre quadrature
 * (gsl_integration_fixed with gsl_integration_fixed_legendre), the only GSL
 * facility the reference uses (Utilities.C:112-122, the EASM temperature).
 * Test infrastructure: nodes and weights come from Newton iteration on the
 * Legendre polynomial P_n (amcafe_gb300/csrc/cafe_quadrature.h, correctly
 * rounded for n = 25), not from GSL itself (which solves the Golub-Welsch
 * eigenproblem), so the EASM path of a reference built on this shim is pinned
 * only up to the last bits of GSL's nodes. */
#ifndef CAFE_REF_SHIM_GSL_INTEGRATION_H
#define CAFE_REF_SHIM_GSL_INTEGRATION_H
#include <stddef.h>
typedef struct { double (*function)(double x, void *params); void *params; } gsl_function;
typedef struct { int kind; } gsl_integration_fixed_type;
typedef struct {
  size_t n;
  double *x;
  double *w;
} gsl_integration_fixed_workspace;
extern const gsl_integration_fixed_type *gsl_integration_fixed_legendre;
gsl_integration_fixed_workspace *gsl_integration_fixed_alloc(const gsl_integration_fixed_type *T,
                                                             size_t n, double a, double b,
                                                             double alpha, double beta);
void gsl_integration_fixed_free(gsl_integration_fixed_workspace *w);
int gsl_integration_fixed(const gsl_function *f, double *result,
                          const gsl_integration_fixed_workspace *w);
#endif
