/* Oracle build shim (test infrastructure): the GSL quadrature API subset used by
 * driftfac.c:21-41.  GSL is not installed; oracle/shim_impl.c implements
 * gsl_integration_qag as adaptive bisection with a 20-point Gauss-Legendre rule
 * and a nested-error estimate, to the requested relative tolerance.  The drift and
 * kick tables the reference builds with it are stored as float
 * (allvars.h:124-125), so any quadrature accurate to 1e-8 yields the same table. */
#ifndef CUCO_ORACLE_GSL_INTEGRATION_SHIM_H
#define CUCO_ORACLE_GSL_INTEGRATION_SHIM_H
#include <stddef.h>
#define GSL_INTEG_GAUSS41 4
typedef struct {
    double (*function)(double x, void *params);
    void *params;
} gsl_function;
typedef struct { size_t limit; } gsl_integration_workspace;
#ifdef __cplusplus
extern "C" {
#endif
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs,
                        double epsrel, size_t limit, int key,
                        gsl_integration_workspace *workspace, double *result,
                        double *abserr);
#ifdef __cplusplus
}
#endif
#endif
