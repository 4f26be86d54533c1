/* Test-infrastructure shim: the quadrature calls of src/cosmo.c:268-292 and
 * src/cosmo_mad.c:283-315, evaluated by the oracle's adaptive Gauss-Legendre
 * rule (converged far below the tolerances the reference requests). */
#ifndef SHIM_GSL_INTEGRATION_H
#define SHIM_GSL_INTEGRATION_H
#include <stddef.h>
typedef struct { double (*function)(double x, void *params); void *params; } gsl_function;
typedef struct gsl_integration_workspace gsl_integration_workspace;
typedef struct gsl_integration_qawo_table gsl_integration_qawo_table;
enum gsl_integration_qawo_enum { GSL_INTEG_COSINE, GSL_INTEG_SINE };
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
gsl_integration_qawo_table *gsl_integration_qawo_table_alloc(double omega, double L,
                                                             enum gsl_integration_qawo_enum sine,
                                                             size_t n);
void gsl_integration_qawo_table_free(gsl_integration_qawo_table *t);
int gsl_integration_qng(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                        double *result, double *abserr, size_t *neval);
int gsl_integration_qagil(gsl_function *f, double b, double epsabs, double epsrel, size_t limit,
                          gsl_integration_workspace *w, double *result, double *abserr);
int gsl_integration_qawf(gsl_function *f, const double a, const double epsabs, const size_t limit,
                         gsl_integration_workspace *w, gsl_integration_workspace *cw,
                         gsl_integration_qawo_table *wf, double *result, double *abserr);
#endif
