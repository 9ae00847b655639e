/* gsl/gsl_integration.h -- shim: QAGS from oracle/qags.c behind the GSL call
 * signatures the reference uses (function_objects/integrator.cpp).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef IMFIT_ORACLE_GSL_INTEGRATION_SHIM_H
#define IMFIT_ORACLE_GSL_INTEGRATION_SHIM_H
#include <stddef.h>
#include "gsl_errno.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct {
  double (*function)(double x, void *params);
  void *params;
} gsl_function;
typedef struct {
  size_t limit;
} gsl_integration_workspace;
typedef struct {
  size_t n;
} gsl_integration_cquad_workspace;
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qags(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                         size_t limit, gsl_integration_workspace *w, double *result, double *abserr);
int gsl_integration_qagi(gsl_function *f, double epsabs, double epsrel, size_t limit,
                         gsl_integration_workspace *w, double *result, double *abserr);
gsl_integration_cquad_workspace *gsl_integration_cquad_workspace_alloc(size_t n);
void gsl_integration_cquad_workspace_free(gsl_integration_cquad_workspace *w);
int gsl_integration_cquad(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                          gsl_integration_cquad_workspace *ws, double *result, double *abserr,
                          size_t *nevals);
#ifdef __cplusplus
}
#endif
#endif
