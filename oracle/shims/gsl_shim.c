/* gsl_shim.c -- the GSL entry points the reference's hot-path sources call,
 * implemented over oracle/qags.c.  TEST INFRASTRUCTURE ONLY. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include "gsl/gsl_integration.h"
#include "gsl/gsl_spline2d.h"
#include "../qags.h"

gsl_error_handler_t *gsl_set_error_handler_off(void) { return NULL; }

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n) {
  gsl_integration_workspace *w = (gsl_integration_workspace *)malloc(sizeof(*w));
  w->limit = n;
  return w;
}
void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }

int gsl_integration_qags(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                         size_t limit, gsl_integration_workspace *w, double *result, double *abserr) {
  if (limit > w->limit) limit = w->limit;
  int st = qags_integrate(f->function, f->params, a, b, epsabs, epsrel, (int)limit, result, abserr,
                          NULL, NULL);
  switch (st) {
    case QAGS_OK: return GSL_SUCCESS;
    case QAGS_MAXITER: return GSL_EMAXITER;
    case QAGS_ROUND: return GSL_EROUND;
    case QAGS_SING: return GSL_ESING;
    case QAGS_DIVERGE: return GSL_EDIVERGE;
    default: return GSL_FAILURE;
  }
}

int gsl_integration_qagi(gsl_function *f, double epsabs, double epsrel, size_t limit,
                         gsl_integration_workspace *w, double *result, double *abserr) {
  (void)f; (void)epsabs; (void)epsrel; (void)limit; (void)w;
  fprintf(stderr, "oracle gsl shim: gsl_integration_qagi is not provided\n");
  *result = NAN;
  *abserr = NAN;
  return GSL_FAILURE;
}

gsl_integration_cquad_workspace *gsl_integration_cquad_workspace_alloc(size_t n) {
  gsl_integration_cquad_workspace *w = (gsl_integration_cquad_workspace *)malloc(sizeof(*w));
  w->n = n;
  return w;
}
void gsl_integration_cquad_workspace_free(gsl_integration_cquad_workspace *w) { free(w); }
int gsl_integration_cquad(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                          gsl_integration_cquad_workspace *ws, double *result, double *abserr,
                          size_t *nevals) {
  (void)f; (void)a; (void)b; (void)epsabs; (void)epsrel; (void)ws;
  fprintf(stderr, "oracle gsl shim: gsl_integration_cquad is not provided\n");
  *result = NAN;
  *abserr = NAN;
  if (nevals) *nevals = 0;
  return GSL_FAILURE;
}

static const gsl_interp2d_type bicubic_kind = {1};
const gsl_interp2d_type *gsl_interp2d_bicubic = &bicubic_kind;
gsl_interp_accel *gsl_interp_accel_alloc(void) { return (gsl_interp_accel *)calloc(1, sizeof(gsl_interp_accel)); }
void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }
gsl_spline2d *gsl_spline2d_alloc(const gsl_interp2d_type *T, size_t xsize, size_t ysize) {
  (void)T;
  gsl_spline2d *s = (gsl_spline2d *)malloc(sizeof(*s));
  s->nx = xsize;
  s->ny = ysize;
  return s;
}
int gsl_spline2d_init(gsl_spline2d *interp, const double xa[], const double ya[], const double za[],
                      size_t xsize, size_t ysize) {
  (void)interp; (void)xa; (void)ya; (void)za; (void)xsize; (void)ysize;
  return 0;
}
double gsl_spline2d_eval(const gsl_spline2d *interp, double x, double y, gsl_interp_accel *xa,
                         gsl_interp_accel *ya) {
  (void)interp; (void)x; (void)y; (void)xa; (void)ya;
  return NAN;
}
void gsl_spline2d_free(gsl_spline2d *interp) { free(interp); }
double gsl_sf_bessel_K1(double x) { (void)x; return NAN; }
