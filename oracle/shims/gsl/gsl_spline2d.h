/* gsl/gsl_spline2d.h -- shim: allocation succeeds (the reference builds a
 * bicubic PSF interpolator for every oversampled PSF), evaluation is not
 * available and returns NaN.  PointSource functions, the only users of the
 * interpolated value, are outside the oracle.  TEST INFRASTRUCTURE ONLY. */
#ifndef IMFIT_ORACLE_GSL_SPLINE2D_SHIM_H
#define IMFIT_ORACLE_GSL_SPLINE2D_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { int kind; } gsl_interp2d_type;
typedef struct { size_t nx, ny; } gsl_spline2d;
typedef struct { size_t cache; } gsl_interp_accel;
extern const gsl_interp2d_type *gsl_interp2d_bicubic;
gsl_interp_accel *gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel *a);
gsl_spline2d *gsl_spline2d_alloc(const gsl_interp2d_type *T, size_t xsize, size_t ysize);
int gsl_spline2d_init(gsl_spline2d *interp, const double xa[], const double ya[], const double za[],
                      size_t xsize, size_t ysize);
double gsl_spline2d_eval(const gsl_spline2d *interp, double x, double y, gsl_interp_accel *xa,
                         gsl_interp_accel *ya);
void gsl_spline2d_free(gsl_spline2d *interp);
#ifdef __cplusplus
}
#endif
#endif
