/* gsl/gsl_sf_bessel.h -- shim declaration only (no oracle function uses it).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef IMFIT_ORACLE_GSL_SF_BESSEL_SHIM_H
#define IMFIT_ORACLE_GSL_SF_BESSEL_SHIM_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_bessel_K1(double x);
#ifdef __cplusplus
}
#endif
#endif
