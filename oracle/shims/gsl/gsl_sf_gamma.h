/* gsl/gsl_sf_gamma.h -- shim: the Gamma function from the C library (used by
 * the reference only in Sersic::TotalFlux).  TEST INFRASTRUCTURE ONLY. */
#ifndef IMFIT_ORACLE_GSL_SF_GAMMA_SHIM_H
#define IMFIT_ORACLE_GSL_SF_GAMMA_SHIM_H
#include <math.h>
static inline double gsl_sf_gamma(double x) { return tgamma(x); }
#endif
