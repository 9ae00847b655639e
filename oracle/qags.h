/* qags.h -- adaptive Gauss-Kronrod quadrature with epsilon-algorithm
 * extrapolation (the QAGS method of QUADPACK, Piessens, de Doncker-Kapenga,
 * Ueberhuber & Kahaner 1983, routine DQAGSE), restated for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The reference integrates its 3-D line-of-sight
 * functions with GSL's gsl_integration_qags (function_objects/integrator.cpp:42-55,
 * epsabs = 0, epsrel = 1e-6, limit = 1000).  GSL is not installed here, so
 * this file provides the same published algorithm; it backs both the gsl/
 * shim used to compile the reference sources and the oracle restatement.
 */
#ifndef IMFIT_ORACLE_QAGS_H
#define IMFIT_ORACLE_QAGS_H
#ifdef __cplusplus
extern "C" {
#endif

typedef double (*qags_fn)(double x, void *params);

enum {
  QAGS_OK = 0,
  QAGS_MAXITER = 1,   /* subdivision limit reached */
  QAGS_ROUND = 2,     /* roundoff prevents the tolerance */
  QAGS_SING = 3,      /* bad integrand behaviour */
  QAGS_NOCONV = 4,    /* extrapolation table does not converge */
  QAGS_DIVERGE = 5,   /* integral probably divergent */
  QAGS_BADTOL = 6     /* tolerance cannot be achieved */
};

/* Returns one of the codes above; *result/*abserr are always written.
 * *nsub (optional) receives the number of subintervals used and *neval the
 * number of integrand evaluations. */
int qags_integrate(qags_fn f, void *params, double a, double b, double epsabs, double epsrel,
                   int limit, double *result, double *abserr, int *nsub, int *neval);

/* One 21-point Gauss-Kronrod panel on [a,b] (QUADPACK DQK21). */
void qags_qk21(qags_fn f, void *params, double a, double b, double *result, double *abserr,
               double *resabs, double *resasc);

#ifdef __cplusplus
}
#endif
#endif
