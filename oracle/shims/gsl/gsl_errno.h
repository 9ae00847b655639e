/* gsl/gsl_errno.h -- shim for compiling the reference's sources into the
 * CPU oracle (GSL is not installed here).  TEST INFRASTRUCTURE ONLY. */
#ifndef IMFIT_ORACLE_GSL_ERRNO_SHIM_H
#define IMFIT_ORACLE_GSL_ERRNO_SHIM_H
#ifdef __cplusplus
extern "C" {
#endif
#define GSL_SUCCESS 0
#define GSL_FAILURE (-1)
#define GSL_EMAXITER 11
#define GSL_EROUND 18
#define GSL_ESING 21
#define GSL_EDIVERGE 22
typedef void gsl_error_handler_t(const char *reason, const char *file, int line, int gsl_errno);
gsl_error_handler_t *gsl_set_error_handler_off(void);
#ifdef __cplusplus
}
#endif
#endif
