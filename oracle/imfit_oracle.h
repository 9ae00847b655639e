/* imfit_oracle.h -- CPU FP64 restatement of the reference's model-image and
 * fit-statistic path (ModelObject + the hot-path FunctionObjects + Convolver +
 * OversampledRegion + downsample + statistics).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU library is checked
 * against (tests/, __graft_entry__.smoke(), bench.py's CPU-baseline leg).
 * The product library never links or calls it.
 *
 * The call sequence mirrors the reference's ModelObject (core/model_object.h):
 * functions are added first, then PSF, then the image size / data, then
 * errors, mask and statistic choice, then orc_final_setup.
 */
#ifndef IMFIT_ORACLE_H
#define IMFIT_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_model orc_model;

orc_model *orc_create(void);
void orc_destroy(orc_model *m);
void orc_set_max_threads(orc_model *m, int n);
/* pad FFTs to 2,3,5,7-smooth sizes (>= the reference's N+P-1): same
 * convolution up to rounding, faster transforms; call before the image size */
void orc_set_fft_smooth(orc_model *m, int flag);

/* name = config-file function name; newSet = 1 starts a new function set
 * (its own X0,Y0).  Returns 0, or -1 for an unknown name. */
int orc_add_function(orc_model *m, const char *name, int newSet, int subsampling);
int orc_finish_functions(orc_model *m);

int orc_add_psf(orc_model *m, int ncols, int nrows, const double *psf, int normalize);
/* region in 1-based inclusive pixel coordinates, like "x1:x2,y1:y2" */
int orc_add_oversampled_psf(orc_model *m, int ncols, int nrows, const double *psf, int scale,
                            int x1, int x2, int y1, int y2, int normalize);
int orc_setup_model_image(orc_model *m, int ncols, int nrows);
int orc_add_image_data(orc_model *m, const double *pix, int ncols, int nrows);
void orc_add_image_characteristics(orc_model *m, double gain, double rn, double texp, int ncomb,
                                   double sky);
int orc_add_error_vector(orc_model *m, const double *pix, int ncols, int nrows, int type);
int orc_add_mask_vector(orc_model *m, const double *pix, int ncols, int nrows, int type);
int orc_use_cash(orc_model *m);
void orc_use_pmlr(orc_model *m);
int orc_use_model_errors(orc_model *m);
int orc_final_setup(orc_model *m);

int orc_n_params(orc_model *m);
long orc_n_data(orc_model *m);
long orc_n_valid(orc_model *m);
int orc_which_statistic(orc_model *m);
int orc_model_size(orc_model *m, int *ncols, int *nrows);
int orc_fft_size(orc_model *m, int *ncols, int *nrows);

void orc_create_model_image(orc_model *m, const double *params);
int orc_set_point_source_method(orc_model *m, int index, int method);
int orc_get_single_function_image(orc_model *m, const double *params, int index, double *out);
int orc_interpolate_psf(int kind, const double *psf, int ncols, int nrows, const double *dx, const double *dy,
                        long n, double *out);
double orc_lanczos(double x, int n);
int orc_get_model_image(orc_model *m, double *out);
int orc_get_expanded_model_image(orc_model *m, double *out, long n);
void orc_compute_deviates(orc_model *m, double *out, const double *params);
double orc_get_fit_statistic(orc_model *m, const double *params);
int orc_get_weights(orc_model *m, double *out);          /* 1/sigma^2 form */
int orc_get_internal_weights(orc_model *m, double *out); /* 1/sigma (masked) */
int orc_get_mask(orc_model *m, double *out);
int orc_get_data(orc_model *m, double *out);
int orc_get_extra_cash_terms(orc_model *m, double *out);

int orc_use_bootstrap(orc_model *m, unsigned long seed);
int orc_make_bootstrap_sample(orc_model *m);
long orc_get_bootstrap_indices(orc_model *m, long *out);

/* one-sided finite-difference Jacobian of the deviates (column-major,
 * nData x nParams), with mpfit's default step rule */
int orc_fd_jacobian(orc_model *m, const double *params, double *fjac);

double orc_function_value(const char *name, const double *params, double x0, double y0, double x,
                          double y, int subsampling);
double orc_function_total_flux(const char *name, const double *params);
/* QAGS relative tolerance of the 3-D functions' line-of-sight integrals
 * (default 1e-6 as the reference; a value <= 0 restores it) */
void orc_set_los_epsrel(double epsrel);
int orc_function_nparams(const char *name);
/* number of QAGS subintervals used for one 3-D function pixel (instrumentation) */
int orc_function_qags_nsub(const char *name, const double *params, double x0, double y0, double x,
                           double y);

#ifdef __cplusplus
}
#endif
#endif
