/* fftw3.h -- minimal FFTW3-API shim used only to compile the reference's own
 * hot-path sources (convolver.cpp, psf_oversampling_info.cpp) into the test
 * oracle.  FFTW3 is not installed on this machine; the transforms are the
 * project-written FP64 FFT in oracle/fft_ref.c.  TEST INFRASTRUCTURE ONLY.
 *
 * Only the calls the reference makes are provided: r2c/c2r 2-D plans,
 * execute/destroy, malloc/free and the threading hooks (accepted; the FFT
 * itself uses OpenMP).
 */
#ifndef IMFIT_ORACLE_FFTW3_SHIM_H
#define IMFIT_ORACLE_FFTW3_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);

#ifdef __cplusplus
}
#endif
#endif
