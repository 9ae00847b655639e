/* fft_ref.h -- FP64 mixed-radix complex FFT for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This is part of the CPU oracle that the GPU path
 * is checked against; nothing in the product library links it.
 *
 * Any length is accepted: factors 4, 2, 3, 5, 7 use small butterflies and any
 * remaining prime factor p is handled by a direct length-p DFT inside the same
 * Stockham (self-sorting, out-of-place) pass structure.  The transform is
 * unnormalised in both directions, like FFTW's documented convention
 * (forward = exp(-2 pi i jk/n), backward = exp(+2 pi i jk/n)).
 */
#ifndef IMFIT_ORACLE_FFT_REF_H
#define IMFIT_ORACLE_FFT_REF_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fftref_plan fftref_plan;

fftref_plan *fftref_plan_create(int n);
void fftref_plan_destroy(fftref_plan *p);
int fftref_plan_length(const fftref_plan *p);
/* In-place transform of n interleaved complex values; work holds 2n doubles.
 * sign = -1 forward, +1 backward. */
void fftref_exec(const fftref_plan *p, double *data, double *work, int sign);

/* 2-D real transforms in the row-major layout FFTW's r2c/c2r_2d use:
 * real array n0 x n1, half spectrum n0 x (n1/2+1) interleaved complex.
 * c2r is unnormalised and may overwrite its input. */
typedef struct fftref_plan2d fftref_plan2d;
fftref_plan2d *fftref_plan2d_create(int n0, int n1);
void fftref_plan2d_destroy(fftref_plan2d *p);
void fftref_r2c_2d(const fftref_plan2d *p, const double *in, double *out);
void fftref_c2r_2d(const fftref_plan2d *p, double *in, double *out);

#ifdef __cplusplus
}
#endif
#endif
