/* fftw3_shim.c -- FFTW3-API shim over oracle/fft_ref.c (TEST INFRASTRUCTURE
 * ONLY; see fftw3.h).  Plans remember their arrays, as FFTW plans do, so
 * fftw_execute(plan) transforms the arrays given at planning time. */
#define _POSIX_C_SOURCE 200112L
#include <stdlib.h>
#include "fftw3.h"
#include "../fft_ref.h"

struct fftw_plan_s {
  int kind; /* 0 = r2c, 1 = c2r */
  fftref_plan2d *p;
  double *rin, *rout;
  double *cin, *cout;
};

void *fftw_malloc(size_t n) {
  void *p = NULL;
  if (posix_memalign(&p, 64, n ? n : 1) != 0) return NULL;
  return p;
}
void fftw_free(void *p) { free(p); }

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags) {
  (void)flags;
  struct fftw_plan_s *pl = (struct fftw_plan_s *)calloc(1, sizeof(*pl));
  pl->kind = 0;
  pl->p = fftref_plan2d_create(n0, n1);
  pl->rin = in;
  pl->cout = (double *)out;
  return pl;
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags) {
  (void)flags;
  struct fftw_plan_s *pl = (struct fftw_plan_s *)calloc(1, sizeof(*pl));
  pl->kind = 1;
  pl->p = fftref_plan2d_create(n0, n1);
  pl->cin = (double *)in;
  pl->rout = out;
  return pl;
}

void fftw_execute(const fftw_plan pl) {
  if (pl->kind == 0)
    fftref_r2c_2d(pl->p, pl->rin, pl->cout);
  else
    fftref_c2r_2d(pl->p, pl->cin, pl->rout);
}

void fftw_destroy_plan(fftw_plan pl) {
  if (!pl) return;
  fftref_plan2d_destroy(pl->p);
  free(pl);
}
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int nthreads) { (void)nthreads; }
void fftw_cleanup_threads(void) {}
