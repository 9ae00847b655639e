/* fft_ref.c -- FP64 mixed-radix complex FFT for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see fft_ref.h).  Written from the textbook
 * Stockham autosort formulation of the Cooley-Tukey algorithm: pass p with
 * radix R and span Ns reads x[j + r*n/R], applies the twiddle
 * exp(sign*2*pi*i*r*(j mod Ns)/(Ns*R)), does a length-R DFT and writes the
 * results to y[(j/Ns)*Ns*R + (j mod Ns) + t*Ns].  The output comes out in
 * natural order after the last pass.
 *
 * It stands in for FFTW3 (which is not installed here) behind the fftw3.h
 * shim used to compile the reference's own convolver.cpp, and it is the FFT of
 * the restated convolution in imfit_oracle.c.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "fft_ref.h"

#define MAX_FACTORS 64

struct fftref_plan {
  int n;
  int nf;
  int factors[MAX_FACTORS];
  double *tw; /* tw[2k], tw[2k+1] = cos, -sin of 2 pi k / n (forward table) */
};

static int factorize(int n, int *f) {
  int nf = 0;
  while (n % 4 == 0) { f[nf++] = 4; n /= 4; }
  while (n % 2 == 0) { f[nf++] = 2; n /= 2; }
  for (int p = 3; n > 1; p += 2) {
    while (n % p == 0) { f[nf++] = p; n /= p; }
    if (p * p > n && n > 1) { f[nf++] = n; n = 1; }
  }
  return nf;
}

fftref_plan *fftref_plan_create(int n) {
  if (n < 1) return NULL;
  fftref_plan *p = (fftref_plan *)calloc(1, sizeof(fftref_plan));
  p->n = n;
  p->nf = factorize(n, p->factors);
  p->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  const double twopi = 6.283185307179586476925286766559;
  for (int k = 0; k < n; k++) {
    double a = twopi * (double)k / (double)n;
    p->tw[2 * k] = cos(a);
    p->tw[2 * k + 1] = -sin(a);
  }
  return p;
}

void fftref_plan_destroy(fftref_plan *p) {
  if (!p) return;
  free(p->tw);
  free(p);
}

int fftref_plan_length(const fftref_plan *p) { return p->n; }

/* twiddle exp(sign * 2 pi i * idx / n) */
static inline void twid(const fftref_plan *p, long idx, int sign, double *c, double *s) {
  long k = idx % p->n;
  *c = p->tw[2 * k];
  *s = (sign < 0) ? p->tw[2 * k + 1] : -p->tw[2 * k + 1];
}

void fftref_exec(const fftref_plan *p, double *data, double *work, int sign) {
  const int n = p->n;
  if (n == 1) return;
  double *x = data, *y = work;
  int Ns = 1;
  double vr[64], vi[64];
  double *bigr = NULL, *bigi = NULL;
  for (int f = 0; f < p->nf; f++) {
    const int R = p->factors[f];
    const int m = n / R;
    double *ur = vr, *ui = vi;
    if (R > 32) {
      if (!bigr) {
        bigr = (double *)malloc(sizeof(double) * 4 * (size_t)n);
        bigi = bigr + 2 * (size_t)n;
      }
      ur = bigr;
      ui = bigi;
    }
    double *wr = ur + R, *wi = ui + R;
    for (int j = 0; j < m; j++) {
      const int k = j % Ns;
      for (int r = 0; r < R; r++) {
        double ar = x[2 * (j + r * m)], ai = x[2 * (j + r * m) + 1];
        if (r && k) {
          double c, s;
          twid(p, (long)r * k * (n / (Ns * R)), sign, &c, &s);
          double tr = ar * c - ai * s;
          ai = ar * s + ai * c;
          ar = tr;
        }
        ur[r] = ar;
        ui[r] = ai;
      }
      if (R == 2) {
        wr[0] = ur[0] + ur[1]; wi[0] = ui[0] + ui[1];
        wr[1] = ur[0] - ur[1]; wi[1] = ui[0] - ui[1];
      } else if (R == 4) {
        double a0r = ur[0] + ur[2], a0i = ui[0] + ui[2];
        double a1r = ur[0] - ur[2], a1i = ui[0] - ui[2];
        double a2r = ur[1] + ur[3], a2i = ui[1] + ui[3];
        double dr = ur[1] - ur[3], di = ui[1] - ui[3];
        /* s*i*(dr + i di) = (-s*di) + i (s*dr) */
        double er = -sign * di, ei = sign * dr;
        wr[0] = a0r + a2r; wi[0] = a0i + a2i;
        wr[2] = a0r - a2r; wi[2] = a0i - a2i;
        wr[1] = a1r + er;  wi[1] = a1i + ei;
        wr[3] = a1r - er;  wi[3] = a1i - ei;
      } else {
        for (int t = 0; t < R; t++) {
          double sr = 0.0, si = 0.0;
          for (int r = 0; r < R; r++) {
            double c, s;
            twid(p, (long)((r * t) % R) * (n / R), sign, &c, &s);
            sr += ur[r] * c - ui[r] * s;
            si += ur[r] * s + ui[r] * c;
          }
          wr[t] = sr;
          wi[t] = si;
        }
      }
      const int base = (j / Ns) * Ns * R + k;
      for (int t = 0; t < R; t++) {
        y[2 * (base + t * Ns)] = wr[t];
        y[2 * (base + t * Ns) + 1] = wi[t];
      }
    }
    double *tmp = x; x = y; y = tmp;
    Ns *= R;
  }
  if (x != data) memcpy(data, x, sizeof(double) * 2 * (size_t)n);
  free(bigr);
}

/* ----------------------------- 2-D real transforms ----------------------- */

struct fftref_plan2d {
  int n0, n1, nc; /* rows, columns, half-spectrum columns */
  fftref_plan *prow, *pcol;
};

fftref_plan2d *fftref_plan2d_create(int n0, int n1) {
  fftref_plan2d *p = (fftref_plan2d *)calloc(1, sizeof(fftref_plan2d));
  p->n0 = n0;
  p->n1 = n1;
  p->nc = n1 / 2 + 1;
  p->prow = fftref_plan_create(n1);
  p->pcol = fftref_plan_create(n0);
  return p;
}

void fftref_plan2d_destroy(fftref_plan2d *p) {
  if (!p) return;
  fftref_plan_destroy(p->prow);
  fftref_plan_destroy(p->pcol);
  free(p);
}

/* Rows are transformed two at a time: z = a + i b, then
 * A[k] = (Z[k] + conj Z[-k]) / 2 and B[k] = (Z[k] - conj Z[-k]) / (2i). */
void fftref_r2c_2d(const fftref_plan2d *p, const double *in, double *out) {
  const int n0 = p->n0, n1 = p->n1, nc = p->nc;
#pragma omp parallel
  {
    double *z = (double *)malloc(sizeof(double) * 4 * (size_t)(n1 > n0 ? n1 : n0));
    double *w = z + 2 * (size_t)(n1 > n0 ? n1 : n0);
#pragma omp for schedule(static)
    for (int r = 0; r < n0; r += 2) {
      const int haveB = (r + 1 < n0);
      const double *a = in + (size_t)r * n1;
      const double *b = haveB ? a + n1 : NULL;
      for (int k = 0; k < n1; k++) {
        z[2 * k] = a[k];
        z[2 * k + 1] = haveB ? b[k] : 0.0;
      }
      fftref_exec(p->prow, z, w, -1);
      double *oa = out + 2 * (size_t)r * nc;
      double *ob = haveB ? oa + 2 * (size_t)nc : NULL;
      for (int k = 0; k < nc; k++) {
        int mk = (n1 - k) % n1;
        double zr = z[2 * k], zi = z[2 * k + 1];
        double cr = z[2 * mk], ci = -z[2 * mk + 1];
        oa[2 * k] = 0.5 * (zr + cr);
        oa[2 * k + 1] = 0.5 * (zi + ci);
        if (haveB) {
          /* (Z - conjZ(-k)) / (2i) */
          double dr = zr - cr, di = zi - ci;
          ob[2 * k] = 0.5 * di;
          ob[2 * k + 1] = -0.5 * dr;
        }
      }
    }
#pragma omp for schedule(static)
    for (int c = 0; c < nc; c++) {
      for (int r = 0; r < n0; r++) {
        z[2 * r] = out[2 * ((size_t)r * nc + c)];
        z[2 * r + 1] = out[2 * ((size_t)r * nc + c) + 1];
      }
      fftref_exec(p->pcol, z, w, -1);
      for (int r = 0; r < n0; r++) {
        out[2 * ((size_t)r * nc + c)] = z[2 * r];
        out[2 * ((size_t)r * nc + c) + 1] = z[2 * r + 1];
      }
    }
    free(z);
  }
}

void fftref_c2r_2d(const fftref_plan2d *p, double *in, double *out) {
  const int n0 = p->n0, n1 = p->n1, nc = p->nc;
#pragma omp parallel
  {
    double *z = (double *)malloc(sizeof(double) * 4 * (size_t)(n1 > n0 ? n1 : n0));
    double *w = z + 2 * (size_t)(n1 > n0 ? n1 : n0);
#pragma omp for schedule(static)
    for (int c = 0; c < nc; c++) {
      for (int r = 0; r < n0; r++) {
        z[2 * r] = in[2 * ((size_t)r * nc + c)];
        z[2 * r + 1] = in[2 * ((size_t)r * nc + c) + 1];
      }
      fftref_exec(p->pcol, z, w, +1);
      for (int r = 0; r < n0; r++) {
        in[2 * ((size_t)r * nc + c)] = z[2 * r];
        in[2 * ((size_t)r * nc + c) + 1] = z[2 * r + 1];
      }
    }
#pragma omp for schedule(static)
    for (int r = 0; r < n0; r += 2) {
      const int haveB = (r + 1 < n0);
      const double *ia = in + 2 * (size_t)r * nc;
      const double *ib = haveB ? ia + 2 * (size_t)nc : NULL;
      /* Hermitian extension of each row; the imaginary parts of the DC and
       * (even-length) Nyquist bins are dropped, as a c2r transform does. */
      for (int k = 0; k < n1; k++) {
        double ar, ai, br = 0.0, bi = 0.0;
        int kk = (k < nc) ? k : n1 - k;
        int conj = (k >= nc);
        ar = ia[2 * kk];
        ai = ia[2 * kk + 1];
        if (haveB) { br = ib[2 * kk]; bi = ib[2 * kk + 1]; }
        if (kk == 0 || (2 * kk == n1)) { ai = 0.0; bi = 0.0; }
        if (conj) { ai = -ai; bi = -bi; }
        /* z = A + i B */
        z[2 * k] = ar - bi;
        z[2 * k + 1] = ai + br;
      }
      fftref_exec(p->prow, z, w, +1);
      double *oa = out + (size_t)r * n1;
      double *ob = haveB ? oa + n1 : NULL;
      for (int k = 0; k < n1; k++) {
        oa[k] = z[2 * k];
        if (haveB) ob[k] = z[2 * k + 1];
      }
    }
    free(z);
  }
}
