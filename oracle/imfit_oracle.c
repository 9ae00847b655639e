/* imfit_oracle.c -- CPU FP64 restatement of the reference's model-image and
 * fit-statistic path.  TEST INFRASTRUCTURE ONLY (see imfit_oracle.h).
 *
 * Every routine restates the reference routine named in its comment, with the
 * same floating-point expression order (compiled with -ffp-contract=off), so
 * on the same inputs it reproduces the reference to the last bit except where
 * the FFT differs (FFTW vs the project FFT in fft_ref.c).
 * All file:line citations are relative to the reference project root.
 */
#define _POSIX_C_SOURCE 200112L
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "imfit_oracle.h"
#include "fft_ref.h"
#include "qags.h"

#define DEG2RAD 0.017453292519943295 /* function_objects/func_sersic.cpp:64 */
#define SUBSAMPLE_R 10               /* function_objects/func_sersic.cpp:66 */
#define LOG_SMALL_VALUE 1.0e-25      /* core/model_object.cpp:86 */
#define COSH_LIMIT 100.0             /* function_objects/func_expdisk3d.cpp:64 */
#define EXPDISK_INTEG_MULT 20.0      /* function_objects/func_expdisk3d.cpp:66 */
#define QAGS_LIMIT 1000              /* function_objects/integrator.cpp:36 */
#define QAGS_EPSREL 1.0e-6           /* function_objects/integrator.cpp:37 */
#define MAXFUNC 64
#define MAXREGIONS 16

enum { F_SERSIC = 1, F_EXP, F_FLATSKY, F_GRING, F_MOFFAT, F_GAUSS, F_EXPDISK3D, F_FERRERS3D, F_POINTSOURCE,
       F_POINTSOURCEROT, F_TILTEDSKY };
enum { INTERP_BICUBIC = 1, INTERP_LANCZOS2 = 2, INTERP_LANCZOS3 = 3 };
#define IS_POINT_SOURCE(t) ((t) == F_POINTSOURCE || (t) == F_POINTSOURCEROT)

typedef struct {
  int type, npar, subsampling;
  double x0, y0;
  double PA, ell, q, cosPA, sinPA;
  double n, I_e, r_e, bn, invn;            /* Sersic */
  double I_0, h;                           /* Exponential, Moffat/Gaussian I_0 */
  double I_sky;                            /* FlatSky */
  double m_x, m_y;                         /* TiltedSkyPlane (I_0 above) */
  double A, R_ring, sigma_r, twosig2;      /* GaussianRing, Gaussian */
  double fwhm, beta, alpha, sigma;         /* Moffat, Gaussian */
  double inc, cosInc, sinInc, J_0, z_0, alpha3, scaledZ0, two_to_alpha; /* 3-D */
  double barPA, cosBarPA, sinBarPA, R_bar, qb, q_z, a2, b2, c2, nf, integLimit;
  double I_tot;                            /* PointSource, PointSourceRot */
  int method;                              /* requested interpolation (optional parameter "method") */
  int osScale;                             /* PointSource::oversamplingScale (state kept between calls) */
  const struct ointerp *interp;            /* the interpolator currently assigned */
} ofunc;

static int type_from_name(const char *name, int *npar) {
  struct { const char *n; int t, p; } tab[] = {
      {"Sersic", F_SERSIC, 5},           {"Exponential", F_EXP, 4},
      {"FlatSky", F_FLATSKY, 1},         {"GaussianRing", F_GRING, 5},
      {"Moffat", F_MOFFAT, 5},           {"Gaussian", F_GAUSS, 4},
      {"ExponentialDisk3D", F_EXPDISK3D, 6}, {"FerrersBar3D", F_FERRERS3D, 8},
      {"PointSource", F_POINTSOURCE, 1},     {"PointSourceRot", F_POINTSOURCEROT, 2},
      {"TiltedSkyPlane", F_TILTEDSKY, 3}};
  for (size_t i = 0; i < sizeof(tab) / sizeof(tab[0]); i++)
    if (strcmp(name, tab[i].n) == 0) {
      if (npar) *npar = tab[i].p;
      return tab[i].t;
    }
  return 0;
}

/* Calculate_bn: function_objects/helper_funcs.cpp:14-29 (Ciotti & Bertin 1999
 * for n > 0.36, MacArthur et al. 2003 polynomial below). */
static double calc_bn(double n) {
  double n2 = n * n, b_n;
  if (n > 0.36) {
    b_n = 2 * n - 0.333333333333333 + 0.009876543209876543 / n + 0.0018028610621203215 / n2 +
          0.00011409410586365319 / (n2 * n) - 7.1510122958919723e-05 / (n2 * n2);
  } else {
    b_n = 0.01945 + -0.8902 * n + 10.95 * n2 + -19.67 * n2 * n + 13.43 * n2 * n2;
  }
  return b_n;
}

/* FunctionObject::Setup for each class:
 *   Sersic        function_objects/func_sersic.cpp:109-127
 *   Exponential   function_objects/func_exp.cpp:104-119
 *   FlatSky       function_objects/func_flatsky.cpp:85-90
 *   GaussianRing  function_objects/func_gaussian-ring.cpp:102-121
 *   Moffat        function_objects/func_moffat.cpp:111-131
 *   Gaussian      function_objects/func_gaussian.cpp:104-119
 *   ExpDisk3D     function_objects/func_expdisk3d.cpp:149-171
 *   FerrersBar3D  function_objects/func_ferrersbar3d.cpp:125-165
 *   TiltedSkyPlane function_objects/func_tilted-sky-plane.cpp:85-93 */
static void func_setup(ofunc *f, const double *p, double xc, double yc) {
  f->x0 = xc;
  f->y0 = yc;
  switch (f->type) {
    case F_SERSIC:
      f->PA = p[0]; f->ell = p[1]; f->n = p[2]; f->I_e = p[3]; f->r_e = p[4];
      f->q = 1.0 - f->ell;
      f->cosPA = cos((f->PA + 90.0) * DEG2RAD);
      f->sinPA = sin((f->PA + 90.0) * DEG2RAD);
      f->bn = calc_bn(f->n);
      f->invn = 1.0 / f->n;
      break;
    case F_EXP:
      f->PA = p[0]; f->ell = p[1]; f->I_0 = p[2]; f->h = p[3];
      f->q = 1.0 - f->ell;
      f->cosPA = cos((f->PA + 90.0) * DEG2RAD);
      f->sinPA = sin((f->PA + 90.0) * DEG2RAD);
      break;
    case F_FLATSKY:
      f->I_sky = p[0];
      break;
    case F_TILTEDSKY:
      f->I_0 = p[0]; f->m_x = p[1]; f->m_y = p[2];
      break;
    case F_GRING:
      f->PA = p[0]; f->ell = p[1]; f->A = p[2]; f->R_ring = p[3]; f->sigma_r = p[4];
      f->q = 1.0 - f->ell;
      f->cosPA = cos((f->PA + 90.0) * DEG2RAD);
      f->sinPA = sin((f->PA + 90.0) * DEG2RAD);
      f->twosig2 = 2.0 * f->sigma_r * f->sigma_r;
      break;
    case F_MOFFAT: {
      f->PA = p[0]; f->ell = p[1]; f->I_0 = p[2]; f->fwhm = p[3]; f->beta = p[4];
      f->q = 1.0 - f->ell;
      f->cosPA = cos((f->PA + 90.0) * DEG2RAD);
      f->sinPA = sin((f->PA + 90.0) * DEG2RAD);
      double exponent = pow(2.0, 1.0 / f->beta);
      f->alpha = 0.5 * f->fwhm / sqrt(exponent - 1.0);
      break;
    }
    case F_GAUSS:
      f->PA = p[0]; f->ell = p[1]; f->I_0 = p[2]; f->sigma = p[3];
      f->q = 1.0 - f->ell;
      f->cosPA = cos((f->PA + 90.0) * DEG2RAD);
      f->sinPA = sin((f->PA + 90.0) * DEG2RAD);
      f->twosig2 = 2.0 * f->sigma * f->sigma;
      break;
    case F_EXPDISK3D:
      f->PA = p[0]; f->inc = p[1]; f->J_0 = p[2]; f->h = p[3]; f->n = p[4]; f->z_0 = p[5];
      f->cosPA = cos((f->PA + 90.0) * DEG2RAD);
      f->sinPA = sin((f->PA + 90.0) * DEG2RAD);
      f->cosInc = cos(f->inc * DEG2RAD);
      f->sinInc = sin(f->inc * DEG2RAD);
      f->alpha3 = 2.0 / f->n;
      f->scaledZ0 = f->alpha3 * f->z_0;
      f->two_to_alpha = pow(2.0, f->alpha3);
      break;
    case F_FERRERS3D: {
      f->PA = p[0]; f->inc = p[1]; f->barPA = p[2]; f->J_0 = p[3]; f->R_bar = p[4];
      f->qb = p[5]; f->q_z = p[6]; f->nf = p[7];
      f->cosPA = cos((f->PA + 90.0) * DEG2RAD);
      f->sinPA = sin((f->PA + 90.0) * DEG2RAD);
      f->cosBarPA = cos((f->barPA + 90.0) * DEG2RAD);
      f->sinBarPA = sin((f->barPA + 90.0) * DEG2RAD);
      f->cosInc = cos(f->inc * DEG2RAD);
      f->sinInc = sin(f->inc * DEG2RAD);
      f->a2 = f->R_bar * f->R_bar;
      f->b2 = f->qb * f->qb * f->a2;
      f->c2 = f->q_z * f->q_z * f->a2;
      double t = sqrt(f->b2) * f->sinInc;
      f->integLimit = 1.01 * ((t < f->R_bar) ? f->R_bar : t);
      break;
    }
    case F_POINTSOURCE: /* func_pointsource.cpp:206-211 */
      f->I_tot = p[0];
      break;
    case F_POINTSOURCEROT: /* func_pointsource-rot.cpp:210-221 */
      f->PA = p[0];
      f->I_tot = p[1];
      f->cosPA = cos((f->PA + 90.0) * DEG2RAD);
      f->sinPA = sin((f->PA + 90.0) * DEG2RAD);
      break;
  }
}

/* ------------------------- PSF interpolation ---------------------------- */
/* function_objects/psf_interpolators.cpp.  The PSF's pixel centres sit at
 * offsets n - (N-1)/2 from its centre; outside [-(N-1)/2, (N-1)/2] the value is 0.
 *
 * Bicubic: the reference calls GSL's gsl_interp2d_bicubic (GSL 2.x, version
 * not pinned by the reference; Ubuntu libgsl-dev in its CI).  Its published
 * method: the partial derivatives z_x, z_y, z_xy at every grid point come from
 * natural cubic splines through each grid line (z_xy = spline derivative along
 * x of z_y), and each cell is the bicubic Hermite patch matching z, z_x, z_y,
 * z_xy at its four corners; a point on an interior grid line belongs to the
 * cell above it, the last grid line to the cell below.  Restated here from
 * that description; pinned by unit_tests/unittest_psf_interpolators.t.h.
 *
 * Lanczos2/3: psf_interpolators.cpp:139-300 -- a sum over the (2n+1)^2 nearest
 * samples (FindIndex = floor(x - x_0)), weights Lanczos(dx) Lanczos(dy), and
 * the PSF read as data[ix * nColumns + iy] (x index first, as the reference
 * indexes it). */
typedef struct ointerp {
  int kind, nc, nr;
  double xb, yb;
  double *z, *zx, *zy, *zxy; /* bicubic: [row iy][col ix] */
  double *data;              /* lanczos: copy of the PSF, row-major */
} ointerp;

/* derivative of the natural cubic spline through (k, v[k*stride]), k < n, at
 * every knot, written to out[k*stride] (unit knot spacing) */
static void spline_knot_derivs(const double *v, long stride, int n, double *out) {
  double *M = (double *)calloc((size_t)n, sizeof(double));
  double *c = (double *)calloc((size_t)n, sizeof(double));
  double *d = (double *)calloc((size_t)n, sizeof(double));
  /* second derivatives M: M_0 = M_{n-1} = 0, M_{k-1} + 4 M_k + M_{k+1} = 6 (v_{k+1} - 2 v_k + v_{k-1}) */
  if (n > 2) {
    int m = n - 2;
    for (int i = 0; i < m; i++) {
      int k = i + 1;
      double rhs = 6.0 * (v[(k + 1) * stride] - 2.0 * v[k * stride] + v[(k - 1) * stride]);
      double diag = 4.0;
      if (i > 0) {
        double w = 1.0 / c[i - 1];
        diag -= w;
        rhs -= w * d[i - 1];
      }
      c[i] = diag;
      d[i] = rhs;
    }
    /* back substitution: c holds the eliminated diagonal, d the eliminated rhs */
    M[m] = d[m - 1] / c[m - 1];
    for (int i = m - 2; i >= 0; i--) M[i + 1] = (d[i] - M[i + 2]) / c[i];
  }
  for (int k = 0; k < n - 1; k++)
    out[k * stride] = (v[(k + 1) * stride] - v[k * stride]) - (2.0 * M[k] + M[k + 1]) / 6.0;
  out[(n - 1) * stride] = (v[(n - 1) * stride] - v[(n - 2) * stride]) + (M[n - 2] + 2.0 * M[n - 1]) / 6.0;
  free(M);
  free(c);
  free(d);
}

static void interp_free(ointerp *ip) {
  free(ip->z);
  free(ip->zx);
  free(ip->zy);
  free(ip->zxy);
  free(ip->data);
  memset(ip, 0, sizeof(*ip));
}

static int interp_build(ointerp *ip, int kind, const double *psf, int nc, int nr) {
  interp_free(ip);
  if (nc < 4 || nr < 4) return -2; /* model_object.cpp:356-361 */
  ip->kind = kind;
  ip->nc = nc;
  ip->nr = nr;
  ip->xb = (nc - 1) / 2.0;
  ip->yb = (nr - 1) / 2.0;
  long np = (long)nc * nr;
  if (kind == INTERP_BICUBIC) {
    ip->z = (double *)malloc(sizeof(double) * np);
    ip->zx = (double *)malloc(sizeof(double) * np);
    ip->zy = (double *)malloc(sizeof(double) * np);
    ip->zxy = (double *)malloc(sizeof(double) * np);
    memcpy(ip->z, psf, sizeof(double) * np);
    for (int r = 0; r < nr; r++) spline_knot_derivs(ip->z + (long)r * nc, 1, nc, ip->zx + (long)r * nc);
    for (int c = 0; c < nc; c++) spline_knot_derivs(ip->z + c, nc, nr, ip->zy + c);
    for (int r = 0; r < nr; r++) spline_knot_derivs(ip->zy + (long)r * nc, 1, nc, ip->zxy + (long)r * nc);
  } else {
    ip->data = (double *)malloc(sizeof(double) * np);
    memcpy(ip->data, psf, sizeof(double) * np);
  }
  return 0;
}

/* Lanczos kernel: psf_interpolators.cpp:299-309 */
static double lanczos(double x, int n) {
  const double pi = 3.14159265358979, pi2 = 9.86960440108936;
  double a = fabs(x);
  if (a < 1.0e-6) return 1.0;
  if (a > n) return 0.0;
  return (n * sin(pi * a) * sin(pi * a / n)) / (pi2 * a * a);
}

/* cubic Hermite basis on [0,1]: value weights for the left/right ends and
 * slope weights for the left/right ends */
static void hermite(double t, double *h0, double *h1, double *g0, double *g1) {
  double t2 = t * t, t3 = t2 * t;
  *h0 = 2.0 * t3 - 3.0 * t2 + 1.0;
  *h1 = -2.0 * t3 + 3.0 * t2;
  *g0 = t3 - 2.0 * t2 + t;
  *g1 = t3 - t2;
}

static double interp_value(const ointerp *ip, double x, double y) {
  if (x < -ip->xb || x > ip->xb || y < -ip->yb || y > ip->yb) return 0.0;
  if (ip->kind == INTERP_BICUBIC) {
    double fx = x + ip->xb, fy = y + ip->yb; /* grid coordinates */
    int i = (int)floor(fx), j = (int)floor(fy);
    if (i > ip->nc - 2) i = ip->nc - 2;
    if (j > ip->nr - 2) j = ip->nr - 2;
    double t = (x - (i - ip->xb)), u = (y - (j - ip->yb));
    double a0, a1, b0, b1, c0, c1, e0, e1;
    hermite(t, &a0, &a1, &b0, &b1);
    hermite(u, &c0, &c1, &e0, &e1);
    const int nc = ip->nc;
    long k00 = (long)j * nc + i, k10 = k00 + 1, k01 = k00 + nc, k11 = k01 + 1;
    double v = 0.0;
    v += ip->z[k00] * a0 * c0 + ip->z[k10] * a1 * c0 + ip->z[k01] * a0 * c1 + ip->z[k11] * a1 * c1;
    v += ip->zx[k00] * b0 * c0 + ip->zx[k10] * b1 * c0 + ip->zx[k01] * b0 * c1 + ip->zx[k11] * b1 * c1;
    v += ip->zy[k00] * a0 * e0 + ip->zy[k10] * a1 * e0 + ip->zy[k01] * a0 * e1 + ip->zy[k11] * a1 * e1;
    v += ip->zxy[k00] * b0 * e0 + ip->zxy[k10] * b1 * e0 + ip->zxy[k01] * b0 * e1 + ip->zxy[k11] * b1 * e1;
    return v;
  }
  int n = (ip->kind == INTERP_LANCZOS2) ? 2 : 3;
  int imx = (int)floor((x + ip->xb) / 1.0), imy = (int)floor((y + ip->yb) / 1.0);
  double v = 0.0;
  for (int a = -n; a <= n; a++) {
    int ix = imx + a;
    if (ix < 0 || ix >= ip->nc) continue;
    double xd = ix - ip->xb;
    for (int b = -n; b <= n; b++) {
      int iy = imy + b;
      if (iy < 0 || iy >= ip->nr) continue;
      double yd = iy - ip->yb;
      v += lanczos(x - xd, n) * lanczos(y - yd, n) * ip->data[(long)ix * ip->nc + iy];
    }
  }
  return v;
}

/* PointSource::GetValue / PointSourceRot::GetValue (func_pointsource.cpp:220-229,
 * func_pointsource-rot.cpp:229-243) */
static double point_source_value(const ofunc *f, double x, double y) {
  double xd = f->osScale * (x - f->x0), yd = f->osScale * (y - f->y0);
  if (f->type == F_POINTSOURCEROT) {
    double xp = xd * f->cosPA + yd * f->sinPA;
    double yp = -xd * f->sinPA + yd * f->cosPA;
    xd = xp;
    yd = yp;
  }
  return f->I_tot * interp_value(f->interp, xd, yd);
}

/* CalculateIntensity(r) of the 2-D radial classes */
static double radial_intensity(const ofunc *f, double r) {
  switch (f->type) {
    case F_SERSIC: /* func_sersic.cpp:134-140 */
      return f->I_e * exp(-f->bn * (pow((r / f->r_e), f->invn) - 1.0));
    case F_EXP: /* func_exp.cpp:126-129 */
      return f->I_0 * exp(-r / f->h);
    case F_GRING: { /* func_gaussian-ring.cpp:126-133 */
      double rd = fabs(r - f->R_ring);
      return f->A * exp(-(rd * rd) / f->twosig2);
    }
    case F_MOFFAT: { /* func_moffat.cpp:138-146 */
      double sr = r / f->alpha;
      return f->I_0 / pow((1.0 + sr * sr), f->beta);
    }
    case F_GAUSS: { /* func_gaussian.cpp:125-131 */
      double r2 = r * r;
      return f->I_0 * exp(-r2 / f->twosig2);
    }
  }
  return 0.0;
}

/* CalculateSubsamples: func_sersic.cpp:197-213, func_exp.cpp:181-197,
 * func_moffat.cpp:199-215, func_gaussian.cpp:182-198; GaussianRing never
 * subsamples (func_gaussian-ring.cpp:186-190). */
static int n_subsamples(const ofunc *f, double r) {
  int ns = 1;
  if (!f->subsampling || !(r < 10.0)) return 1;
  double scale, rin;
  switch (f->type) {
    case F_SERSIC: scale = f->r_e; rin = 4.0; break;
    case F_EXP: scale = f->h; rin = 3.0; break;
    case F_MOFFAT: scale = f->alpha; rin = 3.0; break;
    case F_GAUSS: scale = f->sigma; rin = 3.0; break;
    default: return 1;
  }
  if ((scale <= 1.0) && (r <= 1.0)) {
    int k = (f->type == F_SERSIC || f->type == F_EXP) ? (int)(2 * SUBSAMPLE_R / scale)
                                                      : (int)(4 * SUBSAMPLE_R / scale);
    ns = (k < 100) ? k : 100;
  } else {
    if (r <= rin) {
      ns = 2 * SUBSAMPLE_R;
    } else {
      int k = (int)(2 * SUBSAMPLE_R / r);
      ns = (k < 100) ? k : 100;
    }
  }
  return ns;
}

/* LuminosityDensity: function_objects/func_expdisk3d.cpp:226-266 */
static double expdisk3d_density(double s, void *pv) {
  const double *pp = (const double *)pv;
  double x_d0 = pp[0], y_d0 = pp[1], z_d0 = pp[2], cosInc = pp[3], sinInc = pp[4], J_0 = pp[5];
  double h = pp[6], z_0 = pp[7], scaledZ0 = pp[8], two_to_alpha = pp[9], alpha = pp[10];
  double y_d = y_d0 + s * sinInc;
  double z_d = z_d0 - s * cosInc;
  double R = sqrt(x_d0 * x_d0 + y_d * y_d);
  double z = fabs(z_d);
  double vs;
  if ((z / scaledZ0) > COSH_LIMIT)
    vs = two_to_alpha * exp(-z / z_0);
  else {
    double sech = 1.0 / cosh(z / scaledZ0);
    vs = pow(sech, alpha);
  }
  return J_0 * exp(-R / h) * vs;
}

/* LuminosityDensity_FerrersBar: function_objects/func_ferrersbar3d.cpp:230-258,
 * with Compute3dObjectCoords from function_objects/helper_funcs_3d.cpp:65-82
 * (note the reference pairs y_bar with a^2 and x_bar with b^2). */
static double ferrers3d_density(double s, void *pv) {
  const double *pp = (const double *)pv;
  double x_d0 = pp[0], y_d0 = pp[1], z_d0 = pp[2], cosInc = pp[3], sinInc = pp[4];
  double cosB = pp[5], sinB = pp[6], J_0 = pp[7], a2 = pp[8], b2 = pp[9], c2 = pp[10], n = pp[11];
  double y_d = y_d0 + s * sinInc;
  double z_d = z_d0 - s * cosInc;
  double x_bar = x_d0 * cosB + y_d * sinB;
  double y_bar = -x_d0 * sinB + y_d * cosB;
  double z_bar = fabs(z_d);
  double m2 = y_bar * y_bar / a2 + x_bar * x_bar / b2 + z_bar * z_bar / c2;
  if (m2 > 1.0) return 0.0;
  return J_0 * pow((1.0 - m2), n);
}

/* relative tolerance of the line-of-sight QAGS: the reference's 1e-6 unless a
 * test asks for a tighter "exact" value (orc_set_los_epsrel) */
static double g_los_epsrel = QAGS_EPSREL;

void orc_set_los_epsrel(double epsrel) { g_los_epsrel = (epsrel > 0.0) ? epsrel : QAGS_EPSREL; }

static double los_integral(const ofunc *f, double x, double y, int *nsub) {
  double x_diff = x - f->x0, y_diff = y - f->y0;
  double xp = x_diff * f->cosPA + y_diff * f->sinPA;
  double yp = -x_diff * f->sinPA + y_diff * f->cosPA;
  double pp[12];
  double result, abserr, lim;
  pp[0] = xp;
  pp[1] = yp * f->cosInc;
  pp[2] = yp * f->sinInc;
  pp[3] = f->cosInc;
  pp[4] = f->sinInc;
  if (f->type == F_EXPDISK3D) { /* func_expdisk3d.cpp:178-218 */
    pp[5] = f->J_0; pp[6] = f->h; pp[7] = f->z_0; pp[8] = f->scaledZ0;
    pp[9] = f->two_to_alpha; pp[10] = f->alpha3;
    lim = EXPDISK_INTEG_MULT * f->h;
    qags_integrate(expdisk3d_density, pp, -lim, lim, 0, g_los_epsrel, QAGS_LIMIT, &result, &abserr,
                   nsub, NULL);
  } else { /* func_ferrersbar3d.cpp:172-210 */
    pp[5] = f->cosBarPA; pp[6] = f->sinBarPA; pp[7] = f->J_0; pp[8] = f->a2; pp[9] = f->b2;
    pp[10] = f->c2; pp[11] = f->nf;
    lim = f->integLimit;
    qags_integrate(ferrers3d_density, pp, -lim, lim, 0, g_los_epsrel, QAGS_LIMIT, &result, &abserr,
                   nsub, NULL);
  }
  return result;
}

/* GetValue(x,y): func_sersic.cpp:147-189 (same structure in the other radial
 * classes), FlatSky func_flatsky.cpp:95-98, TiltedSkyPlane
 * func_tilted-sky-plane.cpp:98-104, 3-D classes via los_integral. */
static double func_value(const ofunc *f, double x, double y) {
  if (f->type == F_FLATSKY) return f->I_sky;
  if (f->type == F_TILTEDSKY) return f->I_0 + f->m_x * (x - f->x0) + f->m_y * (y - f->y0);
  if (f->type == F_EXPDISK3D || f->type == F_FERRERS3D) return los_integral(f, x, y, NULL);
  double x_diff = x - f->x0, y_diff = y - f->y0;
  double q = (f->type == F_FLATSKY) ? 1.0 : f->q;
  double xp = x_diff * f->cosPA + y_diff * f->sinPA;
  double yps = (-x_diff * f->sinPA + y_diff * f->cosPA) / q;
  double r = sqrt(xp * xp + yps * yps);
  int ns = n_subsamples(f, r);
  if (ns > 1) {
    double d = 1.0 / ns;
    double xs0 = x - 0.5 + 0.5 * d;
    double ys0 = y - 0.5 + 0.5 * d;
    double sum = 0.0;
    for (int ii = 0; ii < ns; ii++) {
      double xi = xs0 + ii * d;
      for (int jj = 0; jj < ns; jj++) {
        double yi = ys0 + jj * d;
        x_diff = xi - f->x0;
        y_diff = yi - f->y0;
        xp = x_diff * f->cosPA + y_diff * f->sinPA;
        yps = (-x_diff * f->sinPA + y_diff * f->cosPA) / q;
        r = sqrt(xp * xp + yps * yps);
        sum += radial_intensity(f, r);
      }
    }
    return sum / (ns * ns);
  }
  return radial_intensity(f, r);
}

/* TotalFlux: func_sersic.cpp:246-251 (Gamma from the C library), func_exp.cpp:210-213 */
static double func_total_flux(const ofunc *f) {
  if (f->type == F_SERSIC) {
    double bn2n = pow(f->bn, 2.0 * f->n);
    double L = 2 * 3.14159265358979 * f->n * exp(f->bn) * f->I_e * (f->r_e * f->r_e);
    return f->q * L * tgamma(2 * f->n) / bn2n;
  }
  if (f->type == F_EXP) return (1.0 - f->ell) * 2.0 * 3.14159265358979 * f->I_0 * f->h * f->h;
  if (IS_POINT_SOURCE(f->type)) return f->I_tot; /* func_pointsource.cpp:241-244 */
  return -1.0;
}

/* ------------------------------- Convolver ------------------------------ */
/* core/convolver.cpp:204-331 (DoFullSetup), :340-414 (ConvolveImage),
 * :421-441 (ShiftAndWrapPSF) */
typedef struct {
  int nColsImg, nRowsImg, nColsPsf, nRowsPsf, nColsPad, nRowsPad;
  long nPad, nPadC;
  double rescale;
  double *psf;      /* normalised copy */
  double *psfFFT;   /* half spectrum, interleaved */
  double *padded, *cbuf, *outbuf;
  fftref_plan2d *plan;
} oconv;

static double kahan_sum(const double *v, long n) {
  double sum = 0.0, err = 0.0, adj, tmp;
  for (long k = 0; k < n; k++) {
    adj = v[k] - err;
    tmp = sum + adj;
    err = (tmp - sum) - adj;
    sum = tmp;
  }
  return sum;
}

/* smallest 2,3,5,7-smooth integer >= n (optional padding for speed only:
 * linear convolution is unchanged by extra zero padding) */
static int smooth_at_least(int n) {
  for (int m = n;; m++) {
    int k = m;
    while (k % 2 == 0) k /= 2;
    while (k % 3 == 0) k /= 3;
    while (k % 5 == 0) k /= 5;
    while (k % 7 == 0) k /= 7;
    if (k == 1) return m;
  }
}

static int conv_setup(oconv *c, const double *psf, int ncp, int nrp, int normalize, int nci, int nri,
                      int smooth) {
  memset(c, 0, sizeof(*c));
  c->nColsPsf = ncp;
  c->nRowsPsf = nrp;
  c->nColsImg = nci;
  c->nRowsImg = nri;
  c->nColsPad = nci + ncp - 1;
  c->nRowsPad = nri + nrp - 1;
  if (smooth) {
    c->nColsPad = smooth_at_least(c->nColsPad);
    c->nRowsPad = smooth_at_least(c->nRowsPad);
  }
  c->nPad = (long)c->nColsPad * c->nRowsPad;
  c->rescale = 1.0 / c->nPad;
  c->nPadC = (long)c->nRowsPad * (c->nColsPad / 2 + 1);
  long np = (long)ncp * nrp;
  c->psf = (double *)malloc(sizeof(double) * np);
  memcpy(c->psf, psf, sizeof(double) * np);
  if (normalize) {
    double s = kahan_sum(c->psf, np);
    for (long k = 0; k < np; k++) c->psf[k] = c->psf[k] / s;
  }
  c->padded = (double *)calloc((size_t)c->nPad, sizeof(double));
  c->outbuf = (double *)calloc((size_t)c->nPad, sizeof(double));
  c->cbuf = (double *)calloc(2 * (size_t)c->nPadC, sizeof(double));
  c->psfFFT = (double *)calloc(2 * (size_t)c->nPadC, sizeof(double));
  c->plan = fftref_plan2d_create(c->nRowsPad, c->nColsPad);
  int cx = ncp / 2, cy = nrp / 2;
  for (int i = 0; i < nrp; i++)
    for (int j = 0; j < ncp; j++) {
      int dc = (c->nColsPad - cx + j) % c->nColsPad;
      int dr = (c->nRowsPad - cy + i) % c->nRowsPad;
      c->padded[(long)dr * c->nColsPad + dc] = c->psf[(long)i * ncp + j];
    }
  fftref_r2c_2d(c->plan, c->padded, c->psfFFT);
  return 0;
}

static void conv_free(oconv *c) {
  free(c->psf);
  free(c->padded);
  free(c->outbuf);
  free(c->cbuf);
  free(c->psfFFT);
  fftref_plan2d_destroy(c->plan);
}

static void conv_apply(oconv *c, double *img) {
  memset(c->padded, 0, sizeof(double) * (size_t)c->nPad);
  for (int i = 0; i < c->nRowsImg; i++)
    for (int j = 0; j < c->nColsImg; j++)
      c->padded[(long)i * c->nColsPad + j] = img[(long)i * c->nColsImg + j];
  fftref_r2c_2d(c->plan, c->padded, c->cbuf);
  for (long z = 0; z < c->nPadC; z++) {
    double a = c->cbuf[2 * z], b = c->cbuf[2 * z + 1];
    double cc = c->psfFFT[2 * z], d = c->psfFFT[2 * z + 1];
    c->cbuf[2 * z] = a * cc - b * d;
    c->cbuf[2 * z + 1] = b * cc + a * d;
  }
  fftref_c2r_2d(c->plan, c->cbuf, c->outbuf);
  for (int i = 0; i < c->nRowsImg; i++)
    for (int j = 0; j < c->nColsImg; j++)
      img[(long)i * c->nColsImg + j] = c->rescale * c->outbuf[(long)i * c->nColsPad + j];
}

/* ---------------------------- model object ------------------------------ */
typedef struct {
  int x1, y1, nBaseCols, nBaseRows, scale;
  int nPsfCols, nPsfRows, doConv;
  int nModelCols, nModelRows;
  long nModelVals;
  double subpixFrac, startOff;
  double *model;
  oconv conv;
  ointerp interp; /* bicubic, from the oversampled PSF as given (oversampled_region.cpp:181-186) */
} oregion;

struct orc_model {
  int nFunctions, nParamsTot, functionsDone;
  ofunc f[MAXFUNC];
  int setStart[MAXFUNC];
  int paramOffset[MAXFUNC], x0Index[MAXFUNC];
  int nDataCols, nDataRows, nModelCols, nModelRows, nPsfCols, nPsfRows;
  long nDataVals, nValid, nModelVals;
  int doConv, modelSetupDone, modelComputed;
  int dataValsSet, weightValsSet, maskExists, dataErrors, modelErrors, externalErrors;
  int useCash, pmlr, doBootstrap;
  double gain, rn, texp, sky, effGain, rnAduSq;
  int ncomb;
  double *data, *weight, *mask, *extra, *model, *dev;
  long *bootIdx;
  oconv conv;
  int nRegions;
  oregion reg[MAXREGIONS];
  int maxThreads;
  int fftSmooth;
  int nPointSources;
  double *psfLocal; /* AddPSFVector's copy (NormalizePSF'd when asked) */
  ointerp mainInterp;
};

orc_model *orc_create(void) {
  orc_model *m = (orc_model *)calloc(1, sizeof(orc_model));
  /* defaults: core/model_object.cpp:108-175 */
  m->dataErrors = 1;
  m->gain = 1.0;
  m->texp = m->effGain = 1.0;
  m->ncomb = 1;
  m->sky = m->rn = m->rnAduSq = 0.0;
  return m;
}

void orc_destroy(orc_model *m) {
  if (!m) return;
  free(m->data);
  free(m->weight);
  free(m->mask);
  free(m->extra);
  free(m->model);
  free(m->dev);
  free(m->bootIdx);
  free(m->psfLocal);
  interp_free(&m->mainInterp);
  if (m->doConv) conv_free(&m->conv);
  for (int i = 0; i < m->nRegions; i++) {
    free(m->reg[i].model);
    if (m->reg[i].doConv) conv_free(&m->reg[i].conv);
    interp_free(&m->reg[i].interp);
  }
  free(m);
}

void orc_set_fft_smooth(orc_model *m, int flag) { m->fftSmooth = flag ? 1 : 0; }

void orc_set_max_threads(orc_model *m, int n) {
  m->maxThreads = n;
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}

int orc_add_function(orc_model *m, const char *name, int newSet, int subsampling) {
  int np = 0;
  int t = type_from_name(name, &np);
  if (!t || m->nFunctions >= MAXFUNC) return -1;
  ofunc *f = &m->f[m->nFunctions];
  memset(f, 0, sizeof(*f));
  f->type = t;
  f->npar = np;
  f->subsampling = subsampling ? 1 : 0;
  f->method = INTERP_BICUBIC; /* func_pointsource.h:53 */
  f->osScale = 1;
  m->setStart[m->nFunctions] = (newSet || m->nFunctions == 0) ? 1 : 0;
  if (IS_POINT_SOURCE(t)) m->nPointSources++;
  m->nFunctions++;
  return 0;
}

/* PointSource optional parameter "method" (func_pointsource.cpp:140-180):
 * 1 bicubic, 2 lanczos2, 3 lanczos3.  ModelObject builds one interpolator,
 * of the first point source's kind, for all of them
 * (model_object.cpp:294-305, 345-381). */
int orc_set_point_source_method(orc_model *m, int index, int method) {
  if (index < 0 || index >= m->nFunctions || !IS_POINT_SOURCE(m->f[index].type)) return -1;
  if (method < INTERP_BICUBIC || method > INTERP_LANCZOS3) return -3;
  if (m->f[index].type == F_POINTSOURCEROT && method == INTERP_LANCZOS3) return -3;
  m->f[index].method = method;
  interp_free(&m->mainInterp);
  return 0;
}

static int ensure_main_interp(orc_model *m) {
  if (!m->nPointSources || m->mainInterp.kind) return 0;
  if (!m->psfLocal) return -1; /* model_object.cpp:349-353: no PSF image */
  int method = INTERP_BICUBIC;
  for (int n = 0; n < m->nFunctions; n++)
    if (IS_POINT_SOURCE(m->f[n].type)) {
      method = m->f[n].method;
      break;
    }
  return interp_build(&m->mainInterp, method, m->psfLocal, m->nPsfCols, m->nPsfRows);
}

/* DefineFunctionSets + PopulateParameterNames: core/model_object.cpp:387-410 */
int orc_finish_functions(orc_model *m) {
  int off = 0, x0i = 0;
  for (int n = 0; n < m->nFunctions; n++) {
    if (m->setStart[n]) {
      x0i = off;
      off += 2;
    }
    m->x0Index[n] = x0i;
    m->paramOffset[n] = off;
    off += m->f[n].npar;
  }
  m->nParamsTot = off;
  m->functionsDone = 1;
  return 0;
}

/* AddPSFVector: core/model_object.cpp:827-876 */
int orc_add_psf(orc_model *m, int ncols, int nrows, const double *psf, int normalize) {
  long np = (long)ncols * nrows;
  double s = 0.0;
  for (long i = 0; i < np; i++) {
    if (!isfinite(psf[i])) return -1;
    s += psf[i];
  }
  if (normalize && s <= 0.0) return -1;
  m->nPsfCols = ncols;
  m->nPsfRows = nrows;
  m->conv.psf = (double *)malloc(sizeof(double) * np);
  memcpy(m->conv.psf, psf, sizeof(double) * np);
  m->conv.nColsPsf = normalize; /* stash the flag until the image size is known */
  m->doConv = 1;
  free(m->psfLocal);
  m->psfLocal = (double *)malloc(sizeof(double) * np);
  memcpy(m->psfLocal, psf, sizeof(double) * np);
  if (normalize) { /* NormalizePSF: model_object.cpp:2581-2594 */
    double ks = kahan_sum(m->psfLocal, np);
    for (long k = 0; k < np; k++) m->psfLocal[k] = m->psfLocal[k] / ks;
  }
  interp_free(&m->mainInterp);
  return m->modelSetupDone ? -1 : 0;
}

/* SetupModelImage: core/model_object.cpp:488-527 */
int orc_setup_model_image(orc_model *m, int ncols, int nrows) {
  if (ncols < 1 || nrows < 1) return -1;
  m->nDataCols = ncols;
  m->nDataRows = nrows;
  m->nDataVals = (long)ncols * nrows;
  if (m->doConv) {
    m->nModelCols = ncols + 2 * m->nPsfCols;
    m->nModelRows = nrows + 2 * m->nPsfRows;
    double *psf = m->conv.psf;
    int normalize = m->conv.nColsPsf;
    conv_setup(&m->conv, psf, m->nPsfCols, m->nPsfRows, normalize, m->nModelCols, m->nModelRows, m->fftSmooth);
    free(psf);
  } else {
    m->nModelCols = ncols;
    m->nModelRows = nrows;
  }
  m->nModelVals = (long)m->nModelCols * m->nModelRows;
  m->model = (double *)calloc((size_t)m->nModelVals, sizeof(double));
  m->modelSetupDone = 1;
  return 0;
}

int orc_add_image_data(orc_model *m, const double *pix, int ncols, int nrows) {
  m->nDataVals = m->nValid = (long)ncols * nrows;
  m->data = (double *)malloc(sizeof(double) * m->nDataVals);
  memcpy(m->data, pix, sizeof(double) * m->nDataVals);
  m->dataValsSet = 1;
  return orc_setup_model_image(m, ncols, nrows);
}

/* AddImageCharacteristics: core/model_object.cpp:532-547 */
void orc_add_image_characteristics(orc_model *m, double gain, double rn, double texp, int ncomb,
                                   double sky) {
  m->gain = gain;
  m->rn = rn;
  m->texp = texp;
  m->ncomb = ncomb;
  m->sky = sky;
  m->effGain = gain * texp * ncomb;
  m->rnAduSq = rn * rn / (m->effGain * m->effGain);
}

/* AddErrorVector: core/model_object.cpp:573-619 */
int orc_add_error_vector(orc_model *m, const double *pix, int ncols, int nrows, int type) {
  long n = (long)ncols * nrows;
  if (n != m->nDataVals) return -1;
  free(m->weight);
  m->weight = (double *)malloc(sizeof(double) * n);
  memcpy(m->weight, pix, sizeof(double) * n);
  m->weightValsSet = 1;
  m->externalErrors = 1;
  switch (type) {
    case 100: for (long z = 0; z < n; z++) m->weight[z] = 1.0 / m->weight[z]; break;
    case 110: for (long z = 0; z < n; z++) m->weight[z] = 1.0 / sqrt(m->weight[z]); break;
    case 120: for (long z = 0; z < n; z++) m->weight[z] = sqrt(m->weight[z]); break;
    default: m->weightValsSet = 0; return -1;
  }
  return 0;
}

/* GenerateErrorVector: core/model_object.cpp:642-673 */
static void generate_error_vector(orc_model *m) {
  if (!m->weight) m->weight = (double *)calloc((size_t)m->nDataVals, sizeof(double));
  for (long z = 0; z < m->nDataVals; z++) {
    double tf = m->data[z] + m->sky;
    if (tf < 0.0) tf = 0.0;
    double ns = tf / m->effGain + m->ncomb * m->rnAduSq;
    m->weight[z] = 1.0 / sqrt(ns);
  }
  m->weightValsSet = 1;
}

/* GenerateExtraCashTerms: core/model_object.cpp:695-709 */
static void generate_extra_cash_terms(orc_model *m) {
  for (long z = 0; z < m->nDataVals; z++) {
    double dv = m->effGain * (m->data[z] + m->sky);
    m->extra[z] = (dv <= 0.0) ? 0.0 : dv * log(dv) - dv;
  }
}

/* AddMaskVector: core/model_object.cpp:721-787 */
int orc_add_mask_vector(orc_model *m, const double *pix, int ncols, int nrows, int type) {
  long n = (long)ncols * nrows;
  if (n != m->nDataVals) return -1;
  free(m->mask);
  m->mask = (double *)malloc(sizeof(double) * n);
  memcpy(m->mask, pix, sizeof(double) * n);
  m->nValid = 0;
  if (type == 10) {
    for (long z = 0; z < n; z++) {
      if (!isfinite(m->mask[z]) || m->mask[z] > 0.0) m->mask[z] = 0.0;
      else { m->mask[z] = 1.0; m->nValid++; }
    }
  } else if (type == 20) {
    for (long z = 0; z < n; z++) {
      if (!isfinite(m->mask[z]) || m->mask[z] < 1.0) m->mask[z] = 0.0;
      else { m->mask[z] = 1.0; m->nValid++; }
    }
  } else {
    m->maskExists = 0;
    return -1;
  }
  m->maskExists = 1;
  return 0;
}

/* UseCashStatistic / UsePoissonMLR / UseModelErrors: core/model_object.cpp:1501-1587 */
int orc_use_cash(orc_model *m) {
  m->useCash = 1;
  if (!m->weight) m->weight = (double *)calloc((size_t)m->nDataVals, sizeof(double));
  if (!m->extra) m->extra = (double *)calloc((size_t)m->nDataVals, sizeof(double));
  for (long z = 0; z < m->nDataVals; z++) m->weight[z] = 1.0;
  m->weightValsSet = 1;
  return 0;
}
void orc_use_pmlr(orc_model *m) {
  m->pmlr = 1;
  orc_use_cash(m);
}
int orc_use_model_errors(orc_model *m) {
  m->modelErrors = 1;
  m->dataErrors = 0;
  if (!m->weight) m->weight = (double *)calloc((size_t)m->nDataVals, sizeof(double));
  for (long z = 0; z < m->nDataVals; z++) m->weight[z] = 1.0;
  m->weightValsSet = 1;
  return 0;
}

/* FinalSetupForFitting: core/model_object.cpp:967-1079 (with ApplyMask
 * :794-816, CheckWeightVector :2508-2550, VetDataVector :2496-2506) */
int orc_final_setup(orc_model *m) {
  int ret = 0;
  long n = m->nDataVals;
  if (!m->maskExists) {
    m->mask = (double *)malloc(sizeof(double) * n);
    for (long z = 0; z < n; z++) m->mask[z] = 1.0;
    m->maskExists = 1;
  }
  for (long z = 0; z < n; z++)
    if (m->mask[z] > 0.0 && !isfinite(m->data[z])) {
      m->mask[z] = 0.0;
      m->nValid--;
    }
  if (!m->useCash && m->dataErrors && !m->externalErrors) generate_error_vector(m);
  if (m->useCash && m->pmlr) generate_extra_cash_terms(m);
  if (m->externalErrors) {
    for (long z = 0; z < n; z++)
      if (m->mask[z] > 0.0 && !isfinite(m->weight[z])) {
        m->mask[z] = 0.0;
        m->weight[z] = 0.0;
        m->nValid--;
      }
  }
  if (m->weightValsSet && m->maskExists) {
    for (long z = 0; z < n; z++) {
      double nv = m->mask[z] * m->weight[z];
      if (!isfinite(nv) && m->mask[z] == 0.0) nv = 0.0;
      m->weight[z] = nv;
    }
  }
  {
    int nonfinite = 0, negative = 0;
    for (long z = 0; z < n; z++)
      if (m->mask[z] > 0.0) {
        if (!isfinite(m->weight[z])) nonfinite = 1;
        else if (m->weight[z] < 0.0) negative = 1;
      }
    if (nonfinite || negative) ret = -1;
  }
  if (m->dataValsSet) {
    int bad = 0;
    for (long z = 0; z < n; z++)
      if (!isfinite(m->data[z])) {
        if (m->mask[z] > 0.0) bad = 1;
        else m->data[z] = 0.0;
      }
    if (bad) ret = -2;
  }
  if (m->nValid < 1) ret = -3;
  return ret;
}

int orc_n_params(orc_model *m) { return m->nParamsTot; }
long orc_n_data(orc_model *m) { return m->nDataVals; }
long orc_n_valid(orc_model *m) { return m->nValid; }
int orc_which_statistic(orc_model *m) {
  if (m->useCash) return m->pmlr ? 3 : 2;
  if (m->modelErrors) return 11;
  if (m->externalErrors) return 12;
  return 10;
}
int orc_model_size(orc_model *m, int *nc, int *nr) {
  *nc = m->nModelCols;
  *nr = m->nModelRows;
  return 0;
}
int orc_fft_size(orc_model *m, int *nc, int *nr) {
  *nc = m->doConv ? m->conv.nColsPad : 0;
  *nr = m->doConv ? m->conv.nRowsPad : 0;
  return 0;
}

/* AddOversampledPsfInfo: core/model_object.cpp:881-952, with
 * OversampledRegion::SetupModelImage core/oversampled_region.cpp:207-273 */
int orc_add_oversampled_psf(orc_model *m, int ncols, int nrows, const double *psf, int scale,
                            int x1, int x2, int y1, int y2, int normalize) {
  if (m->nRegions >= MAXREGIONS || !m->modelSetupDone) return -1;
  for (long i = 0; i < (long)ncols * nrows; i++)
    if (!isfinite(psf[i])) return -1;
  if (x1 < 1) x1 = 1;
  if (y1 < 1) y1 = 1;
  if (x2 > m->nDataCols) x2 = m->nDataCols;
  if (y2 > m->nDataRows) y2 = m->nDataRows;
  oregion *r = &m->reg[m->nRegions];
  memset(r, 0, sizeof(*r));
  r->x1 = x1;
  r->y1 = y1;
  r->nBaseCols = x2 - x1 + 1;
  r->nBaseRows = y2 - y1 + 1;
  r->scale = scale;
  r->subpixFrac = 1.0 / scale;
  r->startOff = 0.5 * r->subpixFrac - 0.5;
  r->nPsfCols = ncols;
  r->nPsfRows = nrows;
  r->doConv = 1;
  int nrc = r->nBaseCols * scale, nrr = r->nBaseRows * scale;
  r->nModelCols = nrc + 2 * ncols;
  r->nModelRows = nrr + 2 * nrows;
  r->nModelVals = (long)r->nModelCols * r->nModelRows;
  conv_setup(&r->conv, psf, ncols, nrows, normalize, r->nModelCols, r->nModelRows, m->fftSmooth);
  r->model = (double *)calloc((size_t)r->nModelVals, sizeof(double));
  if (ncols >= 4 && nrows >= 4) interp_build(&r->interp, INTERP_BICUBIC, psf, ncols, nrows);
  m->nRegions++;
  return 0;
}

static void setup_functions(orc_model *m, const double *params) {
  double x0 = 0.0, y0 = 0.0;
  for (int n = 0; n < m->nFunctions; n++) {
    if (m->setStart[n]) {
      x0 = params[m->x0Index[n]];
      y0 = params[m->x0Index[n] + 1];
    }
    func_setup(&m->f[n], params + m->paramOffset[n], x0, y0);
  }
}

/* Kahan sum over components: core/model_object.cpp:1158-1172 */
static inline double pixel_sum(const orc_model *m, double x, double y) {
  double s = 0.0, err = 0.0, adj, tmp;
  for (int n = 0; n < m->nFunctions; n++) {
    if (IS_POINT_SOURCE(m->f[n].type)) continue;
    adj = func_value(&m->f[n], x, y) - err;
    tmp = s + adj;
    err = (tmp - s) - adj;
    s = tmp;
  }
  return s;
}

/* DownsampleAndReplace: core/downsample.cpp:54-109 (nRows_subregion is
 * computed from the column count there; reproduced). */
static void downsample_replace(const oregion *r, double *mainImg, int nMainCols, int mainPsfCols,
                               int mainPsfRows) {
  const int nOC = r->nModelCols, scale = r->scale;
  int j1 = r->x1 - 1 + mainPsfCols;
  int i1 = r->y1 - 1 + mainPsfRows;
  int nColsSub = (int)((nOC - 2 * r->nPsfCols) / scale);
  int nRowsSub = (int)((nOC - 2 * r->nPsfRows) / scale);
  double area = scale * scale;
  for (int i = i1; i < i1 + nRowsSub; i++)
    for (int j = j1; j < j1 + nColsSub; j++) {
      int jj1 = (j - j1) * scale + r->nPsfCols;
      int ii1 = (i - i1) * scale + r->nPsfRows;
      double b = 0.0;
      for (int ii = ii1; ii < ii1 + scale; ii++)
        for (int jj = jj1; jj < jj1 + scale; jj++) b += r->model[(long)ii * nOC + jj];
      mainImg[(long)i * nMainCols + j] = b / area;
    }
}

/* Kahan sum over the point sources among functions [n0, n1) */
static inline double point_source_sum(const orc_model *m, int n0, int n1, double x, double y) {
  double s = 0.0, err = 0.0, adj, tmp;
  for (int n = n0; n < n1; n++) {
    if (!IS_POINT_SOURCE(m->f[n].type)) continue;
    adj = point_source_value(&m->f[n], x, y) - err;
    tmp = s + adj;
    err = (tmp - s) - adj;
    s = tmp;
  }
  return s;
}

/* Function set [n0, n1) (all functions, or the one of GetSingleFunctionImage)
 * on the model grid and the oversampled regions.  Point sources are added
 * after the convolution, with the ModelObject's interpolator on the main grid
 * (model_object.cpp:1183-1216) and the region's bicubic one at the region's
 * scale there (oversampled_region.cpp:363-408); each point source keeps the
 * last region's scale afterwards, as PointSource::oversamplingScale does. */
static void model_pass(orc_model *m, int n0, int n1, int convolveMain) {
  const long nmv = m->nModelVals;
  const int nmc = m->nModelCols;
  const int pr = m->doConv ? m->nPsfRows : 0, pc = m->doConv ? m->nPsfCols : 0;
  int nps = 0;
  for (int n = n0; n < n1; n++) nps += IS_POINT_SOURCE(m->f[n].type);
#pragma omp parallel for schedule(static, 10)
  for (long k = 0; k < nmv; k++) {
    long j = k % nmc, i = k / nmc;
    double y = (double)(i - pr + 1);
    double x = (double)(j - pc + 1);
    double s = 0.0, err = 0.0, adj, tmp;
    for (int n = n0; n < n1; n++) {
      if (IS_POINT_SOURCE(m->f[n].type)) continue;
      adj = func_value(&m->f[n], x, y) - err;
      tmp = s + adj;
      err = (tmp - s) - adj;
      s = tmp;
    }
    m->model[i * nmc + j] = s;
  }
  if (m->doConv && convolveMain) conv_apply(&m->conv, m->model);
  if (nps) {
    for (int n = n0; n < n1; n++)
      if (IS_POINT_SOURCE(m->f[n].type)) m->f[n].interp = &m->mainInterp;
#pragma omp parallel for schedule(static, 10)
    for (long k = 0; k < nmv; k++) {
      long j = k % nmc, i = k / nmc;
      m->model[i * nmc + j] += point_source_sum(m, n0, n1, (double)(j - pc + 1), (double)(i - pr + 1));
    }
  }
  for (int rr = 0; rr < m->nRegions; rr++) {
    oregion *r = &m->reg[rr];
    const int rmc = r->nModelCols;
#pragma omp parallel for schedule(static, 10)
    for (long k = 0; k < r->nModelVals; k++) {
      long j = k % rmc, i = k / rmc;
      double y = r->y1 + r->startOff + (i - r->nPsfRows) * r->subpixFrac;
      double x = r->x1 + r->startOff + (j - r->nPsfCols) * r->subpixFrac;
      double s = 0.0, err = 0.0, adj, tmp;
      for (int n = n0; n < n1; n++) {
        if (IS_POINT_SOURCE(m->f[n].type)) continue;
        adj = func_value(&m->f[n], x, y) - err;
        tmp = s + adj;
        err = (tmp - s) - adj;
        s = tmp;
      }
      r->model[i * rmc + j] = s;
    }
    conv_apply(&r->conv, r->model);
    if (nps) {
      for (int n = n0; n < n1; n++)
        if (IS_POINT_SOURCE(m->f[n].type)) {
          m->f[n].interp = &r->interp;
          m->f[n].osScale = r->scale;
        }
#pragma omp parallel for schedule(static, 10)
      for (long k = 0; k < r->nModelVals; k++) {
        long j = k % rmc, i = k / rmc;
        double y = r->y1 + r->startOff + (i - r->nPsfRows) * r->subpixFrac;
        double x = r->x1 + r->startOff + (j - r->nPsfCols) * r->subpixFrac;
        r->model[i * rmc + j] += point_source_sum(m, n0, n1, x, y);
      }
    }
    downsample_replace(r, m->model, nmc, pc, pr);
  }
}

/* CreateModelImage: core/model_object.cpp:1103-1229; oversampled regions via
 * OversampledRegion::ComputeRegionAndDownsample core/oversampled_region.cpp:284-430 */
void orc_create_model_image(orc_model *m, const double *params) {
  if (ensure_main_interp(m)) return;
  setup_functions(m, params);
  model_pass(m, 0, m->nFunctions, 1);
  m->modelComputed = 1;
}

/* GetSingleFunctionImage: core/model_object.cpp:1241-1336 (no convolution of
 * a point source on the main grid; the regions see this function alone). */
int orc_get_single_function_image(orc_model *m, const double *params, int index, double *out) {
  if (index < 0 || index >= m->nFunctions || !m->model) return -1;
  if (ensure_main_interp(m)) return -1;
  setup_functions(m, params);
  model_pass(m, index, index + 1, !IS_POINT_SOURCE(m->f[index].type));
  m->modelComputed = 1;
  return orc_get_model_image(m, out);
}

static inline long model_index(const orc_model *m, long z) {
  if (!m->doConv) return z;
  long row = z / m->nDataCols;
  long col = z - row * m->nDataCols;
  return (long)m->nModelCols * (m->nPsfRows + row) + m->nPsfCols + col;
}

int orc_get_model_image(orc_model *m, double *out) {
  if (!m->modelComputed) return -1;
  for (long z = 0; z < m->nDataVals; z++) out[z] = m->model[model_index(m, z)];
  return 0;
}

int orc_get_expanded_model_image(orc_model *m, double *out, long n) {
  if (!m->modelComputed || n > m->nModelVals) return -1;
  memcpy(out, m->model, sizeof(double) * n);
  return 0;
}

/* UpdateWeightVector: core/model_object.cpp:1345-1381 */
static void update_weights(orc_model *m) {
  for (long z = 0; z < m->nDataVals; z++) {
    if (!m->maskExists || m->mask[z] > 0) {
      double tf = m->model[model_index(m, z)] + m->sky;
      double ns = tf / m->effGain + m->ncomb * m->rnAduSq;
      m->weight[z] = 1.0 / sqrt(ns);
    }
  }
}

/* ComputePoissonMLRDeviate: core/model_object.cpp:1386-1401 */
static double pmlr_deviate(const orc_model *m, long i, long im) {
  double mv = m->effGain * (m->model[im] + m->sky);
  double dv = m->effGain * (m->data[i] + m->sky);
  double lm = (mv <= 0) ? LOG_SMALL_VALUE : log(mv);
  return sqrt(2.0 * m->weight[i] * fabs(mv - dv * lm + m->extra[i]));
}

/* ComputeDeviates: core/model_object.cpp:1413-1496 */
void orc_compute_deviates(orc_model *m, double *out, const double *params) {
  orc_create_model_image(m, params);
  if (m->modelErrors) update_weights(m);
  long nz = m->doBootstrap ? m->nValid : m->nDataVals;
  for (long z = 0; z < nz; z++) {
    long b = m->doBootstrap ? m->bootIdx[z] : z;
    long bm = model_index(m, b);
    if (m->pmlr)
      out[z] = pmlr_deviate(m, b, bm);
    else
      out[z] = m->weight[b] * (m->data[b] - m->model[bm]);
  }
}

/* mp_enorm: core/mp_enorm.cpp:51-122 (MINPACK enorm, three accumulators) */
static double enorm(long n, const double *x) {
  const double rdwarf = 3.834e-20, rgiant = 1.304e19;
  double s1 = 0.0, s2 = 0.0, s3 = 0.0, x1max = 0.0, x3max = 0.0, temp;
  double agiant = rgiant / (double)(int)n;
  for (long i = 0; i < n; i++) {
    double xabs = fabs(x[i]);
    if (xabs > rdwarf && xabs < agiant) {
      s2 += xabs * xabs;
      continue;
    }
    if (xabs > rdwarf) {
      if (xabs > x1max) {
        temp = x1max / xabs;
        s1 = 1.0 + s1 * temp * temp;
        x1max = xabs;
      } else {
        temp = xabs / x1max;
        s1 += temp * temp;
      }
      continue;
    }
    if (xabs > x3max) {
      temp = x3max / xabs;
      s3 = 1.0 + s3 * temp * temp;
      x3max = xabs;
    } else if (xabs != 0.0) {
      temp = xabs / x3max;
      s3 += temp * temp;
    }
  }
  if (s1 != 0.0) return x1max * sqrt(s1 + (s2 / x1max) / x1max);
  if (s2 != 0.0) {
    if (s2 >= x3max)
      temp = s2 * (1.0 + (x3max / s2) * (x3max * s3));
    else
      temp = x3max * ((s2 / x3max) + (x3max * s3));
    return sqrt(temp);
  }
  return x3max * sqrt(s3);
}

/* GetFitStatistic / ChiSquared / CashStatistic: core/model_object.cpp:1620-1775 */
double orc_get_fit_statistic(orc_model *m, const double *params) {
  long nz = m->doBootstrap ? m->nValid : m->nDataVals;
  if (!m->useCash) {
    if (!m->dev) m->dev = (double *)calloc((size_t)m->nDataVals, sizeof(double));
    orc_create_model_image(m, params);
    if (m->modelErrors) update_weights(m);
    for (long z = 0; z < nz; z++) {
      long b = m->doBootstrap ? m->bootIdx[z] : z;
      m->dev[z] = m->weight[b] * (m->data[b] - m->model[model_index(m, b)]);
    }
    double chi = enorm(nz, m->dev);
    return chi * chi;
  }
  orc_create_model_image(m, params);
  double cs = 0.0;
  for (long z = 0; z < nz; z++) {
    long b = m->doBootstrap ? m->bootIdx[z] : z;
    double mv = m->effGain * (m->model[model_index(m, b)] + m->sky);
    double dv = m->effGain * (m->data[b] + m->sky);
    double lm = (mv <= 0) ? LOG_SMALL_VALUE : log(mv);
    cs += m->weight[b] * (mv - dv * lm + m->extra[b]);
  }
  return 2.0 * cs;
}

int orc_get_weights(orc_model *m, double *out) {
  if (!m->weightValsSet) return -1;
  for (long z = 0; z < m->nDataVals; z++) out[z] = m->weight[z] * m->weight[z];
  return 0;
}
int orc_get_internal_weights(orc_model *m, double *out) {
  if (!m->weight) return -1;
  memcpy(out, m->weight, sizeof(double) * m->nDataVals);
  return 0;
}
int orc_get_mask(orc_model *m, double *out) {
  if (!m->mask) return -1;
  memcpy(out, m->mask, sizeof(double) * m->nDataVals);
  return 0;
}
int orc_get_data(orc_model *m, double *out) {
  memcpy(out, m->data, sizeof(double) * m->nDataVals);
  return 0;
}
int orc_get_extra_cash_terms(orc_model *m, double *out) {
  if (!m->extra) return -1;
  memcpy(out, m->extra, sizeof(double) * m->nDataVals);
  return 0;
}

/* ----------------------- MT19937 + bootstrap ---------------------------- */
/* Mersenne Twister MT19937 (Matsumoto & Nishimura 1998), restated from the
 * published algorithm as the reference uses it (core/mersenne_twister.cpp:60-166). */
static unsigned long mt_state[624];
static int mt_index = 625;
static void mt_seed(unsigned long s) {
  mt_state[0] = s & 0xffffffffUL;
  for (int i = 1; i < 624; i++) {
    mt_state[i] = (1812433253UL * (mt_state[i - 1] ^ (mt_state[i - 1] >> 30)) + (unsigned long)i);
    mt_state[i] &= 0xffffffffUL;
  }
  mt_index = 624;
}
static unsigned long mt_next(void) {
  static const unsigned long mag01[2] = {0x0UL, 0x9908b0dfUL};
  unsigned long y;
  if (mt_index >= 624) {
    if (mt_index == 625) mt_seed(5489UL);
    int kk;
    for (kk = 0; kk < 624 - 397; kk++) {
      y = (mt_state[kk] & 0x80000000UL) | (mt_state[kk + 1] & 0x7fffffffUL);
      mt_state[kk] = mt_state[kk + 397] ^ (y >> 1) ^ mag01[y & 0x1UL];
    }
    for (; kk < 623; kk++) {
      y = (mt_state[kk] & 0x80000000UL) | (mt_state[kk + 1] & 0x7fffffffUL);
      mt_state[kk] = mt_state[kk + (397 - 624)] ^ (y >> 1) ^ mag01[y & 0x1UL];
    }
    y = (mt_state[623] & 0x80000000UL) | (mt_state[0] & 0x7fffffffUL);
    mt_state[623] = mt_state[396] ^ (y >> 1) ^ mag01[y & 0x1UL];
    mt_index = 0;
  }
  y = mt_state[mt_index++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680UL;
  y ^= (y << 15) & 0xefc60000UL;
  y ^= (y >> 18);
  return y & 0xffffffffUL;
}
static double mt_real2(void) { return (double)mt_next() * (1.0 / 4294967296.0); }

/* UseBootstrap / MakeBootstrapSample: core/model_object.cpp:2042-2087 */
int orc_make_bootstrap_sample(orc_model *m) {
  if (!m->bootIdx) m->bootIdx = (long *)calloc((size_t)m->nValid, sizeof(long));
  for (long i = 0; i < m->nValid; i++) {
    long n;
    do {
      n = (long)floor(mt_real2() * m->nDataVals);
    } while (!(m->weight[n] > 0.0));
    m->bootIdx[i] = n;
  }
  return 0;
}
int orc_use_bootstrap(orc_model *m, unsigned long seed) {
  mt_seed(seed);
  m->doBootstrap = 1;
  return orc_make_bootstrap_sample(m);
}
long orc_get_bootstrap_indices(orc_model *m, long *out) {
  if (!m->bootIdx) return -1;
  memcpy(out, m->bootIdx, sizeof(long) * m->nValid);
  return m->nValid;
}

/* forward-difference Jacobian with mpfit's default step (solvers/mpfit.cpp:1194,1254-1258) */
int orc_fd_jacobian(orc_model *m, const double *params, double *fjac) {
  const int n = m->nParamsTot;
  const long nz = m->doBootstrap ? m->nValid : m->nDataVals;
  double *x = (double *)malloc(sizeof(double) * n);
  double *f0 = (double *)malloc(sizeof(double) * nz);
  double *f1 = (double *)malloc(sizeof(double) * nz);
  memcpy(x, params, sizeof(double) * n);
  orc_compute_deviates(m, f0, x);
  const double eps = sqrt(2.2204460e-16);
  for (int j = 0; j < n; j++) {
    double t = x[j], h = eps * fabs(t);
    if (h == 0.0) h = eps;
    x[j] = t + h;
    orc_compute_deviates(m, f1, x);
    x[j] = t;
    for (long i = 0; i < nz; i++) fjac[(size_t)j * nz + i] = (f1[i] - f0[i]) / h;
  }
  free(x);
  free(f0);
  free(f1);
  return 0;
}

/* --------------------------- single-function helpers --------------------- */
/* PsfInterpolator::GetValue of a kind (1 bicubic, 2 lanczos2, 3 lanczos3) on a
 * PSF image, at offsets (dx, dy) from its centre; n points. */
int orc_interpolate_psf(int kind, const double *psf, int ncols, int nrows, const double *dx, const double *dy,
                        long n, double *out) {
  ointerp ip;
  memset(&ip, 0, sizeof(ip));
  int st = interp_build(&ip, kind, psf, ncols, nrows);
  if (st) return st;
  for (long k = 0; k < n; k++) out[k] = interp_value(&ip, dx[k], dy[k]);
  interp_free(&ip);
  return 0;
}

double orc_lanczos(double x, int n) { return lanczos(x, n); }

double orc_function_value(const char *name, const double *params, double x0, double y0, double x,
                          double y, int subsampling) {
  ofunc f;
  memset(&f, 0, sizeof(f));
  f.type = type_from_name(name, &f.npar);
  if (!f.type) return -1.0;
  f.subsampling = subsampling;
  func_setup(&f, params, x0, y0);
  return func_value(&f, x, y);
}

double orc_function_total_flux(const char *name, const double *params) {
  ofunc f;
  memset(&f, 0, sizeof(f));
  f.type = type_from_name(name, &f.npar);
  if (!f.type) return -1.0;
  func_setup(&f, params, 0.0, 0.0);
  return func_total_flux(&f);
}

int orc_function_nparams(const char *name) {
  int np = 0;
  return type_from_name(name, &np) ? np : -1;
}

int orc_function_qags_nsub(const char *name, const double *params, double x0, double y0, double x,
                           double y) {
  ofunc f;
  memset(&f, 0, sizeof(f));
  f.type = type_from_name(name, &f.npar);
  if (f.type != F_EXPDISK3D && f.type != F_FERRERS3D) return -1;
  func_setup(&f, params, x0, y0);
  int nsub = 0;
  los_integral(&f, x, y, &nsub);
  return nsub;
}
