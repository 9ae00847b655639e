/* qags.c -- QUADPACK QAGS restated for the CPU oracle (TEST INFRASTRUCTURE
 * ONLY; see qags.h for the provenance).
 *
 * Outline of the published algorithm (DQAGSE):
 *   1. one QK21 panel over [a,b]; stop if its error estimate already meets
 *      max(epsabs, epsrel*|I|) (or is exactly zero);
 *   2. otherwise keep a list of subintervals ordered by error estimate and
 *      repeatedly bisect the one with the largest error;
 *   3. once only "small" (deepest-level) intervals carry large errors, feed
 *      the running area sequence to Wynn's epsilon algorithm and accept the
 *      extrapolated value when its error estimate meets the tolerance;
 *   4. roundoff, subdivision-limit and divergence tests decide which of the
 *      plain sum or the extrapolated value is returned.
 * The error estimate of a panel is |K21 - G10| rescaled by
 * resasc*min(1, (200*err/resasc)^1.5) and floored at 50*eps*resabs.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include "qags.h"
#include "gk21_nodes.h"

#define EPSMACH DBL_EPSILON
#define TINY DBL_MIN
#define HUGE_ DBL_MAX

static double panel_error(double err, double resabs, double resasc) {
  err = fabs(err);
  if (resasc != 0.0 && err != 0.0) {
    double scale = pow(200.0 * err / resasc, 1.5);
    err = (scale < 1.0) ? resasc * scale : resasc;
  }
  if (resabs > TINY / (50.0 * EPSMACH)) {
    double floor_err = 50.0 * EPSMACH * resabs;
    if (floor_err > err) err = floor_err;
  }
  return err;
}

void qags_qk21(qags_fn f, void *params, double a, double b, double *result, double *abserr,
               double *resabs, double *resasc) {
  const double mid = 0.5 * (a + b);
  const double half = 0.5 * (b - a);
  const double ahalf = fabs(half);
  double flo[10], fhi[10];
  const double fmid = f(mid, params);
  double gauss = 0.0;
  double kron = fmid * GK21_WGK[10];
  double sabs = fabs(kron);
  /* Gauss nodes sit at the odd positions of the abscissa table */
  for (int j = 0; j < 5; j++) {
    const int k = 2 * j + 1;
    const double dx = half * GK21_XGK[k];
    const double f1 = f(mid - dx, params), f2 = f(mid + dx, params);
    flo[k] = f1;
    fhi[k] = f2;
    gauss += GK21_WG[j] * (f1 + f2);
    kron += GK21_WGK[k] * (f1 + f2);
    sabs += GK21_WGK[k] * (fabs(f1) + fabs(f2));
  }
  for (int j = 0; j < 5; j++) {
    const int k = 2 * j;
    const double dx = half * GK21_XGK[k];
    const double f1 = f(mid - dx, params), f2 = f(mid + dx, params);
    flo[k] = f1;
    fhi[k] = f2;
    kron += GK21_WGK[k] * (f1 + f2);
    sabs += GK21_WGK[k] * (fabs(f1) + fabs(f2));
  }
  const double mean = 0.5 * kron;
  double sasc = GK21_WGK[10] * fabs(fmid - mean);
  for (int k = 0; k < 10; k++) sasc += GK21_WGK[k] * (fabs(flo[k] - mean) + fabs(fhi[k] - mean));
  const double raw_err = (kron - gauss) * half;
  *result = kron * half;
  *resabs = sabs * ahalf;
  *resasc = sasc * ahalf;
  *abserr = panel_error(raw_err, *resabs, *resasc);
}

/* ---------------- subinterval list kept ordered by error estimate -------- */
typedef struct {
  int limit, size;
  int nrmax;     /* position in order[] of the interval to bisect next */
  int imax;      /* its index */
  int maxlevel;  /* deepest bisection level seen */
  double *lo, *hi, *area, *err;
  int *order, *level;
} ivlist;

static int ivlist_init(ivlist *w, int limit, double a, double b) {
  w->limit = limit;
  w->lo = (double *)malloc(sizeof(double) * 4 * (size_t)limit);
  w->order = (int *)malloc(sizeof(int) * 2 * (size_t)limit);
  if (!w->lo || !w->order) return -1;
  w->hi = w->lo + limit;
  w->area = w->hi + limit;
  w->err = w->area + limit;
  w->level = w->order + limit;
  w->size = 0;
  w->nrmax = 0;
  w->imax = 0;
  w->maxlevel = 0;
  w->lo[0] = a;
  w->hi[0] = b;
  w->area[0] = 0.0;
  w->err[0] = 0.0;
  w->order[0] = 0;
  w->level[0] = 0;
  return 0;
}

static void ivlist_free(ivlist *w) {
  free(w->lo);
  free(w->order);
}

/* Re-establish the descending error order after interval imax was replaced
 * by its two halves (one in place, one appended at the end).  Only the first
 * 'top' entries need to be kept sorted, because that many subdivisions are
 * all that the remaining budget allows. */
static void ivlist_resort(ivlist *w) {
  const int last = w->size - 1;
  int *ord = w->order;
  const double *e = w->err;
  int nr = w->nrmax;
  const int imax = ord[nr];
  if (last < 2) {
    ord[0] = 0;
    ord[1] = 1;
    w->imax = imax;
    return;
  }
  const double emax = e[imax];
  while (nr > 0 && emax > e[ord[nr - 1]]) {
    ord[nr] = ord[nr - 1];
    nr--;
  }
  const int top = (last < w->limit / 2 + 2) ? last : w->limit - last + 1;
  int i = nr + 1;
  while (i < top && emax < e[ord[i]]) {
    ord[i - 1] = ord[i];
    i++;
  }
  ord[i - 1] = imax;
  const double emin = e[last];
  int k = top - 1;
  while (k > i - 2 && emin >= e[ord[k]]) {
    ord[k + 1] = ord[k];
    k--;
  }
  ord[k + 1] = last;
  w->imax = ord[nr];
  w->nrmax = nr;
}

static void ivlist_split(ivlist *w, double a1, double b1, double r1, double e1, double a2,
                         double b2, double r2, double e2) {
  const int im = w->imax, in = w->size;
  const int lev = w->level[im] + 1;
  if (e2 > e1) {
    /* the larger-error half stays in slot im */
    w->lo[im] = a2; w->area[im] = r2; w->err[im] = e2; w->level[im] = lev;
    w->lo[in] = a1; w->hi[in] = b1; w->area[in] = r1; w->err[in] = e1; w->level[in] = lev;
  } else {
    w->hi[im] = b1; w->area[im] = r1; w->err[im] = e1; w->level[im] = lev;
    w->lo[in] = a2; w->hi[in] = b2; w->area[in] = r2; w->err[in] = e2; w->level[in] = lev;
  }
  w->size++;
  if (lev > w->maxlevel) w->maxlevel = lev;
  ivlist_resort(w);
}

static int ivlist_bump_nrmax(ivlist *w) {
  const int last = w->size - 1;
  const int jup = (last > 1 + w->limit / 2) ? w->limit + 1 - last : last;
  for (int k = w->nrmax; k <= jup; k++) {
    const int im = w->order[w->nrmax];
    w->imax = im;
    if (w->level[im] < w->maxlevel) return 1;
    w->nrmax++;
  }
  return 0;
}

/* ---------------- Wynn epsilon table --------------------------------------- */
typedef struct {
  int n;
  double tab[52];
  int nres;
  double last3[3];
} epstable;

static void eps_extrapolate(epstable *t, double *result, double *abserr) {
  double *ep = t->tab;
  const int n0 = t->n - 1;
  const double cur = ep[n0];
  *result = cur;
  *abserr = HUGE_;
  if (n0 < 2) {
    *abserr = fmax(HUGE_, 5.0 * EPSMACH * fabs(cur));
    return;
  }
  const int newelm = n0 / 2;
  int nfin = n0;
  const int nres0 = t->nres;
  ep[n0 + 2] = ep[n0];
  ep[n0] = HUGE_;
  for (int i = 0; i < newelm; i++) {
    double res = ep[n0 - 2 * i + 2];
    const double e0 = ep[n0 - 2 * i - 2];
    const double e1 = ep[n0 - 2 * i - 1];
    const double e2 = res;
    const double d2 = e2 - e1, err2 = fabs(d2);
    const double tol2 = fmax(fabs(e2), fabs(e1)) * EPSMACH;
    const double d3 = e1 - e0, err3 = fabs(d3);
    const double tol3 = fmax(fabs(e1), fabs(e0)) * EPSMACH;
    if (err2 < tol2 && err3 < tol3) {
      /* e0, e1, e2 agree to machine accuracy: converged */
      *result = res;
      *abserr = fmax(err2 + err3, 5.0 * EPSMACH * fabs(res));
      return;
    }
    const double e3 = ep[n0 - 2 * i];
    ep[n0 - 2 * i] = e1;
    const double d1 = e1 - e3, err1 = fabs(d1);
    const double tol1 = fmax(fabs(e1), fabs(e3)) * EPSMACH;
    if (err1 < tol1 || err2 < tol2 || err3 < tol3) {
      nfin = 2 * i;
      break;
    }
    const double ss = (1.0 / d1 + 1.0 / d2) - 1.0 / d3;
    if (fabs(ss * e1) <= 1.0e-4) {
      nfin = 2 * i;
      break;
    }
    res = e1 + 1.0 / ss;
    ep[n0 - 2 * i] = res;
    const double errn = err2 + fabs(res - e2) + err3;
    if (errn <= *abserr) {
      *abserr = errn;
      *result = res;
    }
  }
  if (nfin == 49) nfin = 48;
  if (n0 % 2 == 1) {
    for (int i = 0; i <= newelm; i++) ep[1 + 2 * i] = ep[2 * i + 3];
  } else {
    for (int i = 0; i <= newelm; i++) ep[2 * i] = ep[2 * i + 2];
  }
  if (n0 != nfin) {
    for (int i = 0; i <= nfin; i++) ep[i] = ep[n0 - nfin + i];
  }
  t->n = nfin + 1;
  if (nres0 < 3) {
    t->last3[nres0] = *result;
    *abserr = HUGE_;
  } else {
    *abserr = fabs(*result - t->last3[2]) + fabs(*result - t->last3[1]) +
              fabs(*result - t->last3[0]);
    t->last3[0] = t->last3[1];
    t->last3[1] = t->last3[2];
    t->last3[2] = *result;
  }
  t->nres = nres0 + 1;
  *abserr = fmax(*abserr, 5.0 * EPSMACH * fabs(*result));
}

static int too_small(double a1, double a2, double b2) {
  const double tmp = (1.0 + 100.0 * EPSMACH) * (fabs(a2) + 1000.0 * TINY);
  return fabs(a1) <= tmp && fabs(b2) <= tmp;
}

int qags_integrate(qags_fn f, void *params, double a, double b, double epsabs, double epsrel,
                   int limit, double *result, double *abserr, int *nsub, int *neval) {
  double r0, e0, rabs0, rasc0;
  *result = 0.0;
  *abserr = 0.0;
  if (nsub) *nsub = 0;
  if (neval) *neval = 0;
  if (epsabs <= 0 && (epsrel < 50 * EPSMACH || epsrel < 0.5e-28)) return QAGS_BADTOL;

  qags_qk21(f, params, a, b, &r0, &e0, &rabs0, &rasc0);
  int nev = 21;
  double tol = fmax(epsabs, epsrel * fabs(r0));
  if (e0 <= 100 * EPSMACH * rabs0 && e0 > tol) {
    *result = r0; *abserr = e0;
    if (nsub) *nsub = 1;
    if (neval) *neval = nev;
    return QAGS_ROUND;
  }
  if ((e0 <= tol && e0 != rasc0) || e0 == 0.0) {
    *result = r0; *abserr = e0;
    if (nsub) *nsub = 1;
    if (neval) *neval = nev;
    return QAGS_OK;
  }
  if (limit == 1) {
    *result = r0; *abserr = e0;
    if (nsub) *nsub = 1;
    if (neval) *neval = nev;
    return QAGS_MAXITER;
  }

  ivlist w;
  if (ivlist_init(&w, limit, a, b) != 0) return QAGS_MAXITER;
  w.size = 1;
  w.area[0] = r0;
  w.err[0] = e0;

  epstable tab;
  tab.n = 0;
  tab.nres = 0;
  tab.tab[tab.n++] = r0;

  double area = r0, errsum = e0;
  double res_ext = r0, err_ext = HUGE_;
  double correc = 0.0, ertest = 0.0, erlarge = 0.0;
  const int positive = fabs(r0) >= (1 - 50 * EPSMACH) * rabs0;
  int iter = 1, ktmin = 0, extrap = 0, noext = 0;
  int round1 = 0, round2 = 0, round3 = 0;
  int ier = 0, ier2 = 0;
  int status;

  do {
    const int im = w.imax;
    const double ai = w.lo[im], bi = w.hi[im], ri = w.area[im], ei = w.err[im];
    const int curlev = w.level[im] + 1;
    const double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    double r1, e1, rabs1, rasc1, r2, e2, rabs2, rasc2;
    iter++;
    qags_qk21(f, params, a1, b1, &r1, &e1, &rabs1, &rasc1);
    qags_qk21(f, params, a2, b2, &r2, &e2, &rabs2, &rasc2);
    nev += 42;
    const double r12 = r1 + r2, e12 = e1 + e2;
    const double last_ei = ei;
    /* same update order as the published code so rounding agrees */
    errsum = errsum + e12 - ei;
    area = area + r12 - ri;
    tol = fmax(epsabs, epsrel * fabs(area));
    if (rasc1 != e1 && rasc2 != e2) {
      const double delta = ri - r12;
      if (fabs(delta) <= 1.0e-5 * fabs(r12) && e12 >= 0.99 * ei) {
        if (!extrap) round1++; else round2++;
      }
      if (iter > 10 && e12 > ei) round3++;
    }
    if (round1 + round2 >= 10 || round3 >= 20) ier = 2;
    if (round2 >= 5) ier2 = 1;
    if (too_small(a1, a2, b2)) ier = 4;
    ivlist_split(&w, a1, b1, r1, e1, a2, b2, r2, e2);
    if (errsum <= tol) goto plain_sum;
    if (ier) break;
    if (iter >= limit - 1) { ier = 1; break; }
    if (iter == 2) {
      erlarge = errsum;
      ertest = tol;
      tab.tab[tab.n++] = area;
      continue;
    }
    if (noext) continue;
    erlarge -= last_ei;
    if (curlev < w.maxlevel) erlarge += e12;
    if (!extrap) {
      /* keep bisecting while the worst interval is not yet a smallest one */
      if (w.level[w.imax] < w.maxlevel) continue;
      extrap = 1;
      w.nrmax = 1;
    }
    if (!ier2 && erlarge > ertest) {
      if (ivlist_bump_nrmax(&w)) continue;
    }
    /* extrapolate */
    double reseps, abseps;
    tab.tab[tab.n++] = area;
    eps_extrapolate(&tab, &reseps, &abseps);
    ktmin++;
    if (ktmin > 5 && err_ext < 1.0e-3 * errsum) ier = 5;
    if (abseps < err_ext) {
      ktmin = 0;
      err_ext = abseps;
      res_ext = reseps;
      correc = erlarge;
      ertest = fmax(epsabs, epsrel * fabs(reseps));
      if (err_ext <= ertest) break;
    }
    if (tab.n == 1) noext = 1;
    if (ier == 5) break;
    /* back to the interval with the largest error */
    w.nrmax = 0;
    w.imax = w.order[0];
    extrap = 0;
    erlarge = errsum;
  } while (iter < limit);

  *result = res_ext;
  *abserr = err_ext;
  if (err_ext == HUGE_) goto plain_sum;
  if (ier || ier2) {
    if (ier2) err_ext += correc;
    if (ier == 0) ier = 3;
    if (res_ext != 0.0 && area != 0.0) {
      if (err_ext / fabs(res_ext) > errsum / fabs(area)) goto plain_sum;
    } else if (err_ext > errsum) {
      goto plain_sum;
    } else if (area == 0.0) {
      goto done;
    }
  }
  {
    const double maxarea = fmax(fabs(res_ext), fabs(area));
    if (!positive && maxarea < 0.01 * rabs0) goto done;
  }
  {
    const double ratio = res_ext / area;
    if (ratio < 0.01 || ratio > 100.0 || errsum > fabs(area)) ier = 6;
  }
  goto done;

plain_sum:
  {
    double s = 0.0;
    for (int k = 0; k < w.size; k++) s += w.area[k];
    *result = s;
    *abserr = errsum;
  }
done:
  if (ier > 2) ier--;
  if (nsub) *nsub = w.size;
  if (neval) *neval = nev;
  ivlist_free(&w);
  switch (ier) {
    case 0: status = QAGS_OK; break;
    case 1: status = QAGS_MAXITER; break;
    case 2: status = QAGS_ROUND; break;
    case 3: status = QAGS_SING; break;
    case 4: status = QAGS_NOCONV; break;
    case 5: status = QAGS_DIVERGE; break;
    default: status = QAGS_NOCONV; break;
  }
  return status;
}
