// qags_dev.cuh -- QUADPACK's QAGS (adaptive 21-point Gauss-Kronrod with
// Wynn epsilon extrapolation; Piessens, de Doncker-Kapenga, Ueberhuber &
// Kahaner 1983, routine DQAGSE) as a per-thread FP64 device function.
//
// The reference integrates its 3-D line-of-sight functions with GSL's QAGS
// (function_objects/integrator.cpp:42-55: epsabs 0, epsrel 1e-6, limit 1000).
// This restatement performs the same operations in the same order, so with
// the plain path's --fmad=false build it reproduces the reference's
// subdivision decisions and sums.  The subinterval list holds kQagsCap
// intervals: with limit 1000 the algorithm's ordering window ("top", "jup")
// equals the list size for fewer than 500 intervals, so any integral that
// needs at most kQagsCap intervals follows exactly the reference's path; an
// integral that would need more stops with status kQagsCapped (the LOS
// integrands of the supported functions need at most a few tens).
#pragma once
#include <cfloat>

#include "gk21_nodes.cuh"

namespace imfit {

constexpr int kQagsCap = 64;
constexpr int kQagsLimit = 1000;  // the reference's limit
enum QagsStatus : int {
  kQagsOk = 0, kQagsMaxIter = 1, kQagsRound = 2, kQagsSing = 3, kQagsNoConv = 4, kQagsDiverge = 5,
  kQagsCapped = 7
};

__device__ __forceinline__ double qags_panel_error(double err, double resabs, double resasc) {
  err = fabs(err);
  if (resasc != 0.0 && err != 0.0) {
    double scale = pow(200.0 * err / resasc, 1.5);
    err = (scale < 1.0) ? resasc * scale : resasc;
  }
  if (resabs > DBL_MIN / (50.0 * DBL_EPSILON)) {
    double floor_err = 50.0 * DBL_EPSILON * resabs;
    if (floor_err > err) err = floor_err;
  }
  return err;
}

// One QK21 panel on [a,b].
template <typename F>
__device__ void qags_qk21(const F &f, double a, double b, double &result, double &abserr, double &resabs,
                          double &resasc) {
  const double mid = 0.5 * (a + b);
  const double half = 0.5 * (b - a);
  const double ahalf = fabs(half);
  double flo[10], fhi[10];
  const double fmid = f(mid);
  double gauss = 0.0;
  double kron = fmid * GK21_WGK[10];
  double sabs = fabs(kron);
  for (int j = 0; j < 5; j++) {
    const int k = 2 * j + 1;
    const double dx = half * GK21_XGK[k];
    const double f1 = f(mid - dx), f2 = f(mid + dx);
    flo[k] = f1;
    fhi[k] = f2;
    gauss += GK21_WG[j] * (f1 + f2);
    kron += GK21_WGK[k] * (f1 + f2);
    sabs += GK21_WGK[k] * (fabs(f1) + fabs(f2));
  }
  for (int j = 0; j < 5; j++) {
    const int k = 2 * j;
    const double dx = half * GK21_XGK[k];
    const double f1 = f(mid - dx), f2 = f(mid + dx);
    flo[k] = f1;
    fhi[k] = f2;
    kron += GK21_WGK[k] * (f1 + f2);
    sabs += GK21_WGK[k] * (fabs(f1) + fabs(f2));
  }
  const double mean = 0.5 * kron;
  double sasc = GK21_WGK[10] * fabs(fmid - mean);
  for (int k = 0; k < 10; k++) sasc += GK21_WGK[k] * (fabs(flo[k] - mean) + fabs(fhi[k] - mean));
  const double raw_err = (kron - gauss) * half;
  result = kron * half;
  resabs = sabs * ahalf;
  resasc = sasc * ahalf;
  abserr = qags_panel_error(raw_err, resabs, resasc);
}

// Subinterval list ordered by error estimate (descending through order[]).
struct QagsList {
  int size, nrmax, imax, maxlevel;
  double lo[kQagsCap], hi[kQagsCap], area[kQagsCap], err[kQagsCap];
  int order[kQagsCap], level[kQagsCap];

  __device__ void resort() {
    const int last = size - 1;
    int nr = nrmax;
    const int im = order[nr];
    if (last < 2) {
      order[0] = 0;
      order[1] = 1;
      imax = im;
      return;
    }
    const double emax = err[im];
    while (nr > 0 && emax > err[order[nr - 1]]) {
      order[nr] = order[nr - 1];
      nr--;
    }
    const int top = (last < kQagsLimit / 2 + 2) ? last : kQagsLimit - last + 1;
    int i = nr + 1;
    while (i < top && emax < err[order[i]]) {
      order[i - 1] = order[i];
      i++;
    }
    order[i - 1] = im;
    const double emin = err[last];
    int k = top - 1;
    while (k > i - 2 && emin >= err[order[k]]) {
      order[k + 1] = order[k];
      k--;
    }
    order[k + 1] = last;
    imax = order[nr];
    nrmax = nr;
  }

  __device__ void split(double a1, double b1, double r1, double e1, double a2, double b2, double r2, double e2) {
    const int im = imax, in = size;
    const int lev = level[im] + 1;
    if (e2 > e1) {
      lo[im] = a2; area[im] = r2; err[im] = e2; level[im] = lev;
      lo[in] = a1; hi[in] = b1; area[in] = r1; err[in] = e1; level[in] = lev;
    } else {
      hi[im] = b1; area[im] = r1; err[im] = e1; level[im] = lev;
      lo[in] = a2; hi[in] = b2; area[in] = r2; err[in] = e2; level[in] = lev;
    }
    size++;
    if (lev > maxlevel) maxlevel = lev;
    resort();
  }

  __device__ int bump_nrmax() {
    const int last = size - 1;
    const int jup = (last > 1 + kQagsLimit / 2) ? kQagsLimit + 1 - last : last;
    for (int k = nrmax; k <= jup; k++) {
      const int im = order[nrmax];
      imax = im;
      if (level[im] < maxlevel) return 1;
      nrmax++;
    }
    return 0;
  }
};

struct QagsEps {
  int n;
  double tab[52];
  int nres;
  double last3[3];

  __device__ void extrapolate(double &result, double &abserr) {
    double *ep = tab;
    const int n0 = n - 1;
    const double cur = ep[n0];
    result = cur;
    abserr = DBL_MAX;
    if (n0 < 2) {
      abserr = fmax(DBL_MAX, 5.0 * DBL_EPSILON * fabs(cur));
      return;
    }
    const int newelm = n0 / 2;
    int nfin = n0;
    const int nres0 = nres;
    ep[n0 + 2] = ep[n0];
    ep[n0] = DBL_MAX;
    for (int i = 0; i < newelm; i++) {
      double res = ep[n0 - 2 * i + 2];
      const double e0 = ep[n0 - 2 * i - 2];
      const double e1 = ep[n0 - 2 * i - 1];
      const double e2 = res;
      const double d2 = e2 - e1, err2 = fabs(d2);
      const double tol2 = fmax(fabs(e2), fabs(e1)) * DBL_EPSILON;
      const double d3 = e1 - e0, err3 = fabs(d3);
      const double tol3 = fmax(fabs(e1), fabs(e0)) * DBL_EPSILON;
      if (err2 < tol2 && err3 < tol3) {
        result = res;
        abserr = fmax(err2 + err3, 5.0 * DBL_EPSILON * fabs(res));
        return;
      }
      const double e3 = ep[n0 - 2 * i];
      ep[n0 - 2 * i] = e1;
      const double d1 = e1 - e3, err1 = fabs(d1);
      const double tol1 = fmax(fabs(e1), fabs(e3)) * DBL_EPSILON;
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
      if (errn <= abserr) {
        abserr = errn;
        result = res;
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
    n = nfin + 1;
    if (nres0 < 3) {
      last3[nres0] = result;
      abserr = DBL_MAX;
    } else {
      abserr = fabs(result - last3[2]) + fabs(result - last3[1]) + fabs(result - last3[0]);
      last3[0] = last3[1];
      last3[1] = last3[2];
      last3[2] = result;
    }
    nres = nres0 + 1;
    abserr = fmax(abserr, 5.0 * DBL_EPSILON * fabs(result));
  }
};

__device__ __forceinline__ bool qags_too_small(double a1, double a2, double b2) {
  const double tmp = (1.0 + 100.0 * DBL_EPSILON) * (fabs(a2) + 1000.0 * DBL_MIN);
  return fabs(a1) <= tmp && fabs(b2) <= tmp;
}

// QAGS with epsabs = 0.  Returns a QagsStatus; result is always written.
template <typename F>
__device__ int qags_integrate(const F &f, double a, double b, double epsrel, double &result) {
  double r0, e0, rabs0, rasc0;
  result = 0.0;
  const double epsabs = 0.0;
  qags_qk21(f, a, b, r0, e0, rabs0, rasc0);
  double tol = fmax(epsabs, epsrel * fabs(r0));
  if (e0 <= 100 * DBL_EPSILON * rabs0 && e0 > tol) {
    result = r0;
    return kQagsRound;
  }
  if ((e0 <= tol && e0 != rasc0) || e0 == 0.0) {
    result = r0;
    return kQagsOk;
  }
  QagsList w;
  w.size = 1;
  w.nrmax = 0;
  w.imax = 0;
  w.maxlevel = 0;
  w.lo[0] = a;
  w.hi[0] = b;
  w.area[0] = r0;
  w.err[0] = e0;
  w.order[0] = 0;
  w.level[0] = 0;
  QagsEps tab;
  tab.n = 0;
  tab.nres = 0;
  tab.tab[tab.n++] = r0;

  double area = r0, errsum = e0;
  double res_ext = r0, err_ext = DBL_MAX;
  double correc = 0.0, ertest = 0.0, erlarge = 0.0;
  const int positive = fabs(r0) >= (1 - 50 * DBL_EPSILON) * rabs0;
  int iter = 1, ktmin = 0, extrap = 0, noext = 0;
  int round1 = 0, round2 = 0, round3 = 0;
  int ier = 0, ier2 = 0;
  bool plain = false;

  do {
    if (w.size >= kQagsCap) {
      ier = kQagsCapped;
      break;
    }
    const int im = w.imax;
    const double ai = w.lo[im], bi = w.hi[im], ri = w.area[im], ei = w.err[im];
    const int curlev = w.level[im] + 1;
    const double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    double r1, e1, rabs1, rasc1, r2, e2, rabs2, rasc2;
    iter++;
    qags_qk21(f, a1, b1, r1, e1, rabs1, rasc1);
    qags_qk21(f, a2, b2, r2, e2, rabs2, rasc2);
    const double r12 = r1 + r2, e12 = e1 + e2;
    const double last_ei = ei;
    errsum = errsum + e12 - ei;
    area = area + r12 - ri;
    tol = fmax(epsabs, epsrel * fabs(area));
    if (rasc1 != e1 && rasc2 != e2) {
      const double delta = ri - r12;
      if (fabs(delta) <= 1.0e-5 * fabs(r12) && e12 >= 0.99 * ei) {
        if (!extrap) round1++;
        else round2++;
      }
      if (iter > 10 && e12 > ei) round3++;
    }
    if (round1 + round2 >= 10 || round3 >= 20) ier = 2;
    if (round2 >= 5) ier2 = 1;
    if (qags_too_small(a1, a2, b2)) ier = 4;
    w.split(a1, b1, r1, e1, a2, b2, r2, e2);
    if (errsum <= tol) {
      plain = true;
      break;
    }
    if (ier) break;
    if (iter >= kQagsLimit - 1) {
      ier = 1;
      break;
    }
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
      if (w.level[w.imax] < w.maxlevel) continue;
      extrap = 1;
      w.nrmax = 1;
    }
    if (!ier2 && erlarge > ertest) {
      if (w.bump_nrmax()) continue;
    }
    double reseps, abseps;
    tab.tab[tab.n++] = area;
    tab.extrapolate(reseps, abseps);
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
    w.nrmax = 0;
    w.imax = w.order[0];
    extrap = 0;
    erlarge = errsum;
  } while (iter < kQagsLimit);

  if (ier == kQagsCapped) {
    double s = 0.0;
    for (int k = 0; k < w.size; k++) s += w.area[k];
    result = s;
    return kQagsCapped;
  }
  if (!plain) {
    result = res_ext;
    if (err_ext == DBL_MAX) {
      plain = true;
    } else {
      bool done = false;
      if (ier || ier2) {
        if (ier2) err_ext += correc;
        if (ier == 0) ier = 3;
        if (res_ext != 0.0 && area != 0.0) {
          if (err_ext / fabs(res_ext) > errsum / fabs(area)) plain = true;
        } else if (err_ext > errsum) {
          plain = true;
        } else if (area == 0.0) {
          done = true;
        }
      }
      if (!plain && !done) {
        const double maxarea = fmax(fabs(res_ext), fabs(area));
        if (positive || maxarea >= 0.01 * rabs0) {
          const double ratio = res_ext / area;
          if (ratio < 0.01 || ratio > 100.0 || errsum > fabs(area)) ier = 6;
        }
      }
    }
  }
  if (plain) {
    double s = 0.0;
    for (int k = 0; k < w.size; k++) s += w.area[k];
    result = s;
  }
  if (ier > 2) ier--;
  return ier;
}

}  // namespace imfit
