// lm.cpp -- Levenberg-Marquardt on the normal equations (FP64, host).
//
// One iteration: A = J^T J and b = J^T dev at x come from the evaluator (the
// GPU's forward-mode JtWJ pass); the damped system
//   (A + lambda diag(A)) d = -b
// is solved by Cholesky over the free parameters that are not held at a limit
// by the sign of the gradient; the trial point is clamped to the limits and
// accepted when it lowers S (or, below the evaluator's noise floor, when it
// does not raise it), lambda shrinks by 10 on success and grows by 10 on
// failure (Marquardt's rule, as mpfit's lmpar search ends up doing in effect).
// Convergence: the undamped Gauss-Newton step predicts a relative reduction
// of S of at most ftol (the ftol test of solvers/mpfit.cpp:943-956), or the
// parameters change by at most xtol relative.
#include "lm.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace imfit {

namespace {

// In-place Cholesky of the n x n SPD matrix M (row-major); false if not SPD.
bool cholesky(int n, std::vector<double> &M) {
  for (int j = 0; j < n; j++) {
    double d = M[j * n + j];
    for (int k = 0; k < j; k++) d -= M[j * n + k] * M[j * n + k];
    if (!(d > 0.0) || !std::isfinite(d)) return false;
    d = std::sqrt(d);
    M[j * n + j] = d;
    for (int i = j + 1; i < n; i++) {
      double s = M[i * n + j];
      for (int k = 0; k < j; k++) s -= M[i * n + k] * M[j * n + k];
      M[i * n + j] = s / d;
    }
  }
  return true;
}

void chol_solve(int n, const std::vector<double> &L, const double *rhs, double *x) {
  std::vector<double> y(n);
  for (int i = 0; i < n; i++) {
    double s = rhs[i];
    for (int k = 0; k < i; k++) s -= L[i * n + k] * y[k];
    y[i] = s / L[i * n + i];
  }
  for (int i = n - 1; i >= 0; i--) {
    double s = y[i];
    for (int k = i + 1; k < n; k++) s -= L[k * n + i] * x[k];
    x[i] = s / L[i * n + i];
  }
}

}  // namespace

int lm_minimize(int n, double *x, const int *fixed, const double *lower, const double *upper,
                const LMSettings &set, const JtwjEval &eval, LMResult &res) {
  res = LMResult{};
  auto limited = [&](int j) { return lower && upper && lower[j] < upper[j]; };
  auto clampv = [&](int j, double v) {
    if (!limited(j)) return v;
    return std::min(std::max(v, lower[j]), upper[j]);
  };
  std::vector<int> freeIdx;
  for (int j = 0; j < n; j++) {
    if (!(fixed && fixed[j])) freeIdx.push_back(j);
    x[j] = clampv(j, x[j]);
  }
  std::vector<double> A((size_t)n * n), b(n), At((size_t)n * n), bt(n), xt(n);
  double S = 0.0;
  int st = eval(x, &S, A.data(), b.data());
  res.nEval = 1;
  if (st) return res.status = st;
  res.statInit = res.stat = S;
  if (freeIdx.empty()) return res.status = 1;
  double lambda = 1e-3;

  // active free parameters: not held at a limit by the gradient's sign
  auto active = [&]() {
    std::vector<int> act;
    for (int j : freeIdx) {
      if (limited(j)) {
        if (x[j] <= lower[j] && b[j] > 0.0) continue;  // S decreases towards smaller x_j
        if (x[j] >= upper[j] && b[j] < 0.0) continue;
      }
      act.push_back(j);
    }
    return act;
  };
  // step over the active set for damping lam; returns false if not SPD
  auto solve = [&](const std::vector<int> &act, double lam, std::vector<double> &d) {
    const int na = (int)act.size();
    std::vector<double> M((size_t)na * na), rhs(na);
    for (int i = 0; i < na; i++) {
      for (int k = 0; k < na; k++) M[i * na + k] = A[(size_t)act[i] * n + act[k]];
      const double di = A[(size_t)act[i] * n + act[i]];
      M[i * na + i] = di + lam * (di > 0.0 ? di : 1e-30);
      rhs[i] = -b[act[i]];
    }
    if (!cholesky(na, M)) return false;
    d.assign(na, 0.0);
    chol_solve(na, M, rhs.data(), d.data());
    return true;
  };
  // trial point and the quadratic model's relative reduction for it
  auto trial = [&](const std::vector<int> &act, const std::vector<double> &d) {
    for (int j = 0; j < n; j++) xt[j] = x[j];
    for (size_t i = 0; i < act.size(); i++) xt[act[i]] = clampv(act[i], x[act[i]] + d[i]);
    double bd = 0.0, dad = 0.0;
    for (int i = 0; i < n; i++) {
      const double di = xt[i] - x[i];
      if (di == 0.0) continue;
      bd += b[i] * di;
      for (int k = 0; k < n; k++) dad += di * A[(size_t)i * n + k] * (xt[k] - x[k]);
    }
    return -(2.0 * bd + dad) / S;
  };

  for (int it = 0; it < set.maxIter; it++) {
    res.nIter = it + 1;
    const std::vector<int> act = active();
    if (act.empty()) return res.status = 1;
    std::vector<double> d;
    // convergence: the undamped Gauss-Newton step gains at most ftol
    if (solve(act, 0.0, d)) {
      const double pred0 = trial(act, d);
      if (pred0 <= set.ftol) {
        st = eval(xt.data(), &res.stat, At.data(), bt.data());
        res.nEval++;
        if (st) return res.status = st;
        if (res.stat <= S * (1.0 + set.noise)) {
          for (int j = 0; j < n; j++) x[j] = xt[j];
        } else {
          res.stat = S;
        }
        return res.status = 1;
      }
    }
    for (;;) {
      if (!solve(act, lambda, d)) {
        lambda *= 10.0;
        if (lambda > 1e16) return res.status = 3;
        continue;
      }
      const double pred = trial(act, d);
      double St;
      st = eval(xt.data(), &St, At.data(), bt.data());
      res.nEval++;
      if (st) return res.status = st;
      const bool better = std::isfinite(St) && (St < S || (pred < set.noise && St <= S * (1.0 + set.noise)));
      if (better) {
        double dx = 0.0;
        for (int j = 0; j < n; j++) {
          const double s = std::fabs(xt[j] - x[j]) / std::max(std::fabs(xt[j]), 1e-300);
          dx = std::max(dx, (xt[j] == x[j]) ? 0.0 : s);
          x[j] = xt[j];
        }
        const double act_red = (S - St) / S;
        S = St;
        res.stat = S;
        A.swap(At);
        b.swap(bt);
        lambda = std::max(lambda * 0.1, 1e-12);
        if (act_red >= 0.0 && act_red <= set.ftol && pred <= set.ftol) return res.status = 1;
        if (dx <= set.xtol) return res.status = 2;
        break;
      }
      lambda *= 10.0;
      if (lambda > 1e16) return res.status = 3;
    }
  }
  return res.status = 5;
}

}  // namespace imfit
