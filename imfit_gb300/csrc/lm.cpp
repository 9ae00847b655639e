// lm.cpp -- Levenberg-Marquardt on the normal equations (FP64, host).
//
// One iteration: A = J^T J and b = J^T dev at x come from the evaluator (the
// GPU's forward-mode JtWJ pass); the damped system
//   (A + lambda diag(A)) d = -b
// is solved by Cholesky over the free parameters that have an effect and are
// not held at a limit by the sign of the gradient; the trial point is clamped
// to the limits and accepted when it lowers S (or, below the evaluator's noise
// floor, when it does not raise it).  lambda follows Nielsen's rule (Nielsen
// 1999, IMM-REP-1999-05): on success lambda *= max(1/3, 1 - (2 rho - 1)^3)
// with rho the ratio of actual to predicted reduction, on failure lambda *= nu,
// nu doubling with each consecutive failure.  Stall stop: when kStallRounds
// consecutive rounds have not lowered the best S by more than noise/10
// relative, the iteration stops (the remaining progress is below what the
// FP32-evaluated S can resolve; typically a degenerate valley or a limit).
// Convergence: the undamped Gauss-Newton step predicts a relative reduction
// of S of at most ftol (the ftol test of solvers/mpfit.cpp:943-956); that
// step is then taken.  The test is made on the Gauss-Newton prediction, which
// rests on J^T J and J^T dev (smooth in the parameters), rather than on
// differences of S between steps: the FP32-evaluated S carries rounding
// jitter of about 1e-7 relative, so near the minimum those differences say
// nothing, and a heavily damped step's tiny predicted reduction is no sign of
// convergence either.
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

// Eigen-decomposition of a small symmetric matrix (cyclic Jacobi rotations;
// Golub & Van Loan, Matrix Computations, sec. 8.5).  M is n x n row-major and
// is destroyed; on return w holds the eigenvalues and V (n x n, row-major) the
// eigenvectors as columns.
void sym_eig(int n, std::vector<double> &M, std::vector<double> &w, std::vector<double> &V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) V[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = 0.0;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) off += M[(size_t)p * n + q] * M[(size_t)p * n + q];
    if (off < 1e-30) break;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = M[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double app = M[(size_t)p * n + p], aqq = M[(size_t)q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) {
          const double mkp = M[(size_t)k * n + p], mkq = M[(size_t)k * n + q];
          M[(size_t)k * n + p] = c * mkp - s * mkq;
          M[(size_t)k * n + q] = s * mkp + c * mkq;
        }
        for (int k = 0; k < n; k++) {
          const double mpk = M[(size_t)p * n + k], mqk = M[(size_t)q * n + k];
          M[(size_t)p * n + k] = c * mpk - s * mqk;
          M[(size_t)q * n + k] = s * mpk + c * mqk;
        }
        for (int k = 0; k < n; k++) {
          const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vkp - s * vkq;
          V[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; i++) w[i] = M[(size_t)i * n + i];
}

// Step over the active parameters for damping lam, in Marquardt's diagonal
// scaling: with D = diag(A), solve (C + lam I) y = -D^-1/2 b for
// C = D^-1/2 A D^-1/2 (unit diagonal), d = D^-1/2 y.  lam > 0: Cholesky.
// lam = 0 (Gauss-Newton): the minimum-norm solution over the eigen-directions
// of C above kEigFloor of its largest eigenvalue, so parameter combinations
// the data do not determine (a faint component's shape, a position angle at
// zero ellipticity) get no step instead of a huge one -- the effect of the
// column-pivoted QR in MINPACK-style LM.  Returns false if nothing is
// determined (or, for lam > 0, the system is not positive definite).
constexpr double kPivotFloor = 1e-10;
constexpr double kEigFloor = 1e-9;

// A parameter "has an effect" when moving it by max(|x|, 1) would change S by
// more than 1e-12 S in the Gauss-Newton model (an ellipticity of 0 leaves the
// position angle without one; FP32 sums leave such a row tiny, not zero).
constexpr int kStallRounds = 20;

inline bool has_effect(double Ajj, double xj, double S) {
  const double s = std::max(std::fabs(xj), 1.0);
  return Ajj > 0.0 && std::isfinite(Ajj) && Ajj * s * s > 1e-12 * S;
}

// Nielsen's damping update after a step with gain ratio rho (success) or a failure.
inline void nielsen(bool success, double rho, double &lambda, double &nu) {
  if (success) {
    const double t = 2.0 * rho - 1.0;
    lambda *= std::max(1.0 / 3.0, 1.0 - t * t * t);
    lambda = std::max(lambda, 1e-15);
    nu = 2.0;
  } else {
    lambda *= nu;
    nu *= 2.0;
  }
}

bool lm_step(int n, const double *A, const double *b, const std::vector<int> &act, double lam,
             std::vector<double> &d) {
  const int na = (int)act.size();
  std::vector<double> M((size_t)na * na), rhs(na), sc(na);
  for (int i = 0; i < na; i++) {
    const double di = A[(size_t)act[i] * n + act[i]];
    if (!(di > 0.0) || !std::isfinite(di)) return false;
    sc[i] = 1.0 / std::sqrt(di);
  }
  for (int i = 0; i < na; i++) {
    for (int k = 0; k < na; k++) M[i * na + k] = A[(size_t)act[i] * n + act[k]] * sc[i] * sc[k];
    M[i * na + i] = 1.0 + lam;
    rhs[i] = -b[act[i]] * sc[i];
  }
  std::vector<double> y(na, 0.0);
  if (lam > 0.0) {
    if (!cholesky(na, M)) return false;
    for (int i = 0; i < na; i++)
      if (M[i * na + i] * M[i * na + i] < kPivotFloor * (1.0 + lam)) return false;
    chol_solve(na, M, rhs.data(), y.data());
  } else {
    std::vector<double> w, V;
    sym_eig(na, M, w, V);
    double wmax = 0.0;
    for (double v : w) wmax = std::max(wmax, v);
    if (!(wmax > 0.0)) return false;
    for (int k = 0; k < na; k++) {
      if (!(w[k] > kEigFloor * wmax)) continue;
      double proj = 0.0;
      for (int i = 0; i < na; i++) proj += V[(size_t)i * na + k] * rhs[i];
      proj /= w[k];
      for (int i = 0; i < na; i++) y[i] += V[(size_t)i * na + k] * proj;
    }
  }
  d.assign(na, 0.0);
  for (int i = 0; i < na; i++) d[i] = y[i] * sc[i];
  return true;
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
  double lambda = 1e-3, nu = 2.0;

  // active free parameters: with an effect on S (A_jj > 0) and not held at a
  // limit by the gradient's sign
  auto active = [&]() {
    std::vector<int> act;
    for (int j : freeIdx) {
      if (!has_effect(A[(size_t)j * n + j], x[j], S)) continue;
      if (limited(j)) {
        if (x[j] <= lower[j] && b[j] > 0.0) continue;  // S decreases towards smaller x_j
        if (x[j] >= upper[j] && b[j] < 0.0) continue;
      }
      act.push_back(j);
    }
    return act;
  };
  auto solve = [&](const std::vector<int> &act, double lam, std::vector<double> &d) {
    return lm_step(n, A.data(), b.data(), act, lam, d);
  };
  // trial point and the quadratic model's relative reduction for it; clamped
  // reports whether a limit cut the step
  bool clamped = false;
  auto trial = [&](const std::vector<int> &act, const std::vector<double> &d) {
    clamped = false;
    for (int j = 0; j < n; j++) xt[j] = x[j];
    for (size_t i = 0; i < act.size(); i++) {
      xt[act[i]] = clampv(act[i], x[act[i]] + d[i]);
      if (xt[act[i]] != x[act[i]] + d[i]) clamped = true;
    }
    double bd = 0.0, dad = 0.0;
    for (int i = 0; i < n; i++) {
      const double di = xt[i] - x[i];
      if (di == 0.0) continue;
      bd += b[i] * di;
      for (int k = 0; k < n; k++) dad += di * A[(size_t)i * n + k] * (xt[k] - x[k]);
    }
    return -(2.0 * bd + dad) / S;
  };

  double sBest = S;
  int stall = 0;
  for (int it = 0; it < set.maxIter; it++) {
    res.nIter = it + 1;
    if (S < sBest * (1.0 - 0.1 * set.noise)) {
      sBest = S;
      stall = 0;
    } else if (++stall >= kStallRounds) {
      return res.status = 4;
    }
    const std::vector<int> act = active();
    if (act.empty()) return res.status = 1;
    std::vector<double> d;
    // convergence: the undamped Gauss-Newton step gains at most ftol
    if (solve(act, 0.0, d)) {
      const double pred0 = trial(act, d);
      if (pred0 <= set.ftol && !clamped) {
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
        nielsen(false, 0.0, lambda, nu);
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
        const double rho = (pred > set.noise) ? (S - St) / (pred * S) : 1.0;
        for (int j = 0; j < n; j++) x[j] = xt[j];
        S = St;
        res.stat = S;
        A.swap(At);
        b.swap(bt);
        nielsen(true, rho, lambda, nu);
        break;
      }
      nielsen(false, 0.0, lambda, nu);
      if (lambda > 1e16) return res.status = 3;
    }
  }
  return res.status = 5;
}

}  // namespace imfit

namespace imfit {

namespace {

// One problem's state in the lockstep batch.
struct LMState {
  std::vector<double> A, b;
  double S = 0.0, lambda = 1e-3, nu = 2.0;
  double sBest = 0.0;
  int stall = 0;
  bool done = false, finalStep = false;
  double pred = 0.0;
  std::vector<int> act;
  std::vector<double> step;  // trial - x over all n
};

}  // namespace

int lm_minimize_batch(int B, int n, double *X, const int *fixed, const double *lower, const double *upper,
                      const LMSettings &set, const JtwjBatchEval &eval, LMResult *res) {
  auto limited = [&](int i, int j) { return lower && upper && lower[(size_t)i * n + j] < upper[(size_t)i * n + j]; };
  auto clampv = [&](int i, int j, double v) {
    if (!limited(i, j)) return v;
    return std::min(std::max(v, lower[(size_t)i * n + j]), upper[(size_t)i * n + j]);
  };
  std::vector<int> freeIdx;
  for (int j = 0; j < n; j++)
    if (!(fixed && fixed[j])) freeIdx.push_back(j);
  for (int i = 0; i < B; i++) {
    res[i] = LMResult{};
    for (int j = 0; j < n; j++) X[(size_t)i * n + j] = clampv(i, j, X[(size_t)i * n + j]);
  }
  std::vector<double> S((size_t)B), A((size_t)B * n * n), b((size_t)B * n), T((size_t)B * n);
  std::vector<unsigned char> live((size_t)B, 1);
  int st = eval(X, live.data(), S.data(), A.data(), b.data());
  if (st) return st;
  std::vector<LMState> ps(B);
  for (int i = 0; i < B; i++) {
    ps[i].S = S[i];
    ps[i].sBest = S[i];
    ps[i].A.assign(A.begin() + (size_t)i * n * n, A.begin() + (size_t)(i + 1) * n * n);
    ps[i].b.assign(b.begin() + (size_t)i * n, b.begin() + (size_t)(i + 1) * n);
    res[i].statInit = res[i].stat = S[i];
    res[i].nEval = 1;
    if (freeIdx.empty()) {
      ps[i].done = true;
      res[i].status = 1;
    }
  }
  // damped (lam > 0) or Gauss-Newton (lam = 0) step of problem i over its active set
  auto solve = [&](int i, double lam, std::vector<double> &d) {
    return lm_step(n, ps[i].A.data(), ps[i].b.data(), ps[i].act, lam, d);
  };
  // trial vector of problem i into T, returns the model's relative reduction;
  // clamped reports whether a limit cut the step
  bool clamped = false;
  auto trial = [&](int i, const std::vector<double> &d) {
    LMState &q = ps[i];
    const double *x = X + (size_t)i * n;
    double *t = T.data() + (size_t)i * n;
    clamped = false;
    for (int j = 0; j < n; j++) t[j] = x[j];
    for (size_t k = 0; k < q.act.size(); k++) {
      t[q.act[k]] = clampv(i, q.act[k], x[q.act[k]] + d[k]);
      if (t[q.act[k]] != x[q.act[k]] + d[k]) clamped = true;
    }
    double bd = 0.0, dad = 0.0;
    for (int r = 0; r < n; r++) {
      const double dr = t[r] - x[r];
      if (dr == 0.0) continue;
      bd += q.b[r] * dr;
      for (int c = 0; c < n; c++) dad += dr * q.A[(size_t)r * n + c] * (t[c] - x[c]);
    }
    return -(2.0 * bd + dad) / q.S;
  };

  for (int it = 0; it < set.maxIter; it++) {
    bool any = false;
    for (int i = 0; i < B; i++) {
      LMState &q = ps[i];
      double *t = T.data() + (size_t)i * n;
      for (int j = 0; j < n; j++) t[j] = X[(size_t)i * n + j];
      if (q.done) continue;
      if (q.S < q.sBest * (1.0 - 0.1 * set.noise)) {
        q.sBest = q.S;
        q.stall = 0;
      } else if (++q.stall >= kStallRounds) {
        q.done = true;
        res[i].status = 4;
        continue;
      }
      any = true;
      res[i].nIter = it + 1;
      // active parameters: free and not held at a limit by the gradient's sign
      q.act.clear();
      for (int j : freeIdx) {
        const double xj = X[(size_t)i * n + j];
        if (!has_effect(q.A[(size_t)j * n + j], xj, q.S)) continue;
        if (limited(i, j)) {
          if (xj <= lower[(size_t)i * n + j] && q.b[j] > 0.0) continue;
          if (xj >= upper[(size_t)i * n + j] && q.b[j] < 0.0) continue;
        }
        q.act.push_back(j);
      }
      if (q.act.empty()) {
        q.done = true;
        res[i].status = 1;
        continue;
      }
      std::vector<double> d;
      q.finalStep = false;
      if (solve(i, 0.0, d)) {
        const double pred0 = trial(i, d);
        if (pred0 <= set.ftol && !clamped) {
          q.finalStep = true;
          continue;
        }
      }
      bool ok = false;
      while (!ok) {
        ok = solve(i, q.lambda, d);
        if (!ok) {
          nielsen(false, 0.0, q.lambda, q.nu);
          if (q.lambda > 1e16) break;
        }
      }
      if (!ok) {
        for (int j = 0; j < n; j++) t[j] = X[(size_t)i * n + j];
        q.done = true;
        res[i].status = 3;
        continue;
      }
      q.pred = trial(i, d);
    }
    if (!any) break;
    for (int i = 0; i < B; i++) live[i] = ps[i].done ? 0 : 1;
    st = eval(T.data(), live.data(), S.data(), A.data(), b.data());
    if (st) return st;
    for (int i = 0; i < B; i++) {
      LMState &q = ps[i];
      if (q.done) continue;
      res[i].nEval++;
      double *x = X + (size_t)i * n;
      const double *t = T.data() + (size_t)i * n;
      const double St = S[i];
      const bool better = std::isfinite(St) &&
                          (St < q.S || ((q.finalStep || q.pred < set.noise) && St <= q.S * (1.0 + set.noise)));
      if (q.finalStep) {
        if (better) {
          for (int j = 0; j < n; j++) x[j] = t[j];
          q.S = St;
        }
        res[i].stat = q.S;
        res[i].status = 1;
        q.done = true;
        continue;
      }
      if (better) {
        const double rho = (q.pred > set.noise) ? (q.S - St) / (q.pred * q.S) : 1.0;
        for (int j = 0; j < n; j++) x[j] = t[j];
        q.S = St;
        res[i].stat = St;
        q.A.assign(A.begin() + (size_t)i * n * n, A.begin() + (size_t)(i + 1) * n * n);
        q.b.assign(b.begin() + (size_t)i * n, b.begin() + (size_t)(i + 1) * n);
        nielsen(true, rho, q.lambda, q.nu);
      } else {
        nielsen(false, 0.0, q.lambda, q.nu);
        if (q.lambda > 1e16) {
          q.done = true;
          res[i].status = 3;
        }
      }
    }
  }
  for (int i = 0; i < B; i++)
    if (!ps[i].done) res[i].status = 5;
  return 0;
}

}  // namespace imfit
