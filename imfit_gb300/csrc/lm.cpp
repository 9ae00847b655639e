// lm.cpp -- Levenberg-Marquardt on the normal equations (FP64, host).
//
// The iteration is mpfit's (solvers/mpfit.cpp:551-1060, MINPACK lmder after
// More 1978, "The Levenberg-Marquardt algorithm: implementation and theory"),
// restated on the normal equations that the evaluator supplies (A = J^T J and
// b = J^T dev at x, from the GPU's forward-mode JtWJ pass) instead of a QR
// factorisation of J:
//  * scaling D = the running maximum of J's column norms sqrt(A_jj); trust
//    radius delta, initially 100 ||D x|| (mpfit's stepfactor), on the first
//    iteration cut to the first step's length;
//  * step p = -(A + par D^2)^-1 b with the damping par chosen by MINPACK's
//    lmpar iteration so that ||D p|| is within 10 % of delta (par = 0 when the
//    Gauss-Newton step is shorter), over the free parameters that have an
//    effect and are not pegged (at a limit with the gradient pointing out);
//  * limits (mpfit.cpp:802-835): the whole step is scaled by the largest
//    alpha <= 1 that keeps every parameter within its limits, and the
//    parameter that sets alpha lands exactly on its limit;
//  * ratio of actual to predicted reduction, delta and par updated by
//    lmder's rules, the step accepted when the ratio is >= 1e-4;
//  * stops: mpfit's ftol test on the actual and predicted reductions, its
//    xtol test (delta <= 1e-10 ||D x||), the iteration limit.
// Two additions for an evaluator whose statistic is FP32-summed per CTA and
// so carries rounding jitter of about 1e-7 relative (differences of S below
// that say nothing): convergence is also declared when the undamped
// Gauss-Newton step predicts a relative reduction of at most ftol -- that
// step is then taken if it does not raise S beyond the jitter -- and a step
// whose predicted reduction is below the jitter is accepted when S does not
// rise beyond it.  Stall stop: when kStallRounds consecutive rounds have not
// lowered the best S by more than the jitter / 10, the iteration stops.
#include "lm.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
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

// ----------------------------------------------------------------- trust region
constexpr double kDwarf = 2.2250738585072014e-308;  // smallest normal double
constexpr double kStepFactor = 100.0;                // mpfit's default stepfactor
constexpr double kXtol = 1e-10;                      // mpfit's default xtol

// Cholesky factor of (A + par D^2) over the active parameters (D: one entry
// per active parameter); false if not positive definite.
bool damped_factor(int n, const double *A, const std::vector<int> &act, const std::vector<double> &D, double par,
                   std::vector<double> &L) {
  const int na = (int)act.size();
  L.assign((size_t)na * na, 0.0);
  for (int i = 0; i < na; i++) {
    for (int k = 0; k < na; k++) L[(size_t)i * na + k] = A[(size_t)act[i] * n + act[k]];
    L[(size_t)i * na + i] += par * D[i] * D[i];
  }
  return cholesky(na, L);
}

// MINPACK's lmpar on the normal equations: the damping par >= 0 and the step
// p (one entry per active parameter) for which ||D p|| is within 10 % of
// delta, or par = 0 and the Gauss-Newton step when that is shorter than
// 1.1 delta.  par enters as the previous value (the iteration's start) and
// leaves as the one used.  False when no step can be formed.
bool tr_step(int n, const double *A, const double *b, const std::vector<int> &act, const std::vector<double> &D,
             double delta, double &par, std::vector<double> &p) {
  const int na = (int)act.size();
  std::vector<double> L, w(na), y(na), rhs(na);
  for (int i = 0; i < na; i++) rhs[i] = -b[act[i]];
  auto dnorm = [&](const std::vector<double> &v) {
    double t = 0.0;
    for (int i = 0; i < na; i++) t += (D[i] * v[i]) * (D[i] * v[i]);
    return std::sqrt(t);
  };
  auto wnorm2 = [&](const std::vector<double> &v, double dx) {  // w^T (L L^T)^-1 w, w = D^2 v / dx
    for (int i = 0; i < na; i++) w[i] = D[i] * D[i] * v[i] / dx;
    chol_solve(na, L, w.data(), y.data());
    double t = 0.0;
    for (int i = 0; i < na; i++) t += w[i] * y[i];
    return t;
  };
  const bool gn = lm_step(n, A, b, act, 0.0, p);
  double dxnorm = gn ? dnorm(p) : INFINITY;
  double fp = dxnorm - delta;
  if (gn && fp <= 0.1 * delta) {
    par = 0.0;
    return true;
  }
  double parl = 0.0;
  if (gn && damped_factor(n, A, act, D, 0.0, L)) {  // full rank: Newton's lower bound at par = 0
    const double t2 = wnorm2(p, dxnorm);
    if (t2 > 0.0 && std::isfinite(t2)) parl = fp / (delta * t2);
  }
  double gnorm = 0.0;
  for (int i = 0; i < na; i++) gnorm += (b[act[i]] / D[i]) * (b[act[i]] / D[i]);
  gnorm = std::sqrt(gnorm);
  double paru = gnorm / delta;
  if (paru == 0.0) paru = kDwarf / std::min(delta, 0.1);
  par = std::min(std::max(par, parl), paru);
  if (par == 0.0) par = gn ? gnorm / dxnorm : paru;
  p.assign(na, 0.0);
  bool have = false;
  for (int iter = 0; iter < 10; iter++) {
    if (par == 0.0) par = std::max(kDwarf, 0.001 * paru);
    if (!damped_factor(n, A, act, D, par, L)) {
      parl = par;
      par *= 10.0;
      continue;
    }
    chol_solve(na, L, rhs.data(), p.data());
    have = true;
    dxnorm = dnorm(p);
    const double prev = fp;
    fp = dxnorm - delta;
    if (std::fabs(fp) <= 0.1 * delta || (parl == 0.0 && fp <= prev && prev < 0.0) || iter == 9) break;
    const double parc = fp / (delta * wnorm2(p, dxnorm));
    if (fp > 0.0) parl = std::max(parl, par);
    if (fp < 0.0) paru = std::min(paru, par);
    par = std::max(parl, par + parc);
  }
  return have;
}

// One problem's state.
struct TrState {
  std::vector<double> A, b, diag;  // diag: D over all n parameters
  double S = 0.0, delta = 0.0, par = 0.0, xnorm = 0.0, sBest = 0.0;
  int stall = 0, accepted = 0;
  bool started = false, done = false, finalStep = false;
  std::vector<int> act;
  double pred = 0.0, dirder = 0.0, pnorm = 0.0;
};

// Limits of one problem (lower/upper: n entries or null).
struct Limits {
  const double *lo, *hi;
  bool limited(int j) const { return lo && hi && lo[j] < hi[j]; }
  double clamp(int j, double v) const { return limited(j) ? std::min(std::max(v, lo[j]), hi[j]) : v; }
};

// Next trial point t of problem q at x, or the problem's end (q.done, status
// returned; 0 while running).
int propose(TrState &q, int n, const double *x, double *t, const std::vector<int> &freeIdx, const Limits &lim,
            const LMSettings &set) {
  for (int j = 0; j < n; j++) t[j] = x[j];
  if (q.S < q.sBest * (1.0 - 0.1 * set.noise)) {
    q.sBest = q.S;
    q.stall = 0;
  } else if (++q.stall >= kStallRounds) {
    q.done = true;
    return 4;
  }
  // active parameters: free, with an effect, not pegged by the gradient's sign
  q.act.clear();
  for (int j : freeIdx) {
    if (!has_effect(q.A[(size_t)j * n + j], x[j], q.S)) continue;
    if (lim.limited(j)) {
      if (x[j] <= lim.lo[j] && q.b[j] > 0.0) continue;  // S decreases towards smaller x_j
      if (x[j] >= lim.hi[j] && q.b[j] < 0.0) continue;
    }
    q.act.push_back(j);
  }
  if (q.act.empty()) {
    q.done = true;
    return 1;
  }
  const int na = (int)q.act.size();
  if (!q.started) {
    q.diag.assign(n, 1.0);
    for (int j = 0; j < n; j++) {
      const double c = std::sqrt(std::max(q.A[(size_t)j * n + j], 0.0));
      if (c > 0.0 && std::isfinite(c)) q.diag[j] = c;
    }
    double xn = 0.0;
    for (int j : q.act) xn += (q.diag[j] * x[j]) * (q.diag[j] * x[j]);
    q.xnorm = std::sqrt(xn);
    q.delta = q.xnorm > 0.0 ? kStepFactor * q.xnorm : kStepFactor;
    q.started = true;
  } else {
    for (int j : q.act) q.diag[j] = std::max(q.diag[j], std::sqrt(std::max(q.A[(size_t)j * n + j], 0.0)));
  }
  auto model = [&](const double *tt) {  // the quadratic model's relative reduction for t - x
    double bd = 0.0, dad = 0.0;
    for (int i = 0; i < n; i++) {
      const double di = tt[i] - x[i];
      if (di == 0.0) continue;
      bd += q.b[i] * di;
      for (int k = 0; k < n; k++) dad += di * q.A[(size_t)i * n + k] * (tt[k] - x[k]);
    }
    return -(2.0 * bd + dad) / q.S;
  };
  std::vector<double> p;
  // convergence: the undamped Gauss-Newton step gains at most ftol
  q.finalStep = false;
  if (lm_step(n, q.A.data(), q.b.data(), q.act, 0.0, p)) {
    bool clamped = false;
    for (int k = 0; k < na; k++) {
      const int j = q.act[k];
      t[j] = lim.clamp(j, x[j] + p[k]);
      if (t[j] != x[j] + p[k]) clamped = true;
    }
    if (!clamped && model(t) <= set.ftol) {
      q.finalStep = true;
      return 0;
    }
    for (int j = 0; j < n; j++) t[j] = x[j];
  }
  std::vector<double> D(na);
  for (int k = 0; k < na; k++) D[k] = q.diag[q.act[k]];
  if (!tr_step(n, q.A.data(), q.b.data(), q.act, D, q.delta, q.par, p)) {
    q.done = true;
    return 3;
  }
  // limits: scale the whole step; the parameter that sets alpha lands on its limit
  double alpha = 1.0;
  int hit = -1;
  double hitVal = 0.0;
  for (int k = 0; k < na; k++) {
    const int j = q.act[k];
    if (!lim.limited(j) || p[k] == 0.0) continue;
    double a = 1.0;
    if (p[k] < 0.0 && x[j] + p[k] < lim.lo[j]) a = (lim.lo[j] - x[j]) / p[k];
    if (p[k] > 0.0 && x[j] + p[k] > lim.hi[j]) a = (lim.hi[j] - x[j]) / p[k];
    if (a < alpha) {
      alpha = std::max(a, 0.0);
      hit = j;
      hitVal = p[k] < 0.0 ? lim.lo[j] : lim.hi[j];
    }
  }
  double pn = 0.0, pAp = 0.0;
  for (int k = 0; k < na; k++) {
    const int j = q.act[k];
    p[k] *= alpha;
    t[j] = lim.clamp(j, x[j] + p[k]);
    pn += (D[k] * p[k]) * (D[k] * p[k]);
  }
  if (hit >= 0) t[hit] = hitVal;
  for (int i = 0; i < na; i++)
    for (int k = 0; k < na; k++) pAp += p[i] * q.A[(size_t)q.act[i] * n + q.act[k]] * p[k];
  q.pnorm = std::sqrt(pn);
  if (q.accepted == 0) q.delta = std::min(q.delta, q.pnorm);
  const double t1 = std::max(pAp, 0.0) / q.S, t2 = alpha * q.par * q.pnorm * q.pnorm / q.S;
  q.pred = t1 + 2.0 * t2;
  q.dirder = -(t1 + t2);
  return 0;
}

// Outcome of problem q's trial t (statistic St, At, bt there): accept or
// reject, update delta and par, test for convergence.  Returns the final
// status, or 0 while running.
int settle(TrState &q, int n, double *x, const double *t, double St, const double *At, const double *bt,
           const LMSettings &set) {
  if (q.finalStep) {
    q.done = true;
    if (std::isfinite(St) && St <= q.S * (1.0 + set.noise)) {
      for (int j = 0; j < n; j++) x[j] = t[j];
      q.S = St;
    }
    return 1;
  }
  const bool finite = std::isfinite(St);
  const double actred = (finite && 0.01 * St < q.S) ? 1.0 - St / q.S : -1.0;  // 0.1 fnorm1 < fnorm
  const double ratio = q.pred != 0.0 ? actred / q.pred : 0.0;
  if (ratio <= 0.25) {
    double temp = actred >= 0.0 ? 0.5 : 0.5 * q.dirder / (q.dirder + 0.5 * actred);
    if (!(0.01 * St < q.S) || temp < 0.1 || !std::isfinite(temp)) temp = 0.1;
    q.delta = temp * std::min(q.delta, q.pnorm / 0.1);
    q.par /= temp;
  } else if (q.par == 0.0 || ratio >= 0.75) {
    q.delta = q.pnorm / 0.5;
    q.par *= 0.5;
  }
  const bool accept = finite && (ratio >= 1e-4 || (q.pred < set.noise && St <= q.S * (1.0 + set.noise)));
  if (accept) {
    for (int j = 0; j < n; j++) x[j] = t[j];
    q.S = St;
    std::copy(At, At + (size_t)n * n, q.A.begin());
    std::copy(bt, bt + n, q.b.begin());
    double xn = 0.0;
    for (int j : q.act) xn += (q.diag[j] * x[j]) * (q.diag[j] * x[j]);
    q.xnorm = std::sqrt(xn);
    q.accepted++;
  }
  if (std::fabs(actred) <= set.ftol && q.pred <= set.ftol && 0.5 * ratio <= 1.0) {
    q.done = true;
    return 1;
  }
  if (q.delta <= kXtol * q.xnorm || !(q.delta > kDwarf)) {
    q.done = true;
    return 2;
  }
  if (q.accepted >= set.maxIter) {
    q.done = true;
    return 5;
  }
  return 0;
}

}  // namespace

// Host worker threads for the per-problem steps of a batch: created once per
// batch fit and woken for each phase (two per round), instead of threads
// created and joined per phase -- C5's 4096-problem fits run ~750 phases.
// run(n, f) calls f(i) for i in [0, n); the problems of a batch are
// independent (each step and acceptance touches only problem i's state).
// Small phases run on the calling thread.
class WorkPool {
 public:
  explicit WorkPool(int workers) {
    for (int t = 0; t < workers; t++) th_.emplace_back([this]() { work(); });
  }
  ~WorkPool() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    wake_.notify_all();
    for (auto &t : th_) t.join();
  }
  void run(int n, const std::function<void(int)> &f) {
    if (th_.empty() || n < kMinParallel) {
      for (int i = 0; i < n; i++) f(i);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(m_);
      task_ = &f;
      n_ = n;
      next_.store(0);
      busy_ = (int)th_.size();
      gen_++;
    }
    wake_.notify_all();
    for (int i = next_.fetch_add(1); i < n; i = next_.fetch_add(1)) f(i);
    std::unique_lock<std::mutex> lk(m_);
    idle_.wait(lk, [this]() { return busy_ == 0; });
    task_ = nullptr;
  }

 private:
  static constexpr int kMinParallel = 128;
  void work() {
    long seen = 0;
    for (;;) {
      std::unique_lock<std::mutex> lk(m_);
      wake_.wait(lk, [&]() { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
      const std::function<void(int)> *f = task_;
      const int n = n_;
      lk.unlock();
      for (int i = next_.fetch_add(1); i < n; i = next_.fetch_add(1)) (*f)(i);
      lk.lock();
      if (--busy_ == 0) idle_.notify_one();
    }
  }
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable wake_, idle_;
  const std::function<void(int)> *task_ = nullptr;
  int n_ = 0, busy_ = 0;
  long gen_ = 0;
  bool stop_ = false;
  std::atomic<int> next_{0};
};

static int pool_workers(int B) {
  if (B < 128) return 0;
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  return std::max(0, std::min(hw, 16) - 1);  // the calling thread takes part
}

int lm_minimize_batch(int B, int n, double *X, const int *fixed, const double *lower, const double *upper,
                      const LMSettings &set, const JtwjBatchEval &eval, LMResult *res) {
  auto limits = [&](int i) {
    return Limits{lower ? lower + (size_t)i * n : nullptr, upper ? upper + (size_t)i * n : nullptr};
  };
  std::vector<int> freeIdx;
  for (int j = 0; j < n; j++)
    if (!(fixed && fixed[j])) freeIdx.push_back(j);
  for (int i = 0; i < B; i++) {
    res[i] = LMResult{};
    const Limits lim = limits(i);
    for (int j = 0; j < n; j++) X[(size_t)i * n + j] = lim.clamp(j, X[(size_t)i * n + j]);
  }
  std::vector<double> S((size_t)B), A((size_t)B * n * n), b((size_t)B * n), T((size_t)B * n);
  std::vector<unsigned char> live((size_t)B, 1);
  int st = eval(X, live.data(), S.data(), A.data(), b.data());
  if (st) return st;
  std::vector<TrState> ps(B);
  for (int i = 0; i < B; i++) {
    TrState &q = ps[i];
    q.S = q.sBest = S[i];
    q.A.assign(A.begin() + (size_t)i * n * n, A.begin() + (size_t)(i + 1) * n * n);
    q.b.assign(b.begin() + (size_t)i * n, b.begin() + (size_t)(i + 1) * n);
    res[i].statInit = res[i].stat = S[i];
    res[i].nEval = 1;
    res[i].nIter = 1;
    if (freeIdx.empty()) {
      q.done = true;
      res[i].status = 1;
    }
  }
  // rounds: one trial per running problem, evaluated together; a rejected
  // trial costs a round but no iteration (as mpfit's inner loop)
  const long maxRounds = 20L * set.maxIter + 100;
  WorkPool pool(pool_workers(B));
  // the host steps visit only the problems still running (the last rounds of
  // a large batch have few; small phases run on this thread)
  std::vector<int> run;
  run.reserve(B);
  for (int i = 0; i < B; i++) live[i] = ps[i].done ? 0 : 1;
  for (long round = 0; round < maxRounds; round++) {
    run.clear();
    for (int i = 0; i < B; i++)
      if (!ps[i].done) run.push_back(i);
    if (run.empty()) break;
    const int nr = (int)run.size();
    pool.run(nr, [&](int k) {
      const int i = run[k];
      TrState &q = ps[i];
      const int s = propose(q, n, X + (size_t)i * n, T.data() + (size_t)i * n, freeIdx, limits(i), set);
      if (q.done) res[i].status = s;
    });
    bool any = false;
    for (int i : run) {
      live[i] = ps[i].done ? 0 : 1;
      any = any || live[i];
    }
    if (!any) break;
    st = eval(T.data(), live.data(), S.data(), A.data(), b.data());
    if (st) return st;
    pool.run(nr, [&](int k) {
      const int i = run[k];
      TrState &q = ps[i];
      if (!live[i]) return;
      res[i].nEval++;
      const int s = settle(q, n, X + (size_t)i * n, T.data() + (size_t)i * n, S[i], A.data() + (size_t)i * n * n,
                           b.data() + (size_t)i * n, set);
      res[i].stat = q.S;
      res[i].nIter = q.accepted + 1;
      if (q.done) res[i].status = s;
    });
    for (int i : run)
      if (ps[i].done) live[i] = 0;
  }
  for (int i = 0; i < B; i++)
    if (!ps[i].done) res[i].status = 5;
  return 0;
}

int lm_minimize(int n, double *x, const int *fixed, const double *lower, const double *upper,
                const LMSettings &set, const JtwjEval &eval, LMResult &res) {
  JtwjBatchEval one = [&eval](const double *X, const unsigned char *active, double *S, double *A, double *b) {
    return active[0] ? eval(X, S, A, b) : 0;
  };
  return lm_minimize_batch(1, n, x, fixed, lower, upper, set, one, &res);
}

}  // namespace imfit
