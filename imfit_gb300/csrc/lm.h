// lm.h -- Levenberg-Marquardt on the normal equations, FP64 on the host.
//
// The solver needs, at a parameter vector x, the statistic S = sum dev^2, the
// Gauss-Newton matrix A = J^T J and b = J^T dev of the deviates (J = d dev /
// d x).  It replaces mpfit's QR-factored LM (solvers/mpfit.cpp:551-1060) for
// callers that can supply A and b directly; mpfit's conventions are kept:
// fixed parameters, [lower, upper] limits, the relative-reduction test on the
// statistic with tolerance ftol (tested on the Gauss-Newton prediction), and
// an iteration limit.
#pragma once
#include <functional>

namespace imfit {

struct LMSettings {
  double ftol = 1e-8;    // stop when the Gauss-Newton step's predicted relative reduction of S is <= ftol
  int maxIter = 1000;    // as the reference's LM driver (solvers/levmar_fit.cpp:38)
  double noise = 1e-6;   // relative accuracy of S supplied by the evaluator
};

struct LMResult {
  int status = 0;        // 1 ftol, 2 xtol, 3 no step, 4 stalled below the S noise, 5 iteration limit, <0 error
  int nIter = 0;         // accepted steps + 1 (mpfit's niter)
  int nEval = 0;
  double stat = 0.0;     // S at the returned parameters (from the evaluator)
  double statInit = 0.0;
};

// evaluator: returns 0 on success; fills S, A (n x n, row-major) and b (n)
using JtwjEval = std::function<int(const double *x, double *S, double *A, double *b)>;

// Minimise S over the free parameters; x is updated in place.  lower/upper may
// be null (no limits); entries with lower >= upper are treated as unlimited.
int lm_minimize(int n, double *x, const int *fixed, const double *lower, const double *upper,
                const LMSettings &set, const JtwjEval &eval, LMResult &res);

// Batched form: B independent problems of n parameters advanced in lockstep,
// one evaluator call per round for all that are still running.  X: B x n (row-major) in/out;
// fixed: n flags shared by all problems (may be null); lower/upper: B x n or
// null.  The evaluator receives all B trial vectors and fills S (B), A (B x n x n)
// and b (B x n) for the problems marked active (the others are finished and
// need not be evaluated; their entries are left alone).
using JtwjBatchEval =
    std::function<int(const double *X, const unsigned char *active, double *S, double *A, double *b)>;
int lm_minimize_batch(int B, int n, double *X, const int *fixed, const double *lower, const double *upper,
                      const LMSettings &set, const JtwjBatchEval &eval, LMResult *res);

}  // namespace imfit
