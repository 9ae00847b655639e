"""CPU tests of the library's Levenberg-Marquardt driver (the trust-region
iteration of solvers/mpfit.cpp on normal equations) through
imfit_MinimizeNormalEquations, on least-squares problems with analytic
Jacobians, against scipy's least_squares."""
import numpy as np
import pytest

scipy_opt = pytest.importorskip("scipy.optimize")


def _lm():
    from imfit_gb300 import minimize_normal_equations
    return minimize_normal_equations


def _normal(dev, jac):
    def fun(x):
        d, J = dev(x), jac(x)
        return float(d @ d), J.T @ J, J.T @ d
    return fun


def _decay_problem(seed=3):
    rng = np.random.default_rng(seed)
    t = np.linspace(0.0, 10.0, 200)
    truth = np.array([5.0, 0.7, 0.5])
    sig = 0.05
    y = truth[0] * np.exp(-truth[1] * t) + truth[2] + rng.normal(0.0, sig, t.size)

    def model(x):
        return x[0] * np.exp(-x[1] * t) + x[2]

    def dev(x):
        return (y - model(x)) / sig

    def jac(x):
        e = np.exp(-x[1] * t)
        return -np.stack([e, -x[0] * t * e, np.ones_like(t)], axis=1) / sig

    return dev, jac, truth


def test_far_start_reaches_the_least_squares_minimum():
    """Amplitude 100x off and a decay rate 5x off: the same minimum as
    scipy's trust-region least squares."""
    dev, jac, truth = _decay_problem()
    x0 = np.array([500.0, 3.5, 0.0])
    lo, hi = np.array([0.0, 0.0, -10.0]), np.array([1000.0, 10.0, 10.0])
    r = _lm()(_normal(dev, jac), x0, lower=lo, upper=hi)
    ref = scipy_opt.least_squares(dev, x0, jac=jac, bounds=(lo, hi), xtol=1e-15, ftol=1e-15, gtol=1e-15)
    assert r["status"] in (1, 2)
    assert np.allclose(r["params"], ref.x, rtol=1e-6, atol=1e-9), (r, ref.x)
    assert abs(r["statistic"] - 2 * ref.cost) <= 1e-9 * r["statistic"]


def test_minimum_outside_the_limits_ends_on_the_limit():
    """The unconstrained minimum has rate 0.7; with rate <= 0.5 the fit ends
    exactly on that limit (pegged), the other parameters at their
    constrained optimum."""
    dev, jac, _ = _decay_problem()
    x0 = np.array([2.0, 0.2, 1.0])
    lo, hi = np.array([0.0, 0.0, -10.0]), np.array([100.0, 0.5, 10.0])
    r = _lm()(_normal(dev, jac), x0, lower=lo, upper=hi)
    assert r["params"][1] == 0.5
    ref = scipy_opt.least_squares(dev, x0, jac=jac, bounds=(lo, hi), xtol=1e-15, ftol=1e-15, gtol=1e-15)
    assert np.allclose(r["params"], ref.x, rtol=1e-6, atol=1e-9), (r, ref.x)


def test_rosenbrock_and_fixed_parameters():
    """Rosenbrock's valley as least squares (dev = [10 (y - x^2), 1 - x])
    from (-1.2, 1); with x held fixed at 0.5 only y moves, to 0.25."""
    def dev(p):
        return np.array([10.0 * (p[1] - p[0] ** 2), 1.0 - p[0]])

    def jac(p):
        return np.array([[-20.0 * p[0], 10.0], [-1.0, 0.0]])

    r = _lm()(_normal(dev, jac), [-1.2, 1.0])
    assert r["status"] > 0 and np.allclose(r["params"], [1.0, 1.0], atol=1e-6), r
    r = _lm()(_normal(dev, jac), [0.5, 3.0], fixed=[1, 0])
    assert r["params"][0] == 0.5 and abs(r["params"][1] - 0.25) < 1e-8


def test_parameter_without_effect_stays_put():
    """A parameter the deviates do not depend on (a zero Jacobian column,
    like X0 of a lone FlatSky) keeps its value; the others are fitted."""
    dev0, jac0, _ = _decay_problem()

    def dev(x):
        return dev0(x[:3])

    def jac(x):
        return np.concatenate([jac0(x[:3]), np.zeros((200, 1))], axis=1)

    r = _lm()(_normal(dev, jac), [4.0, 0.6, 0.4, 7.25])
    assert r["params"][3] == 7.25 and r["status"] in (1, 2)
    ref = scipy_opt.least_squares(dev0, [4.0, 0.6, 0.4], jac=jac0, xtol=1e-15, ftol=1e-15, gtol=1e-15)
    assert np.allclose(r["params"][:3], ref.x, rtol=1e-6)


def test_batch_matches_one_at_a_time():
    """imfit_MinimizeNormalEquationsBatch over 256 decay problems (enough to
    run the host steps on the worker pool; per-problem limits on half of
    them, the offset held fixed in all) gives each problem exactly the
    result of its own imfit_MinimizeNormalEquations fit: the problems are
    stepped independently, only their evaluations are batched."""
    from imfit_gb300 import minimize_normal_equations_batch
    B = 256
    probs = [_decay_problem(seed=100 + i) for i in range(B)]
    funs = [_normal(dev, jac) for dev, jac, _ in probs]
    rng = np.random.default_rng(7)
    X0 = np.column_stack([rng.uniform(1.0, 20.0, B), rng.uniform(0.1, 3.0, B), np.full(B, 0.5)])
    lo = np.tile([0.0, 0.0, -10.0], (B, 1))
    hi = np.tile([100.0, 10.0, 10.0], (B, 1))
    hi[::2, 1] = 0.6  # the rate limit binds for some of these
    fixed = [0, 0, 1]

    def batch_fun(X, active):
        S, A, b = np.zeros(B), np.zeros((B, 3, 3)), np.zeros((B, 3))
        for i in np.flatnonzero(active):
            S[i], A[i], b[i] = funs[i](X[i])
        return S, A, b

    rb = minimize_normal_equations_batch(batch_fun, X0, fixed=fixed, lower=lo, upper=hi)
    for i in range(B):
        r = _lm()(funs[i], X0[i], fixed=fixed, lower=lo[i], upper=hi[i])
        assert np.array_equal(rb["params"][i], r["params"]), (i, rb["params"][i], r["params"])
        assert rb["statistic"][i] == r["statistic"] and rb["status"][i] == r["status"]
        assert rb["niter"][i] == r["niter"]
    assert np.all(rb["params"][:, 2] == 0.5)
    assert np.any(rb["params"][::2, 1] == 0.6)
