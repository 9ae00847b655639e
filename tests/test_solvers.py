"""CPU tests of the generation-synchronous differential-evolution driver
(solvers/DESolver.cpp semantics) on a batched numpy objective, and of the
makeimage flux table (core/makeimage_main.cpp:753-785)."""
import numpy as np
import pytest

from imfit_gb300 import solvers


class Quadratic:
    """A batched chi^2-like objective: sum ((x - c) / s)^2 + floor."""

    def __init__(self, c, s, floor=100.0):
        self.c, self.s, self.floor = np.asarray(c, float), np.asarray(s, float), floor
        self.calls = []

    def batch_statistic_and_gradient(self, P, want_grad=True):
        assert not want_grad
        P = np.atleast_2d(P)
        self.calls.append(P.copy())
        return np.sum(((P - self.c) / self.s) ** 2, axis=1) + self.floor

    def get_fit_statistic(self, x):
        return float(self.batch_statistic_and_gradient(x, want_grad=False)[0])


def test_de_finds_the_minimum_one_batch_per_generation():
    c = [3.0, -1.0, 0.5, 20.0]
    q = Quadratic(c, [1.0, 0.1, 2.0, 5.0])
    r = solvers.differential_evolution(q, [0, 0, 0, 10], [-10, -5, -5, 0], [10, 5, 5, 50], ftol=1e-10, seed=3)
    assert r["converged"]
    assert np.allclose(r["params"], c, atol=1e-3 * np.array([1.0, 0.1, 2.0, 5.0]))
    assert r["statistic"] - 100.0 < 1e-5
    # the initial population and then one batched call per generation, NP = 8 x free parameters
    # (the last recorded call is get_fit_statistic at the best vector)
    assert r["batched_calls"] == len(q.calls) - 1 == r["generations"] + 2
    assert all(P.shape == (32, 4) for P in q.calls[:-1])
    # every evaluated vector respects the limits
    allp = np.concatenate(q.calls)
    assert np.all(allp >= [-10, -5, -5, 0]) and np.all(allp <= [10, 5, 5, 50])


def test_de_convergence_checked_every_ten_generations_from_forty():
    q = Quadratic([0.0, 0.0], [1.0, 1.0], floor=1.0)
    r = solvers.differential_evolution(q, [0.5, 0.5], [-1, -1], [1, 1], ftol=1e-3, seed=0)
    assert r["converged"] and r["generations"] >= 40 and r["generations"] % 10 == 0


def test_de_fixed_parameters_and_limits():
    q = Quadratic([1.0, 2.0, 3.0], [1.0, 1.0, 1.0])
    r = solvers.differential_evolution(q, [1.0, 7.0, 0.0], [0, 0, 0], [5, 0, 5], fixed=[False, True, False],
                                       seed=1, ftol=1e-9)
    assert r["population"] == 16
    assert all(np.all(P[:, 1] == 7.0) for P in q.calls[:-1])
    assert np.allclose(r["params"][[0, 2]], [1.0, 3.0], atol=1e-3)
    with pytest.raises(ValueError):
        solvers.differential_evolution(q, [1, 2, 3], [0, 0, np.nan], [5, 5, 5])


def test_de_latin_hypercube_initial_population_is_stratified():
    q = Quadratic([0.0, 0.0, 0.0], [1.0, 1.0, 1.0])
    solvers.differential_evolution(q, [0, 0, 0], [0, 0, 0], [24, 24, 24], max_generations=0, latin_hypercube=True)
    P0 = q.calls[0]
    assert P0.shape == (24, 3)
    for j in range(3):  # one member in each of the 24 strata of every parameter
        assert sorted(np.floor(P0[:, j]).astype(int)) == list(range(24))


def test_flux_table_matches_makeimage_output():
    """Lines of tests/makeimage_reference/makeimage_textout5b (printed fluxes
    of config_makeimage_sersic+exp512b.dat on a 5000 x 5000 image)."""
    from imfit_gb300.cli import flux_table
    S, E = 2.263505e6, 3.534285e5  # within the printed rounding of the reference's values
    lines = flux_table(["Sersic", "Exponential", "FlatSky"], [S, E, 0.0], S + E, labels=["bulge", "disk", ""])
    assert lines[0] == "Component                 Flux        Magnitude   Fraction   Label"
    assert lines[1] == "Sersic                    2.2635e+06      ---     0.86495    bulge"
    assert lines[2] == "Exponential               3.5343e+05      ---     0.13505    disk"
    assert lines[3] == "FlatSky                   0.0000e+00      ---     0.00000"
    assert lines[4] == ""
    assert lines[5] == "Total                     2.6169e+06      ---     1.00000"
    zp = flux_table(["Gaussian"], [1.0e4], 1.0e4, zero_point=26.0)
    assert zp[1] == "Gaussian                  1.0000e+04   16.0000     1.00000"


def test_bootstrap_statistics_follow_the_reference_formulas():
    """core/statistics.cpp:54-100: n - 1 standard deviation; interval indices
    round(0.1585 n) - 1 and round(0.8415 n) of the sorted values."""
    v = np.arange(10.0)[::-1]
    assert solvers.confidence_interval(v) == (1.0, 8.0)  # indices 1 and 8
    assert solvers.confidence_interval([3.0, 1.0]) == (1.0, 3.0)  # clamped for n < 4
    assert abs(solvers.standard_deviation([1.0, 2.0, 3.0, 4.0]) - np.std([1, 2, 3, 4], ddof=1)) < 1e-15
    lines = solvers.bootstrap_summary([1.0, 5.0], np.array([[0.9, 5.0], [1.1, 5.0], [1.0, 5.0]]), ["a", "b"],
                                      fixed=[False, True])
    assert lines[1].endswith("(3 successful iterations):")
    assert lines[3] == "a = 1  +0.1, -0.1    [0.9 -- 1.1, 0.1];  (1 +/- 0.1)"
    assert lines[4] == "b = 5     [fixed parameter]"


def test_bootstrap_file_layout():
    """GetParamHeader / PrintModelParamsHorizontalString (core/model_object.cpp:1941-2033)."""
    from imfit_gb300.config import _NPARAMS
    names = ["X0", "Y0", "PA", "ell", "n", "I_e", "r_e", "I_sky"]
    lines = solvers.bootstrap_file_lines([("Sersic", True), ("FlatSky", False)], names, _NPARAMS,
                                         np.arange(8.0)[None, :] + 0.5, 5)
    assert lines[:2] == ["#", "# Bootstrap resampling output (5 iterations requested):"]
    assert lines[2] == "# X0_1\t\tY0_1\t\tPA_1\tell_1\tn_1\tI_e_1\tr_e_1\tI_sky_2\t"
    assert lines[3].split("\t")[:2] == ["0.5000000000", "1.500000000"]


def test_dream_samples_a_gaussian_posterior():
    """DREAM (cdream/dream.cpp) on log L = -chi^2/2 of independent Gaussians:
    post-burn-in chains reproduce the means and widths; Gelman-Rubin passes."""
    q = Quadratic([1.0, -2.0, 5.0, 0.3], [0.1, 0.5, 2.0, 0.05], floor=0.0)
    r = solvers.dream(q, [0, 0, 0, 0], [-5, -10, -20, -1], [5, 10, 30, 1], burn_in=1000, gelman_evals=2000,
                      max_generations=30000, seed=1)
    assert r["converged"] and r["n_chains"] == 4
    post = r["chains"][r["burn_in"] == 0].reshape(-1, 4)
    assert np.all(np.abs(post.mean(axis=0) - q.c) < 0.15 * q.s)
    assert np.all(np.abs(post.std(axis=0) / q.s - 1.0) < 0.15)
    assert np.all(r["scale_reduction"] < 1.01)


def test_gelman_rubin_and_quantiles():
    """cdream/gelman_rubin.cpp (adjustDF = 0) and GSL's sorted-data quantile."""
    rng = np.random.default_rng(0)
    S = rng.normal(size=(400, 5, 2))
    S[:, :, 1] += np.arange(5)[None, :]  # chains with different means: large R-hat
    r = solvers.gelman_rubin(S)
    n, m = 400, 5
    W = S[:, :, 0].var(axis=0, ddof=1).mean()
    B = S[:, :, 0].mean(axis=0).var(ddof=1)
    assert abs(r[0] - np.sqrt(((n - 1) / n * W + B + B / m) / W)) < 1e-12
    assert r[0] < 1.02 and r[1] > 2.0
    assert solvers._gsl_quantile_sorted([1.0, 2.0, 4.0], 0.25) == 1.5
    assert solvers._gsl_quantile_sorted([1.0, 2.0, 4.0], 0.75) == 3.0


def test_chain_file_layout():
    from imfit_gb300.config import _NPARAMS
    head = solvers.chain_file_header([("Gaussian", True)], ["X0", "Y0", "PA", "ell", "I_0", "sigma"], _NPARAMS)
    assert head == ("# X0_1\t\tY0_1\t\tPA_1\tell_1\tI_0_1\tsigma_1\t  likelihood  burn-in    CR1               "
                    "CR2               CR3        accept")
    row = solvers.chain_file_row([4.114481249, 4.845422845, 142.3764518, 0.1425389645, 232.4511719, 1.04774257],
                                 -2616.014985785, 1, [1 / 3, 1 / 3, 1 / 3], 1)
    # the first row of tests/imfit-mcmc_reference/mcmc_ref1.1.txt_skip3
    assert row == ("4.114481249\t4.845422845\t142.3764518\t0.1425389645\t232.4511719\t1.047742570 "
                   "-2.616014985785e+03 1  3.333333333333e-01 3.333333333333e-01 3.333333333333e-01 1")
