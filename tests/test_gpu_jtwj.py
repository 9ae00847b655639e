"""GPU checks of the forward-mode J^T J / J^T dev (the analytic replacement of
mpfit's finite-difference Jacobian, solvers/mpfit.cpp:1102-1356) and of the
normal-equation Levenberg-Marquardt driver built on it.

Tolerances:
  * statistic sum dev^2: relative 1e-5 against the FP64 oracle;
  * J^T dev and J^T J against the oracle's central finite-difference Jacobian
    of the deviates (subsampling off, so the model is smooth):
    |b - b_fd| <= 2e-3 (|b_fd| + 1e-3 max|b_fd|) and
    |A_jk - A_fd,jk| <= 2e-3 sqrt(A_fd,jj A_fd,kk);
  * 2 J^T dev equals the adjoint gradient of the chi^2 statistic within 1e-4
    (both analytic FP32 forms; they differ only in rounding);
  * LM fit of the reference's n3073 regression case
    (tests/imfit_reference/imfit_textout4) recovers mpfit's parameters within
    2e-4 relative and its chi^2 within 1e-6 relative.
"""
import os

import numpy as np
import pytest

from helpers import relerr

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _case(oracle_mod, stat="chi2", region=True, seed=31):
    from imfit_gb300 import workloads
    wl = workloads.small_case(seed=seed, stat=stat, region=region)
    workloads.synthesize(wl, oracle_mod.OracleModel)
    return wl


def _build(cls, wl, subsample=False):
    m = cls()
    for n, s in wl.functions:
        m.add_function(n, s, subsampling=subsample)
    m.finish_functions()
    m.add_psf(wl.psf)
    m.add_image_data(wl.data)
    m.add_image_characteristics(wl.gain, wl.read_noise, 1.0, 1, wl.original_sky)
    for psf, sc, reg in wl.regions:
        m.add_oversampled_psf(psf, sc, reg)
    if wl.mask is not None:
        m.add_mask_vector(wl.mask)
    if wl.stat == "cash":
        m.use_cash()
    elif wl.stat == "pmlr":
        m.use_pmlr()
    assert m.final_setup() == 0
    return m


def _fd_jacobian(o, p, rel=1e-5):
    cols = []
    for j in range(len(p)):
        h = rel * max(abs(p[j]), 1.0)
        a = np.array(p, dtype=float)
        b = a.copy()
        a[j] += h
        b[j] -= h
        cols.append((o.compute_deviates(a) - o.compute_deviates(b)) / (2 * h))
    return np.array(cols)  # nP x nData


def _check_normal_equations(g, o, p, tol=2e-3):
    s, A, b = g.jtwj(p)
    dev = o.compute_deviates(p)
    J = _fd_jacobian(o, p)
    A_fd = J @ J.T
    b_fd = J @ dev
    assert relerr(s, float(dev @ dev)) < 1e-5
    scale = np.abs(b_fd) + 1e-3 * np.max(np.abs(b_fd))
    assert np.all(np.abs(b - b_fd) / scale < tol), list(zip(g.parameter_names(), b, b_fd))
    d = np.sqrt(np.outer(np.diag(A_fd), np.diag(A_fd)))
    assert np.all(np.abs(A - A_fd) <= tol * d + 1e-30), np.max(np.abs(A - A_fd) / d)
    assert np.array_equal(A, A.T)
    return s, A, b


@pytest.mark.parametrize("region", [False, True])
def test_jtwj_chi2_vs_fd_jacobian(gpu, oracle_mod, region):
    wl = _case(oracle_mod, region=region)
    g = _build(gpu.ModelObject, wl)
    o = _build(oracle_mod.OracleModel, wl)
    for p in (wl.start, wl.truth):
        _check_normal_equations(g, o, p)


def test_jtwj_pmlr_vs_fd_jacobian(gpu, oracle_mod):
    wl = _case(oracle_mod, stat="pmlr", region=False, seed=37)
    g = _build(gpu.ModelObject, wl)
    o = _build(oracle_mod.OracleModel, wl)
    _check_normal_equations(g, o, wl.start)


def test_jtwj_matches_adjoint_gradient(gpu, oracle_mod):
    wl = _case(oracle_mod, region=True, seed=41)
    g = _build(gpu.ModelObject, wl, subsample=True)
    s, A, b = g.jtwj(wl.start)
    s2, grad = g.statistic_and_gradient(wl.start)
    assert relerr(s, s2) < 1e-6
    scale = np.abs(grad) + 1e-3 * np.max(np.abs(grad))
    assert np.all(np.abs(2 * b - grad) / scale < 1e-4), list(zip(2 * b, grad))


def test_jtwj_rejects_cash(gpu, oracle_mod):
    wl = _case(oracle_mod, stat="cash", region=False)
    g = _build(gpu.ModelObject, wl)
    with pytest.raises(gpu.ImfitError) as e:
        g.jtwj(wl.start)
    assert e.value.code == -4


def _n3073(gpu):
    d = np.load(os.path.join(GOLDEN, "n3073.npz"))
    m = gpu.ModelObject()
    m.add_function("Sersic", True)
    m.add_function("Exponential")
    m.finish_functions()
    m.add_psf(d["psf"].astype(np.float64))
    m.add_image_data(d["data"].astype(np.float64))
    m.add_image_characteristics(float(d["gain"]), float(d["read_noise"]), 1.0, 1, float(d["original_sky"]))
    m.add_mask_vector(d["mask"].astype(np.float64))
    assert m.final_setup() == 0
    return m, d


def test_lm_fit_reproduces_mpfit_on_n3073(gpu):
    m, d = _n3073(gpu)
    r = m.fit_lm(d["params"], lower=d["lo"], upper=d["hi"], ftol=1e-8)
    assert r["status"] in (1, 3, 4), r
    want = d["lm_params"]
    err = np.abs(r["params"] - want) / np.abs(want)
    assert np.all(err < 2e-4), list(zip(m.parameter_names(), r["params"], want, err))
    chi2 = m.get_fit_statistic(r["params"])  # FP64 plain path at the fitted point
    assert chi2 <= float(d["lm_chi2"]) * (1 + 1e-6), (chi2, float(d["lm_chi2"]))
    assert relerr(chi2, float(d["lm_chi2_printed"])) < 1e-6


def test_lm_fit_respects_fixed_and_limits(gpu):
    m, d = _n3073(gpu)
    p0 = np.array(d["params"], dtype=float)
    fixed = np.zeros(len(p0), dtype=int)
    fixed[4] = 1                      # Sersic n held
    hi = np.array(d["hi"], dtype=float)
    hi[6] = 24.0                      # Sersic r_e limited below its free optimum (~26.8)
    r = m.fit_lm(p0, fixed=fixed, lower=d["lo"], upper=hi)
    assert r["params"][4] == p0[4]
    assert r["params"][6] <= 24.0
    assert np.all(r["params"] >= d["lo"]) and np.all(r["params"] <= hi)
    assert m.get_fit_statistic(r["params"]) < m.get_fit_statistic(p0)


@pytest.mark.parametrize("region", [False, True])
def test_jacobian_columns_vs_fd(gpu, oracle_mod, region):
    """imfit_GetJacobian (mpfit side = 3 derivative vectors) against the
    oracle's central-difference Jacobian of the deviates, column by column:
    |J - J_fd| <= 2e-3 max|J_fd column| + 1e-6 max|J_fd|; deviates within
    1e-5 of the oracle's (relative to their largest value)."""
    wl = _case(oracle_mod, region=region, seed=53)
    g = _build(gpu.ModelObject, wl)
    o = _build(oracle_mod.OracleModel, wl)
    J, dev = g.jacobian(wl.start)
    J_fd = _fd_jacobian(o, wl.start)
    dev_o = o.compute_deviates(wl.start)
    assert np.max(np.abs(dev - dev_o)) <= 1e-5 * np.max(np.abs(dev_o))
    top = np.max(np.abs(J_fd))
    for j in range(J.shape[0]):
        colmax = np.max(np.abs(J_fd[j]))
        assert np.max(np.abs(J[j] - J_fd[j])) <= 2e-3 * colmax + 1e-6 * top, (g.parameter_names()[j], j)
    # the normal equations from these columns are the JtWJ entry point's
    s, A, b = g.jtwj(wl.start)
    assert np.allclose(J @ J.T, A, rtol=1e-4, atol=1e-6 * np.max(np.abs(A)))


def test_cli_fit_of_n3073(gpu, tmp_path):
    """The imfit-style command line (config file + FITS images) on the n3073
    inputs reproduces mpfit's fit (imfit_textout4) like imfit_FitLM does."""
    from imfit_gb300 import cli, fits
    d = np.load(os.path.join(GOLDEN, "n3073.npz"))
    names = ["X0", "Y0", "PA", "ell", "n", "I_e", "r_e", "PA", "ell", "I_0", "h"]
    lines = [f"GAIN {float(d['gain'])}", f"READNOISE {float(d['read_noise'])}",
             f"ORIGINAL_SKY {float(d['original_sky'])}", ""]
    for j, (nm, v, lo, hi) in enumerate(zip(names, d["params"], d["lo"], d["hi"])):
        if j == 2:
            lines.append("FUNCTION Sersic")
        if j == 7:
            lines.append("FUNCTION Exponential")
        lines.append(f"{nm} {float(v)!r} {float(lo)!r},{float(hi)!r}")
    cfgp = tmp_path / "config.dat"
    cfgp.write_text("\n".join(lines) + "\n")
    for name in ("data", "mask", "psf"):
        fits.write_image(str(tmp_path / f"{name}.fits"), d[name].astype(np.float64))
    p, s = cli.run([str(cfgp), str(tmp_path / "data.fits"), "--psf", str(tmp_path / "psf.fits"),
                    "--mask", str(tmp_path / "mask.fits"), "--save-params", str(tmp_path / "best.dat"),
                    "--save-model", str(tmp_path / "model.fits")])
    err = np.abs(p - d["lm_params"]) / np.abs(d["lm_params"])
    assert np.all(err < 2e-4), err
    assert relerr(s, float(d["lm_chi2_printed"])) < 1e-6
    assert (tmp_path / "best.dat").exists() and fits.read_image(str(tmp_path / "model.fits"))[0].shape == d["data"].shape
