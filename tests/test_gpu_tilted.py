"""GPU tests of the TiltedSkyPlane function (func_tilted-sky-plane.cpp): the
plane I_0 + m_x (x - X0) + m_y (y - Y0) about its function set's centre,
convolved with the PSF like every other non-point-source component, with no
subsampling and zero flux (IsBackground, core/model_object.cpp:2449-2450)."""
import numpy as np
import pytest

from helpers import normwise, relerr

pytestmark = pytest.mark.gpu

FUNCS = [("Sersic", True), ("TiltedSkyPlane", True)]
# X0 Y0 | Sersic PA ell n I_e r_e | X0 Y0 | TiltedSkyPlane I_0 m_x m_y
TRUTH = np.array([38.3, 33.6, 25.0, 0.3, 1.8, 30.0, 7.0, 40.0, 35.0, 20.0, 0.05, -0.03])


def _psf(n=25, fwhm=3.5, beta=3.0):
    yy, xx = np.mgrid[0:n, 0:n] - (n - 1) / 2.0
    a = fwhm / (2.0 * np.sqrt(2.0 ** (1.0 / beta) - 1.0))
    p = (1.0 + ((xx - 0.4) ** 2 + (0.8 * yy) ** 2) / a ** 2) ** (-beta)  # off-centre: the plane shifts
    return p / p.sum()


def _build(m, data=None, psf=True, region=None, nc=80, nr=70):
    for name, new_set in FUNCS:
        m.add_function(name, new_set)
    m.finish_functions()
    if psf:
        m.add_psf(_psf())
    if data is None:
        m.setup_model_image(nc, nr)
    else:
        m.add_image_data(data)
    if region is not None:
        m.add_oversampled_psf(_psf(45, fwhm=10.5), 3, region)
    if data is not None:
        m.add_image_characteristics(1.0, 3.0, 1.0, 1, 0.0)
        assert m.final_setup() == 0
    return m


def test_plane_alone_is_the_reference_expression(gpu):
    """No PSF: the model is I_0 + m_x (x - X0) + m_y (y - Y0) at the IRAF
    pixel centres, in the reference's evaluation order."""
    m = gpu.ModelObject()
    m.add_function("TiltedSkyPlane", True)
    m.finish_functions()
    m.setup_model_image(37, 23)
    p = [12.25, 9.5, 7.0, 0.11, -0.07]
    m.create_model_image(p)
    y, x = np.mgrid[1:24, 1:38].astype(float)
    want = 7.0 + 0.11 * (x - 12.25) + -0.07 * (y - 9.5)
    assert np.max(np.abs(m.get_model_image() - want)) <= 1e-14 * np.max(np.abs(want))
    assert m.parameter_names() == ["X0", "Y0", "I_0", "m_x", "m_y"]


@pytest.mark.parametrize("region", [None, (20, 32, 25, 38)])
def test_plane_against_oracle(gpu, oracle_mod, region):
    """Sersic + TiltedSkyPlane (own function set), PSF with an off-centre
    peak, optionally an oversampled region: plain path against the oracle,
    per function and in total; the plane's flux is zero."""
    g = _build(gpu.ModelObject(), region=region)
    o = _build(oracle_mod.OracleModel(), region=region)
    g.create_model_image(TRUTH)
    o.create_model_image(TRUTH)
    assert normwise(g.get_model_image(), o.get_model_image()) < 1e-12
    for fi in range(2):
        assert normwise(g.get_single_function_image(TRUTH, fi), o.get_single_function_image(TRUTH, fi)) < 1e-12
    total, fluxes = g.find_total_fluxes(TRUTH, 80, 70)
    assert fluxes[1] == 0.0 and total == fluxes[0] > 0.0


def _pair(gpu, oracle_mod, region=None, seed=3):
    o = _build(oracle_mod.OracleModel(), region=region)
    o.create_model_image(TRUTH)
    rng = np.random.default_rng(seed)
    data = rng.poisson(np.clip(o.get_model_image(), 0, None)).astype(np.float64)
    return _build(gpu.ModelObject(), data, region=region), _build(oracle_mod.OracleModel(), data, region=region)


@pytest.mark.parametrize("region", [None, (20, 32, 25, 38)])
def test_fast_path_plane(gpu, oracle_mod, region):
    """Fast statistic + adjoint gradient and J^T J's 2 J^T dev against the
    FP64 statistic and its finite-difference gradient."""
    g, o = _pair(gpu, oracle_mod, region)
    p = TRUTH * np.array([1.0, 1.0, 1.02, 1.05, 0.97, 1.03, 0.95, 1.0, 1.0, 1.04, 1.3, 0.8])
    p[[0, 7, 8]] += [0.3, -0.5, 0.4]
    s64 = g.get_fit_statistic(p)
    assert relerr(s64, o.get_fit_statistic(p)) < 1e-10
    s, grad = g.statistic_and_gradient(p)
    _, gfd = g.statistic_and_gradient_fd(p)
    assert relerr(s, s64) < 1e-5, (s, s64)
    top = np.max(np.abs(gfd))
    assert np.all(np.abs(grad - gfd) <= 3e-3 * np.abs(gfd) + 3e-4 * top), (grad, gfd)
    sj, A, b = g.jtwj(p)
    assert relerr(sj, s64) < 1e-5
    assert np.all(np.abs(2 * b - gfd) <= 3e-3 * np.abs(gfd) + 3e-4 * top), (2 * b, gfd)


def test_lm_fit_recovers_the_slopes(gpu, oracle_mod):
    """LM on the GPU's J^T J, the plane's centre held fixed (it is degenerate
    with I_0): the fit ends at a minimum of the FP64 statistic (negligible
    Newton decrease from the FP64 finite-difference gradient) and the slopes
    come back within about four sigma (sigma(m) ~ 0.003 here) of the truth."""
    g, _ = _pair(gpu, oracle_mod, seed=11)
    start = TRUTH * np.array([1.0, 1.0, 1.05, 1.1, 0.9, 1.1, 0.9, 1.0, 1.0, 1.2, 0.5, 1.6])
    start[[0, 1]] += [0.4, -0.3]
    fixed = np.zeros(len(TRUTH), dtype=bool)
    fixed[[7, 8]] = True
    r = g.fit_lm(start, fixed=fixed)
    assert r["status"] > 0
    assert g.get_fit_statistic(r["params"]) <= g.get_fit_statistic(TRUTH)
    free = ~fixed
    _, gfd = g.statistic_and_gradient_fd(r["params"])
    _, A, _ = g.jtwj(r["params"])
    gf = gfd[free]
    decrease = 0.25 * gf @ np.linalg.solve(A[np.ix_(free, free)], gf)
    assert decrease < 1e-2, decrease
    assert abs(r["params"][10] - TRUTH[10]) < 0.012 and abs(r["params"][11] - TRUTH[11]) < 0.012
