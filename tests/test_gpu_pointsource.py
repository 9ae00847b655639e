"""GPU tests of the PointSource / PointSourceRot functions (post-convolution,
interpolated PSF): the plain FP64 path against the oracle and the reference's
oversampled_pointsource.fits."""
import os

import numpy as np
import pytest

from helpers import normwise

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _moffat_psf(n=25, fwhm=3.5, beta=3.0, dx=0.0):
    yy, xx = np.mgrid[0:n, 0:n] - (n - 1) / 2.0
    a = fwhm / (2.0 * np.sqrt(2.0 ** (1.0 / beta) - 1.0))
    p = (1.0 + ((xx - dx) ** 2 + (0.8 * yy) ** 2) / a ** 2) ** (-beta)  # slightly asymmetric
    return p / p.sum()


FUNCS = [("Sersic", True), ("PointSource", False), ("PointSourceRot", True)]
PARAMS = [40.3, 31.7, 25.0, 0.3, 1.8, 20.0, 8.0, 900.0, 22.6, 44.2, 35.0, 400.0]


def _model(cls, method, region=None, psf=None, nc=70, nr=60):
    m = cls()
    for k, (name, new_set) in enumerate(FUNCS):
        m.add_function(name, new_set)
    m.finish_functions()
    if cls.__name__ == "OracleModel":
        m.set_point_source_method(1, method)
    m.add_psf(_moffat_psf() if psf is None else psf)
    m.setup_model_image(nc, nr)
    if region is not None:
        m.add_oversampled_psf(_moffat_psf(75, fwhm=10.5, dx=0.3), 3, region)
    return m


def _gpu_model(gpu, method, region=None):
    m = gpu.ModelObject()
    for k, (name, new_set) in enumerate(FUNCS):
        m.add_function(name, new_set, optional={"method": method} if k == 1 else None)
    m.finish_functions()
    m.add_psf(_moffat_psf())
    m.setup_model_image(70, 60)
    if region is not None:
        m.add_oversampled_psf(_moffat_psf(75, fwhm=10.5, dx=0.3), 3, region)
    return m


@pytest.mark.parametrize("method", ["bicubic", "lanczos2", "lanczos3"])
def test_point_sources_against_oracle(gpu, oracle_mod, method):
    """Sersic + PointSource + PointSourceRot (second function set) on the
    plain path: the point sources use the first one's interpolator kind."""
    g = _gpu_model(gpu, method)
    o = _model(oracle_mod.OracleModel, method)
    g.create_model_image(PARAMS)
    o.create_model_image(PARAMS)
    assert normwise(g.get_model_image(), o.get_model_image()) < 1e-12
    for fi in range(3):
        assert normwise(g.get_single_function_image(PARAMS, fi), o.get_single_function_image(PARAMS, fi)) < 1e-12


def test_point_sources_with_region_and_persistent_scale(gpu, oracle_mod):
    """An oversampled region over part of a point source: inside, the region's
    bicubic interpolator of the oversampled PSF as given; outside, the main
    PSF.  After the first evaluation the point sources keep the region's
    scale on the main grid too (PointSource::oversamplingScale is never
    reset), so the second evaluation differs from the first -- as in the
    reference."""
    region = (18, 30, 24, 36)
    g = _gpu_model(gpu, "bicubic", region)
    o = _model(oracle_mod.OracleModel, "bicubic", region)
    first = []
    for call in range(3):
        g.create_model_image(PARAMS)
        o.create_model_image(PARAMS)
        gi, oi = g.get_model_image(), o.get_model_image()
        assert normwise(gi, oi) < 1e-11, call
        first.append(gi)
    assert normwise(first[0], first[1]) > 1e-6 and normwise(first[1], first[2]) == 0.0
    for fi in (1, 2):
        assert normwise(g.get_single_function_image(PARAMS, fi), o.get_single_function_image(PARAMS, fi)) < 1e-11


def test_point_source_oversampled_golden(gpu):
    """do_makeimage_tests:74 -> tests/oversampled_pointsource.fits, within one
    float32 ulp."""
    d = np.load(os.path.join(GOLDEN, "pointsource.npz"))
    gm = np.load(os.path.join(GOLDEN, "makeimage.npz"))
    m = gpu.ModelObject()
    m.add_function("PointSource", True)
    m.finish_functions()
    m.add_psf(gm["psf_standard"].astype(np.float64))
    m.setup_model_image(200, 200)
    m.add_oversampled_psf(gm["psf_oversamp"].astype(np.float64), int(d["ps_scale"]), tuple(d["ps_region"]))
    m.create_model_image(d["ps_params"])
    img = m.get_model_image()
    want = d["ps_image"]
    assert np.all(np.abs(img - want) <= np.spacing(np.abs(want)).astype(np.float64) + 1e-12)


def test_point_source_statistic_and_fluxes(gpu, oracle_mod):
    """chi^2 with data-based errors (plain path) and FindTotalFluxes (I_tot)."""
    rng = np.random.default_rng(3)
    o = _model(oracle_mod.OracleModel, "lanczos2")
    o.create_model_image(PARAMS)
    data = rng.poisson(np.clip(o.get_model_image() + 50.0, 0, None)).astype(np.float64)
    stats = []
    for cls in ("gpu", "oracle"):
        if cls == "gpu":
            m = gpu.ModelObject()
            for k, (name, new_set) in enumerate(FUNCS):
                m.add_function(name, new_set, optional={"method": "lanczos2"} if k == 1 else None)
            m.finish_functions()
            m.add_psf(_moffat_psf())
        else:
            m = oracle_mod.OracleModel()
            for name, new_set in FUNCS:
                m.add_function(name, new_set)
            m.finish_functions()
            m.set_point_source_method(1, "lanczos2")
            m.add_psf(_moffat_psf())
        m.add_image_data(data)
        m.add_image_characteristics(1.0, 2.0, 1.0, 1, 50.0)
        assert m.final_setup() == 0
        stats.append(m.get_fit_statistic(PARAMS))
    assert abs(stats[0] - stats[1]) <= 1e-10 * stats[1]
    g = _gpu_model(gpu, "bicubic")
    tot, ind = g.find_total_fluxes(PARAMS, 500, 500)
    assert ind[1] == 900.0 and ind[2] == 400.0


def test_optional_parameter_errors(gpu):
    m = gpu.ModelObject()
    m.add_function("Sersic", True)
    with pytest.raises(gpu.ImfitError):
        m.add_function("Exponential", optional={"method": "bicubic"})
    m = gpu.ModelObject()
    with pytest.raises(gpu.ImfitError):
        m.add_function("PointSourceRot", True, optional={"method": "lanczos3"})
    m = gpu.ModelObject()
    with pytest.raises(gpu.ImfitError):
        m.add_function("PointSource", True, optional={"method": "spline"})


FFUNCS = [("Sersic", True), ("PointSource", False), ("PointSourceRot", True), ("FlatSky", False)]
FTRUTH = np.array([40.3, 31.7, 25.0, 0.3, 1.8, 20.0, 8.0, 3000.0, 22.6, 44.2, 35.0, 1500.0, 50.0])


def _fitted_pair(gpu, oracle_mod, method="bicubic", region=None, seed=5):
    """(GPU handle, oracle handle) with data made from the oracle at FTRUTH."""
    o = oracle_mod.OracleModel()
    for name, new_set in FFUNCS:
        o.add_function(name, new_set)
    o.finish_functions()
    o.set_point_source_method(1, method)
    o.add_psf(_moffat_psf())
    o.setup_model_image(80, 70)
    if region is not None:
        o.add_oversampled_psf(_moffat_psf(75, fwhm=10.5, dx=0.3), 3, region)
    o.create_model_image(FTRUTH)
    rng = np.random.default_rng(seed)
    data = rng.poisson(np.clip(o.get_model_image(), 0, None)).astype(np.float64)
    hs = []
    for kind in ("gpu", "oracle"):
        m = gpu.ModelObject() if kind == "gpu" else oracle_mod.OracleModel()
        for k, (name, new_set) in enumerate(FFUNCS):
            if kind == "gpu":
                m.add_function(name, new_set, optional={"method": method} if k == 1 else None)
            else:
                m.add_function(name, new_set)
        m.finish_functions()
        if kind == "oracle":
            m.set_point_source_method(1, method)
        m.add_psf(_moffat_psf())
        m.add_image_data(data)
        if region is not None:
            m.add_oversampled_psf(_moffat_psf(75, fwhm=10.5, dx=0.3), 3, region)
        m.add_image_characteristics(1.0, 3.0, 1.0, 1, 0.0)
        assert m.final_setup() == 0
        hs.append(m)
    return hs


@pytest.mark.parametrize("method,region", [("bicubic", None), ("lanczos2", None), ("lanczos3", None),
                                           ("bicubic", (18, 30, 24, 36))])
def test_fast_path_point_sources(gpu, oracle_mod, method, region):
    """Fast statistic + adjoint gradient with point sources (main grid and an
    oversampled region over parts of them) against the FP64 statistic and
    its finite-difference gradient; J^T J's gradient 2 J^T dev agrees."""
    g, o = _fitted_pair(gpu, oracle_mod, method, region)
    p = FTRUTH * np.array([1.0, 1.0, 1.02, 1.05, 0.97, 1.03, 0.95, 0.9, 1.0, 1.0, 1.04, 1.1, 1.0])
    p[0] += 0.3
    p[8] -= 0.2
    s64 = g.get_fit_statistic(p)
    assert abs(s64 - o.get_fit_statistic(p)) <= 1e-10 * s64
    if region is not None:  # compare evaluations after the first (the point sources' scale has settled)
        s64 = g.get_fit_statistic(p)
        assert abs(s64 - o.get_fit_statistic(p)) <= 1e-10 * s64
    s, grad = g.statistic_and_gradient(p)
    _, gfd = g.statistic_and_gradient_fd(p)
    assert abs(s - s64) <= 1e-5 * s64, (s, s64)
    top = np.max(np.abs(gfd))
    assert np.all(np.abs(grad - gfd) <= 3e-3 * np.abs(gfd) + 3e-4 * top), (grad, gfd)
    sj, A, b = g.jtwj(p)
    assert abs(sj - s64) <= 1e-5 * s64
    assert np.all(np.abs(2 * b - gfd) <= 3e-3 * np.abs(gfd) + 3e-4 * top), (2 * b, gfd)


def test_fast_path_point_source_state_follows_the_reference(gpu, oracle_mod):
    """With an oversampled region the first evaluation sees scale 1 on the
    main grid and later ones the region's scale, on the fast path as on the
    plain one (and in the oracle)."""
    region = (18, 30, 24, 36)
    g, o = _fitted_pair(gpu, oracle_mod, "bicubic", region)
    p = FTRUTH.copy()
    s_first_fast = g.statistic_and_gradient(p)[0]
    s_first_oracle = o.get_fit_statistic(p)
    s_second_fast = g.statistic_and_gradient(p)[0]
    s_second_oracle = o.get_fit_statistic(p)
    assert abs(s_first_fast - s_first_oracle) <= 1e-5 * s_first_oracle
    assert abs(s_second_fast - s_second_oracle) <= 1e-5 * s_second_oracle
    assert abs(s_first_oracle - s_second_oracle) > 1e-4 * s_first_oracle


def test_lm_fit_with_point_sources(gpu, oracle_mod):
    """LM on the GPU's J^T J fits a Sersic + nuclear point source + offset
    rotated point source + sky image (Poisson noise): it ends below the
    truth's chi^2 and at a minimum of the FP64 statistic -- the Newton
    decrease g^T A^-1 g / 4 left from the FP64 finite-difference gradient is
    negligible.  (The nuclear source trades flux with the Sersic core, so the
    parameters themselves are not compared with the truth.)"""
    g, o = _fitted_pair(gpu, oracle_mod, "bicubic", None, seed=8)
    start = FTRUTH * np.array([1.0, 1.0, 1.05, 1.1, 0.9, 1.1, 0.9, 0.8, 1.0, 1.0, 1.1, 1.2, 1.05])
    start[[0, 1, 8, 9]] += [0.4, -0.3, 0.3, 0.2]
    r = g.fit_lm(start)
    assert r["status"] > 0
    s_fit = g.get_fit_statistic(r["params"])
    assert s_fit <= g.get_fit_statistic(FTRUTH)
    _, gfd = g.statistic_and_gradient_fd(r["params"])
    _, A, _ = g.jtwj(r["params"])
    decrease = 0.25 * gfd @ np.linalg.solve(A, gfd)
    assert decrease < 1e-2 * max(1.0, 1e-6 * s_fit), decrease
    assert abs(r["params"][8] - FTRUTH[8]) < 0.3 and abs(r["params"][9] - FTRUTH[9]) < 0.3
