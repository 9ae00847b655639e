"""CPU tests of the oracle: pinned against the reference's own known answers
(unit_tests/unittest_funcs.t.h), its regression printouts
(tests/imfit_reference/imfit_textout4, 4c, 4d) via committed fixtures, and,
where the reference checkout exists, against the reference's own sources
compiled here (oracle/_ref)."""
import os

import numpy as np
import pytest

import oracle
from helpers import normwise

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _n3073_model(oracle, stat, mask=True):
    d = np.load(os.path.join(GOLDEN, "n3073.npz"))
    m = oracle.OracleModel()
    m.add_function("Sersic", True)
    m.add_function("Exponential")
    m.finish_functions()
    m.add_psf(d["psf"].astype(np.float64))
    m.add_image_data(d["data"].astype(np.float64))
    m.add_image_characteristics(float(d["gain"]), float(d["read_noise"]), 1.0, 1, float(d["original_sky"]))
    if mask:
        m.add_mask_vector(d["mask"].astype(np.float64))
    if stat == "cash":
        m.use_cash()
    assert m.final_setup() == 0
    return m, d


# unit_tests/unittest_funcs.t.h (DELTA = 1e-9), subsampling off as in those tests
KNOWN = [
    ("Exponential", [90, 0, 1, 10], (10, 10), [((10, 10), 1.0), ((11, 10), np.exp(-0.1)), ((10, 11), np.exp(-0.1))]),
    ("Sersic", [90, 0, 2, 1, 10], (10, 10),
     [((10, 10), 39.333062332325284), ((11, 10), 12.315472433581958), ((20, 10), 1.0), ((10, 0), 1.0)]),
    ("Moffat", [90, 0, 1, 10, 3], (10, 10), [((10, 10), 1.0), ((11, 10), 0.96944697430705418),
                                             ((20, 10), 0.11784501202946467)]),
    ("Moffat", [90, 0.5, 1, 10, 1], (10, 10), [((10, 9.5), 0.96153846153846145), ((11, 10), 0.96153846153846145)]),
    ("FerrersBar3D", [0, 0, 0, 1, 100, 1, 1, 2], (100, 100),
     [((100, 100), 106.666666573), ((100, 150), 51.9615240239), ((0, 100), 0.0), ((201, 100), 0.0)]),
    ("FerrersBar3D", [0, 0, 0, 1, 100, 0.5, 1, 2], (100, 100),
     [((100, 100), 106.666666573), ((100, 50), 51.9615240239), ((125, 100), 51.9615240239), ((150, 100), 0.0)]),
]


@pytest.mark.parametrize("name,params,center,cases", KNOWN)
def test_function_known_answers(oracle_mod, name, params, center, cases):
    for (x, y), want in cases:
        got = oracle_mod.function_value(name, params, center[0], center[1], x, y, subsampling=False)
        assert abs(got - want) <= 1e-9, (name, x, y, got, want)


def test_tilted_sky_plane_expression(oracle_mod):
    """TiltedSkyPlane (no known answers in the reference's unit tests): the
    GetValue expression I_0 + m_x (x - x0) + m_y (y - y0)
    (func_tilted-sky-plane.cpp:98-104) in the parameter order I_0, m_x, m_y."""
    for (x, y) in [(1.0, 1.0), (17.5, -3.25), (400.0, 250.0)]:
        got = oracle_mod.function_value("TiltedSkyPlane", [7.5, 0.125, -0.0625], 10.0, 20.0, x, y)
        assert got == 7.5 + 0.125 * (x - 10.0) + -0.0625 * (y - 20.0)


def test_sersic_total_flux_known_answers(oracle_mod):
    # unit_tests/unittest_funcs.t.h:447-500
    for ell, n, want, tol in [(0.0, 1.0, 1194.839934018338, 1e-9), (0.25, 1.0, 0.75 * 1194.839934018338, 1e-9),
                              (0.0, 4.0, 2266.523319362499, 1e-9), (0.0, 0.5, 906.370725112331, 1e-9),
                              (0.0, 10.0, 3546.3105962151512, 1e-7)]:
        got = oracle_mod.function_total_flux("Sersic", [90, ell, n, 1.0, 10.0])
        assert abs(got - want) <= tol


def test_n3073_chi2_and_cash_goldens(oracle_mod):
    # tests/imfit_reference/imfit_textout4c:24 and imfit_textout4d
    m, d = _n3073_model(oracle_mod, "chi2")
    chi2 = m.get_fit_statistic(d["params"])
    assert abs(chi2 - float(d["chi2_printed"])) < 5e-7
    assert chi2 == float(d["chi2_ref"])
    assert m.n_valid == 28754
    m, d = _n3073_model(oracle_mod, "cash")
    cash = m.get_fit_statistic(d["params"])
    assert abs(cash - float(d["cash_printed"])) < 5e-7
    assert cash == float(d["cash_ref"])


def test_n3073_deviates_match_reference_fixture(oracle_mod):
    m, d = _n3073_model(oracle_mod, "chi2")
    dev = m.compute_deviates(d["params"])
    assert np.array_equal(dev, d["deviates_ref"])


def test_small_case_matches_reference_fixture(oracle_mod):
    from imfit_gb300 import workloads
    g = np.load(os.path.join(GOLDEN, "small_case.npz"))
    for stat in ("chi2", "cash", "pmlr"):
        wl = workloads.small_case(stat=stat)
        wl.data = g[f"{stat}_data"]
        m = workloads.configure(oracle_mod.OracleModel(), wl)
        for tag, p in (("truth", wl.truth), ("start", wl.start)):
            assert m.get_fit_statistic(p) == float(g[f"{stat}_{tag}_stat"])
            assert np.array_equal(m.compute_deviates(p), g[f"{stat}_{tag}_dev"])
            assert np.array_equal(m.get_model_image(), g[f"{stat}_{tag}_model"])


def test_makeimage_goldens(oracle_mod):
    g = np.load(os.path.join(GOLDEN, "makeimage.npz"))
    m = oracle_mod.OracleModel()
    m.add_function("Sersic", True)
    m.add_function("Exponential")
    m.finish_functions()
    m.setup_model_image(512, 512)
    m.create_model_image(g["se_params"])
    img = m.get_model_image().astype(np.float32)
    assert np.array_equal(img[192:320, 192:320], g["se_center"])
    corners = np.stack([img[:16, :16], img[:16, -16:], img[-16:, :16], img[-16:, -16:]])
    assert np.array_equal(corners, g["se_corners"])
    m = oracle_mod.OracleModel()
    m.add_function("Gaussian", True)
    m.finish_functions()
    m.add_psf(g["psf_standard"].astype(np.float64))
    m.setup_model_image(200, 200)
    m.add_oversampled_psf(g["psf_oversamp"].astype(np.float64), int(g["ov_scale"]), tuple(g["ov_region"]))
    m.create_model_image(g["ov_params"])
    img = m.get_model_image()
    # FFT-inclusive (FFTW vs the project FFT): normwise 1e-10 in FP64, then float32 storage
    assert normwise(img, g["ov_image"]) < 1e-7


def test_qags_matches_scipy_quadpack(oracle_mod):
    """The restated QAGS agrees with QUADPACK's DQAGSE (scipy.integrate.quad) on the
    line-of-sight integrands of both 3-D functions."""
    scipy_int = pytest.importorskip("scipy.integrate")
    lib = oracle_mod._load("orc")
    import ctypes
    for name, params, pts in [
        ("FerrersBar3D", [20, 85, 40, 1, 30, 0.4, 0.2667, 2], [(10.0, 5.0), (3.2, -1.7), (25.0, 2.0)]),
        ("ExponentialDisk3D", [10, 88, 1.0, 40, 1, 6], [(12.0, 3.0), (-5.5, 0.25), (80.0, -2.0)]),
    ]:
        for (dx, dy) in pts:
            got = oracle_mod.function_value(name, params, 0.0, 0.0, dx, dy, subsampling=False)
            # reference integrand, restated in Python
            pa = np.radians(params[0] + 90.0)
            inc = np.radians(params[1])
            xp = dx * np.cos(pa) + dy * np.sin(pa)
            yp = -dx * np.sin(pa) + dy * np.cos(pa)
            x0, y0, z0 = xp, yp * np.cos(inc), yp * np.sin(inc)
            if name == "FerrersBar3D":
                bpa = np.radians(params[2] + 90.0)
                a2 = params[4] ** 2
                b2 = params[5] ** 2 * a2
                c2 = params[6] ** 2 * a2
                lim = 1.01 * max(np.sqrt(b2) * np.sin(inc), params[4])

                def f(s):
                    yd = y0 + s * np.sin(inc)
                    zd = z0 - s * np.cos(inc)
                    xb = x0 * np.cos(bpa) + yd * np.sin(bpa)
                    yb = -x0 * np.sin(bpa) + yd * np.cos(bpa)
                    m2 = yb * yb / a2 + xb * xb / b2 + zd * zd / c2
                    return 0.0 if m2 > 1 else params[3] * (1 - m2) ** params[7]
            else:
                h, n, zz0 = params[3], params[4], params[5]
                alpha = 2.0 / n
                lim = 20 * h

                def f(s):
                    yd = y0 + s * np.sin(inc)
                    zd = abs(z0 - s * np.cos(inc))
                    R = np.sqrt(x0 * x0 + yd * yd)
                    vs = (2 ** alpha) * np.exp(-zd / zz0) if zd / (alpha * zz0) > 100 else \
                        (1 / np.cosh(zd / (alpha * zz0))) ** alpha
                    return params[2] * np.exp(-R / h) * vs
            want = scipy_int.quad(f, -lim, lim, epsabs=0, epsrel=1e-6, limit=1000)[0]
            assert abs(got - want) <= 1e-9 * max(abs(want), 1.0), (name, dx, dy, got, want)


def test_fft_matches_numpy(oracle_mod):
    """The oracle convolution equals a direct numpy FFT convolution (FP64)."""
    rng = np.random.default_rng(3)
    img = rng.random((23, 31))
    psf = rng.random((7, 5))
    m = oracle_mod.OracleModel()
    m.add_function("FlatSky", True)
    m.finish_functions()
    m.add_psf(psf, normalize=False)
    m.setup_model_image(31 - 10, 23 - 14)  # model = 31 x 23 after padding by 2P
    m.create_model_image([0, 0, 1.0])
    out = m.get_expanded_model_image()
    # constant image: interior of the linear convolution equals sum(psf)
    assert abs(out[11, 15] - psf.sum()) < 1e-12


@pytest.mark.skipif(not oracle.reference_checkout(), reason="reference checkout not present")
def test_restatement_bit_identical_to_reference(oracle_mod):
    from imfit_gb300 import workloads
    oracle_mod.build_reference()
    for stat in ("chi2", "cash", "pmlr"):
        wl = workloads.small_case(seed=11, stat=stat)
        workloads.synthesize(wl, oracle_mod.OracleModel)
        o = workloads.configure(oracle_mod.OracleModel(), wl)
        r = workloads.configure(oracle_mod.RefModel(), wl)
        for p in (wl.truth, wl.start):
            assert o.get_fit_statistic(p) == r.get_fit_statistic(p)
            assert np.array_equal(o.compute_deviates(p), r.compute_deviates(p))
            assert np.array_equal(o.get_model_image(), r.get_model_image())
        assert np.array_equal(o.get_weights(), r.get_weights())
        o.use_bootstrap(5)
        r.use_bootstrap(5)
        assert o.get_fit_statistic(wl.start) == r.get_fit_statistic(wl.start)


@pytest.mark.skipif(not oracle.reference_checkout(), reason="reference checkout not present")
def test_tilted_sky_plane_matches_reference(oracle_mod):
    """Sersic + TiltedSkyPlane (own function set) convolved with an
    off-centre PSF: the oracle's model image equals the reference's."""
    oracle_mod.build_reference()
    yy, xx = np.mgrid[0:15, 0:15] - 7.0
    psf = np.exp(-((xx - 0.6) ** 2 + yy ** 2) / 5.0)
    p = [20.3, 18.6, 25.0, 0.3, 1.8, 30.0, 5.0, 21.0, 19.0, 12.0, 0.05, -0.03]
    imgs = []
    for cls in (oracle_mod.OracleModel, oracle_mod.RefModel):
        m = cls()
        m.add_function("Sersic", True)
        m.add_function("TiltedSkyPlane", True)
        m.finish_functions()
        m.add_psf(psf)
        m.setup_model_image(41, 37)
        m.create_model_image(p)
        imgs.append(m.get_model_image())
    assert np.array_equal(imgs[0], imgs[1])


def test_ic3478_printed_fit_statistic(oracle_mod):
    """tests/imfit_reference/imfit_textout3: chi^2 (data-based errors) at the
    printed best-fit parameters of ic3478rss_64x64.fits is the printed
    CHI-SQUARE; the printed values are rounded to 6 digits, which moves chi^2
    by far less than 1e-6 at a minimum."""
    d = np.load(os.path.join(GOLDEN, "ic3478.npz"))
    m = oracle_mod.OracleModel()
    m.add_function("Sersic", True)
    m.finish_functions()
    m.add_image_data(d["data"].astype(np.float64))
    m.add_image_characteristics(float(d["gain"]), float(d["read_noise"]), 1.0, 1, float(d["original_sky"]))
    assert m.final_setup() == 0
    s = m.get_fit_statistic(d["lm_params_printed"])
    assert abs(s - float(d["lm_chi2_printed"])) < 1e-6 * float(d["lm_chi2_printed"]), s
    assert abs(s / (64 * 64 - 7) - float(d["lm_reduced_printed"])) < 1e-6


def test_psf_interpolators_known_answers(oracle_mod):
    """unit_tests/unittest_psf_interpolators.t.h (DELTA = 1e-8): GSL bicubic
    and Lanczos2 on psf_gauss_sigma0.5_5.fits, and the Lanczos kernel."""
    d = np.load(os.path.join(GOLDEN, "pointsource.npz"))
    psf = d["psf5"].astype(np.float64)
    dx = np.array([0.0, 1.0, 0.0, 0.0, 0.5, 1.5, 0.0])
    dy = np.array([0.0, 0.0, 1.0, -2.0, 0.0, 0.5, 1.5])
    want = [0.73212016, 0.16868566, 0.16868566, 0.0014417765, 0.51973038, 0.00880937, 0.01243073]
    assert np.all(np.abs(oracle_mod.interpolate_psf("bicubic", psf, dx, dy) - want) < 1e-8)
    dx = np.array([0.0, 1.0, 0.0, 0.0, 0.5, 1.5, 0.0, -1.5, -1.9])
    dy = np.array([0.0, 0.0, 1.0, -2.0, 0.0, 0.5, 1.5, -1.5, -1.9])
    want = [0.73212016, 0.16868566, 0.16868566, 0.0014417765, 0.5054706567431267, 0.035119419221815946,
            0.050885502118477165, 0.00352206909108757, 0.0002065470426474115]
    assert np.all(np.abs(oracle_mod.interpolate_psf("lanczos2", psf, dx, dy) - want) < 1e-8)
    for n, xs, ys in ((2, [0.0, 0.5, 1.0, 1.5, 2.0, 3.0], [1.0, 0.5731591682507563, 0.0, -0.06368435202786181,
                                                         0.0, 0.0]),
                      (3, [0.0, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 4.0],
                       [1.0, 0.6079271018540265, 0.0, -0.13509491152311703, 0.0, 0.02431708407416106, 0.0, 0.0])):
        for x, y in zip(xs, ys):
            assert abs(oracle_mod.lanczos(x, n) - y) < 1e-8 and abs(oracle_mod.lanczos(-x, n) - y) < 1e-8
    # outside the PSF's extent: zero
    assert np.all(oracle_mod.interpolate_psf("bicubic", psf, [2.01, 0.0], [0.0, -2.5]) == 0.0)


def test_point_source_oversampled_golden(oracle_mod):
    """do_makeimage_tests:74 -> tests/oversampled_pointsource.fits: a
    PointSource (bicubic) at (100, 100), psf_standard.fits, region
    80:120,80:120 at scale 3 with psf_oversamp.fits (interpolated as given,
    unnormalised).  The reference image is float32: within one float32 ulp."""
    d = np.load(os.path.join(GOLDEN, "pointsource.npz"))
    g = np.load(os.path.join(GOLDEN, "makeimage.npz"))
    m = oracle_mod.OracleModel()
    m.add_function("PointSource", True)
    m.finish_functions()
    m.add_psf(g["psf_standard"].astype(np.float64))
    m.setup_model_image(200, 200)
    m.add_oversampled_psf(g["psf_oversamp"].astype(np.float64), int(d["ps_scale"]), tuple(d["ps_region"]))
    m.create_model_image(d["ps_params"])
    img = m.get_model_image()
    want = d["ps_image"]
    ulp = np.spacing(np.abs(want)).astype(np.float64)
    assert np.all(np.abs(img - want) <= ulp + 1e-12), np.max(np.abs(img - want) / (ulp + 1e-30))


@pytest.mark.skipif(not oracle.reference_checkout(), reason="reference checkout not present")
@pytest.mark.parametrize("inc", [80.0, 86.5, 90.0])
@pytest.mark.parametrize("psf", [False, True])
def test_los3d_restatement_bit_identical_to_reference(oracle_mod, inc, psf):
    """ExponentialDisk3D + FerrersBar3D (function_objects/func_expdisk3d.cpp:149-268,
    func_ferrersbar3d.cpp:125-261, integrated by core/integrator.cpp:42-55):
    the restatement's model image and chi^2 equal the reference's own
    sources compiled here, with and without a PSF, edge-on to 80 degrees."""
    from imfit_gb300 import workloads
    oracle_mod.build_reference()
    wl = workloads.c3(size=48, psf_size=15)
    if not psf:
        wl.psf = None
    for i in (3, 9):
        wl.truth[i] = inc
    wl.start[3] = wl.start[9] = min(inc + 0.7, 90.0)
    workloads.synthesize(wl, oracle_mod.OracleModel)
    o = workloads.configure(oracle_mod.OracleModel(), wl)
    r = workloads.configure(oracle_mod.RefModel(), wl)
    for p in (wl.truth, wl.start):
        assert o.get_fit_statistic(p) == r.get_fit_statistic(p)
        assert np.array_equal(o.get_model_image(), r.get_model_image())


def test_los3d_golden(oracle_mod):
    """The restatement against the reference's own 96x96 3-D images and chi^2
    (tests/golden/los3d.npz, written by oracle/_ref): equal to 1e-12."""
    from imfit_gb300 import workloads
    d = np.load(os.path.join(GOLDEN, "los3d.npz"))
    wl = workloads.c3(size=96, psf_size=15)
    wl.data = d["data"]
    nopsf = workloads.c3(size=96, psf_size=15)
    nopsf.psf = None
    m0 = workloads.configure(oracle_mod.OracleModel(), nopsf, with_data=False)
    m = workloads.configure(oracle_mod.OracleModel(), wl)
    for tag in ("truth", "start"):
        p = d[tag]
        m0.create_model_image(p)
        assert normwise(m0.get_model_image(), d[f"{tag}_model_nopsf"]) < 1e-12
        s = m.get_fit_statistic(p)
        assert abs(s - float(d[f"{tag}_stat"])) <= 1e-12 * abs(float(d[f"{tag}_stat"]))
        assert normwise(m.get_model_image(), d[f"{tag}_model"]) < 1e-12


def test_reference_qags_tolerance_error_at_disk_centre(oracle_mod):
    """The reference integrates the line of sight with QAGS at epsrel 1e-6
    (core/integrator.cpp:42-55).  Its own 96x96 ExponentialDisk3D + FerrersBar3D
    image (los3d.npz) differs from near-exact integrals (QAGS at epsrel 1e-11)
    by several 1e-5 of the image maximum, at the disk's centre pixel: the
    radial cusp at y_d = 0 falls inside one of its panels there.  This pins
    why the fast form is compared with exact integrals and not pixel by pixel
    with the reference."""
    from imfit_gb300 import workloads
    d = np.load(os.path.join(GOLDEN, "los3d.npz"))
    wl = workloads.c3(size=96, psf_size=15)
    wl.psf = None
    m = workloads.configure(oracle_mod.OracleModel(), wl, with_data=False)
    oracle_mod.set_los_epsrel(1e-11)
    try:
        m.create_model_image(d["truth"])
        exact = m.get_model_image()
    finally:
        oracle_mod.set_los_epsrel(0)
    ref = d["truth_model_nopsf"]
    diff = np.abs(ref - exact) / np.abs(exact).max()
    assert 1e-5 < diff.max() < 2e-4
    r, c = np.unravel_index(np.argmax(diff), diff.shape)
    rc, cc = np.unravel_index(np.argmax(exact), exact.shape)
    assert abs(r - rc) <= 2 and abs(c - cc) <= 2
    # away from the centre the reference's integrals are good to ~1e-8
    far = np.ones_like(diff, dtype=bool)
    far[rc - 4:rc + 5, cc - 4:cc + 5] = False
    assert diff[far].max() < 1e-6


@pytest.mark.parametrize("name", ["C1", "C2", "C3", "C4"])
def test_bench_size_oracle_matches_reference_golden(oracle_mod, name):
    """The restatement at the benchmark configurations' full sizes (C2: padded
    FFT of 1150 + 63 - 1 = 1212 with a 315x315 region PSF; C3 at 512x512;
    C4 Cash) against the reference's own values (bench_sizes.npz, written by
    oracle/_ref): statistic to 1e-12, model-image digests to 1e-12."""
    import bench_cases
    fx = np.load(os.path.join(GOLDEN, "bench_sizes.npz"))
    wl = bench_cases.build(name)
    assert np.allclose(bench_cases.data_digest(wl), fx[f"{name}_data"], rtol=1e-13, atol=0)
    m = workloads_configure(oracle_mod.OracleModel, wl)
    for tag, p in bench_cases.vectors(wl):
        assert np.array_equal(p, fx[f"{name}_{tag}_params"])
        s = m.get_fit_statistic(p)
        want = float(fx[f"{name}_{tag}_stat"])
        assert abs(s - want) <= 1e-12 * abs(want), (tag, s, want)
        rows, cols, sample = bench_cases.digest(m.get_model_image())
        for got, key in ((rows, "rows"), (cols, "cols"), (sample, "sample")):
            assert normwise(got, fx[f"{name}_{tag}_{key}"]) < 1e-12, (tag, key)


def workloads_configure(cls, wl):
    from imfit_gb300 import workloads
    return workloads.configure(cls(), wl)
