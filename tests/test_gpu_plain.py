"""GPU parity of the plain FP64 path (the ModelObject drop-in) through the C ABI.

Tolerances (from the specification of the plain form):
  * model image without PSF: per-pixel relative 1e-12;
  * anything after the FFT convolution: normwise 1e-10 (max |d| / max |ref|);
  * fit statistics: relative 1e-10;
  * mask / weight / extra-term preparation: bit-exact.
The reference values come from the C restatement (oracle/) run on the same
inputs, and from fixtures produced by the reference's own code.
"""
import os

import numpy as np
import pytest

from helpers import normwise, pixelwise, relerr

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _pair(gpu, oracle_mod, wl):
    from imfit_gb300 import workloads
    g = workloads.configure(gpu.ModelObject(), wl)
    o = workloads.configure(oracle_mod.OracleModel(), wl)
    return g, o


@pytest.mark.parametrize("stat", ["chi2", "cash", "pmlr"])
def test_small_case_parity(gpu, oracle_mod, stat):
    from imfit_gb300 import workloads
    fx = np.load(os.path.join(GOLDEN, "small_case.npz"))
    wl = workloads.small_case(stat=stat)
    wl.data = fx[f"{stat}_data"]
    g, o = _pair(gpu, oracle_mod, wl)
    assert g.n_valid == o.n_valid
    assert np.array_equal(g.get_weights(), o.get_weights())
    for tag, p in (("truth", wl.truth), ("start", wl.start)):
        sg, so = g.get_fit_statistic(p), o.get_fit_statistic(p)
        assert relerr(sg, so) < 1e-10, (tag, sg, so)
        assert relerr(sg, float(fx[f"{stat}_{tag}_stat"])) < 1e-10
        mg = g.get_model_image()
        assert normwise(mg, o.get_model_image()) < 1e-10
        assert normwise(mg, fx[f"{stat}_{tag}_model"]) < 1e-10
        dg, do = g.compute_deviates(p), o.compute_deviates(p)
        assert normwise(dg, do) < 1e-10
        eo = o.get_expanded_model_image()
        assert normwise(g.get_expanded_model_image(), eo) < 1e-10


def test_model_without_psf_pixelwise_1e12(gpu, oracle_mod):
    """Pre-FFT parity: Sersic + Exponential + GaussianRing + Moffat + Gaussian
    + FlatSky, subsampling on, no PSF."""
    fns = [("Sersic", True), ("Exponential", False), ("GaussianRing", False), ("Moffat", True),
           ("Gaussian", False), ("FlatSky", False)]
    p = [40.2, 30.7, 30.0, 0.3, 2.7, 12.0, 8.0, 70.0, 0.5, 6.0, 11.0, 20.0, 0.2, 2.0, 14.0, 3.0,
         20.6, 41.4, 0.0, 0.1, 50.0, 3.5, 2.5, 10.0, 0.0, 7.0, 0.9, 1.5]
    models = []
    for cls in (gpu.ModelObject, oracle_mod.OracleModel):
        m = cls()
        for n, s in fns:
            m.add_function(n, s)
        m.finish_functions()
        m.setup_model_image(80, 60)
        m.create_model_image(p)
        models.append(m.get_model_image())
    assert pixelwise(models[0], models[1]) < 1e-12


def test_small_re_subsampling_branch(gpu, oracle_mod):
    """r_e <= 1 and r <= 1 gives up to 100 x 100 subsamples per pixel."""
    p = [10.3, 10.6, 0.0, 0.2, 4.0, 100.0, 0.3]
    out = []
    for cls in (gpu.ModelObject, oracle_mod.OracleModel):
        m = cls()
        m.add_function("Sersic", True)
        m.finish_functions()
        m.setup_model_image(21, 21)
        m.create_model_image(p)
        out.append(m.get_model_image())
    assert pixelwise(out[0], out[1]) < 1e-12


def test_n3073_golden(gpu):
    """tests/imfit_reference/imfit_textout4c:24 (chi^2) and imfit_textout4d (Cash)."""
    d = np.load(os.path.join(GOLDEN, "n3073.npz"))
    for stat, key in (("chi2", "chi2"), ("cash", "cash")):
        m = gpu.ModelObject()
        m.add_function("Sersic", True)
        m.add_function("Exponential")
        m.finish_functions()
        m.add_psf(d["psf"].astype(np.float64))
        m.add_image_data(d["data"].astype(np.float64))
        m.add_image_characteristics(float(d["gain"]), float(d["read_noise"]), 1.0, 1, float(d["original_sky"]))
        m.add_mask_vector(d["mask"].astype(np.float64))
        if stat == "cash":
            m.use_cash()
        assert m.final_setup() == 0
        assert m.n_valid == 28754
        s = m.get_fit_statistic(d["params"])
        # printed to 6 decimals; a 3e8 Cash value also carries ~1e-15 relative summation-order noise
        printed = float(d[f"{key}_printed"])
        assert abs(s - printed) <= max(5e-7, 1e-14 * abs(printed))
        assert relerr(s, float(d[f"{key}_ref"])) < 1e-10
        if stat == "chi2":
            assert normwise(m.compute_deviates(d["params"]), d["deviates_ref"]) < 1e-10


def test_makeimage_goldens(gpu):
    """do_makeimage_tests: tests/sersic+exp_orig.fits and tests/oversampled_orig.fits."""
    g = np.load(os.path.join(GOLDEN, "makeimage.npz"))
    m = gpu.ModelObject()
    m.add_function("Sersic", True)
    m.add_function("Exponential")
    m.finish_functions()
    m.setup_model_image(512, 512)
    m.create_model_image(g["se_params"])
    img = m.get_model_image()
    want = g["se_center"].astype(np.float64)
    got = img[192:320, 192:320]
    # float32 storage of the reference's FP64 image: within one float32 ulp
    assert np.all(np.abs(got - want) <= np.spacing(g["se_center"]).astype(np.float64))
    assert np.mean(got.astype(np.float32) == g["se_center"]) > 0.99
    m = gpu.ModelObject()
    m.add_function("Gaussian", True)
    m.finish_functions()
    m.add_psf(g["psf_standard"].astype(np.float64))
    m.setup_model_image(200, 200)
    m.add_oversampled_psf(g["psf_oversamp"].astype(np.float64), int(g["ov_scale"]), tuple(g["ov_region"]))
    m.create_model_image(g["ov_params"])
    assert normwise(m.get_model_image(), g["ov_image"]) < 1e-7


def test_error_mask_variants(gpu, oracle_mod):
    """External sigma / variance / weight images, MASK_ZERO_IS_BAD, non-finite pixels."""
    from imfit_gb300 import workloads
    wl = workloads.small_case(seed=21, region=False, mask=False)
    workloads.synthesize(wl, oracle_mod.OracleModel)
    rng = np.random.default_rng(5)
    sig = np.sqrt(np.abs(wl.data) + 20.0)
    sig[3, 4] = 0.0  # 1/0 -> inf: masked by FinalSetupForFitting
    data = wl.data.copy()
    data[5, 6] = np.nan  # non-finite data pixel: masked
    mask = (rng.random(data.shape) > 0.08).astype(np.float64)  # 1 = good
    for etype, err in ((100, sig), (110, sig ** 2), (120, 1.0 / np.where(sig > 0, sig, 1.0) ** 2)):
        res = []
        for cls in (gpu.ModelObject, oracle_mod.OracleModel):
            m = cls()
            for n, s in wl.functions:
                m.add_function(n, s)
            m.finish_functions()
            m.add_psf(wl.psf)
            m.add_image_data(data)
            m.add_image_characteristics(wl.gain, wl.read_noise, 1.0, 1, wl.original_sky)
            m.add_error_vector(err, etype)
            m.add_mask_vector(mask, 20)
            res.append((m.final_setup(), m.n_valid, m.get_weights(), m.get_fit_statistic(wl.start)))
        assert res[0][0] == res[1][0]
        assert res[0][1] == res[1][1]
        assert np.array_equal(res[0][2], res[1][2])
        assert relerr(res[0][3], res[1][3]) < 1e-10


def test_model_errors_and_bootstrap(gpu, oracle_mod):
    from imfit_gb300 import workloads
    wl = workloads.small_case(seed=31)
    workloads.synthesize(wl, oracle_mod.OracleModel)
    g = gpu.ModelObject()
    o = oracle_mod.OracleModel()
    for m in (g, o):
        for n, s in wl.functions:
            m.add_function(n, s)
        m.finish_functions()
        m.add_psf(wl.psf)
        m.add_image_data(wl.data)
        m.add_image_characteristics(wl.gain, wl.read_noise, 1.0, 1, wl.original_sky)
        for psf, sc, reg in wl.regions:
            m.add_oversampled_psf(psf, sc, reg)
        m.use_model_errors()
        m.add_mask_vector(wl.mask)
        assert m.final_setup() == 0
    assert relerr(g.get_fit_statistic(wl.start), o.get_fit_statistic(wl.start)) < 1e-10
    assert normwise(g.get_weights(), o.get_weights()) < 1e-12
    g.use_bootstrap(12345)
    o.use_bootstrap(12345)
    for _ in range(2):
        assert relerr(g.get_fit_statistic(wl.truth), o.get_fit_statistic(wl.truth)) < 1e-10
        assert normwise(g.compute_deviates(wl.truth, g.n_valid), o.compute_deviates(wl.truth, o.n_valid)) < 1e-10
        g.make_bootstrap_sample()
        o.make_bootstrap_sample()


def test_fd_gradient_matches_oracle_jacobian(gpu, oracle_mod):
    """Plain FP64 + forward-difference gradient = 2 J^T dev with mpfit's step rule."""
    from imfit_gb300 import workloads
    wl = workloads.small_case(seed=41, region=False)
    workloads.synthesize(wl, oracle_mod.OracleModel)
    g, o = _pair(gpu, oracle_mod, wl)
    s, grad = g.statistic_and_gradient_fd(wl.start)
    J = o.fd_jacobian(wl.start)
    dev = o.compute_deviates(wl.start)
    want = 2.0 * J @ dev
    assert relerr(s, o.get_fit_statistic(wl.start)) < 1e-10
    scale = np.abs(want) + 1e-3 * np.max(np.abs(want))
    assert np.all(np.abs(grad - want) / scale < 1e-4), (grad, want)


def test_call_order_and_input_errors(gpu):
    m = gpu.ModelObject()
    with pytest.raises(gpu.ImfitError):
        m.add_function("NoSuchFunction")
    m.add_function("Sersic", True)
    m.finish_functions()
    m.setup_model_image(16, 16)
    # PSF after SetupModelImage is an error (core/model_object.cpp:870-873)
    with pytest.raises(gpu.ImfitError):
        m.add_psf(np.ones((3, 3)))
    m2 = gpu.ModelObject()
    m2.add_function("FlatSky", True)
    m2.finish_functions()
    with pytest.raises(gpu.ImfitError):
        m2.add_psf(np.full((3, 3), np.nan))
    with pytest.raises(gpu.ImfitError):
        m2.add_psf(-np.ones((3, 3)))
    # every pixel masked -> FinalSetupForFitting returns -3
    m3 = gpu.ModelObject()
    m3.add_function("FlatSky", True)
    m3.finish_functions()
    m3.add_image_data(np.ones((8, 8)))
    m3.add_mask_vector(np.ones((8, 8)))
    assert m3.final_setup() == -3
    with pytest.raises(gpu.ImfitError):
        m3.get_model_image()  # not computed yet


def test_single_function_images_sum_to_the_model(gpu, oracle_mod):
    """GetSingleFunctionImage: with convolution and an oversampled region the
    per-function images add up to the model image (the pipeline is linear)."""
    from imfit_gb300 import workloads
    wl = workloads.small_case(seed=3, region=True)
    workloads.synthesize(wl, oracle_mod.OracleModel)
    m = workloads.configure(gpu.ModelObject(), wl)
    m.create_model_image(wl.start)
    full = m.get_model_image()
    parts = [m.get_single_function_image(wl.start, i) for i in range(len(wl.functions))]
    assert np.max(np.abs(sum(parts) - full)) <= 1e-12 * np.max(np.abs(full))
    # a background alone is flat (I_sky times the PSF sum), shown here without the region
    sky = parts[-1]
    assert np.allclose(sky[0, 0], wl.start[-1], rtol=1e-12)


def test_find_total_fluxes(gpu, oracle_mod):
    """FindTotalFluxes: analytic Sersic/Exponential (against the oracle's
    TotalFlux restatement); grid integration for a Moffat against the sum of
    the oracle's GetValue over the same grid (the reference's integration,
    subsampling included), and against the closed form
    pi alpha^2 I_0 q / (beta - 1) to the accuracy of that pixel sum."""
    m = gpu.ModelObject()
    m.add_function("Sersic", True)
    m.add_function("Exponential")
    m.add_function("Moffat")
    m.add_function("FlatSky")
    m.finish_functions()
    m.setup_model_image(10, 10)
    sersic = [30.0, 0.2, 2.5, 10.0, 12.0]
    exp_ = [50.0, 0.4, 5.0, 20.0]
    moffat = [10.0, 0.1, 100.0, 4.0, 4.0]
    p = [5.0, 5.0] + sersic + exp_ + moffat + [3.0]
    size = 241
    total, ind = m.find_total_fluxes(p, size, size)
    assert relerr(ind[0], oracle_mod.function_total_flux("Sersic", sersic)) < 1e-12
    assert relerr(ind[1], oracle_mod.function_total_flux("Exponential", exp_)) < 1e-12
    c = 0.5 * size
    ref = sum(oracle_mod.function_value("Moffat", moffat, c, c, float(j + 1), float(i + 1))
              for i in range(size) for j in range(size))
    assert relerr(ind[2], ref) < 1e-12
    fwhm, beta, q = 4.0, 4.0, 0.9
    alpha = fwhm / (2.0 * np.sqrt(2.0 ** (1.0 / beta) - 1.0))
    assert relerr(ind[2], np.pi * alpha ** 2 * 100.0 * q / (beta - 1.0)) < 2e-3
    assert ind[3] == 0.0
    assert relerr(total, ind.sum()) < 1e-15
