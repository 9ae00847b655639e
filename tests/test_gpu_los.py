"""GPU checks of the 3-D line-of-sight functions (ExponentialDisk3D,
FerrersBar3D; function_objects/func_expdisk3d.cpp, func_ferrersbar3d.cpp).

Plain FP64 form (device QAGS per pixel, the drop-in):
  * FerrersBar3D known answers of unit_tests/unittest_funcs.t.h:2068-2116 within 1e-9;
  * model image against the FP64 oracle: 1e-12 relative pixelwise without a
    PSF, 1e-10 (normwise) after the FFT convolution; statistic within 1e-10.
Fast form (FP32 warp-cooperative adaptive Gauss-Kronrod, FP64 reductions):
  * model image within 2e-6 of the maximum against near-exact integrals
    (oracle QAGS at epsrel 1e-11);
  * statistic within 1e-5 of the FP64 oracle at the reference's tolerance;
  * adjoint gradient against FP64 central differences of the oracle:
    |g - g_fd| <= 2e-3 (|g_fd| + 1e-3 max|g_fd|).
"""
import numpy as np
import pytest

from helpers import normwise, pixelwise, relerr

pytestmark = pytest.mark.gpu


def _ferrers_model(gpu, params, n=203):
    # centre at (101, 100): the reference's cases at x = 0 and x = 200 (pixel
    # centres 100 px from the centre) become x = 1 and x = 201 of this grid
    m = gpu.ModelObject()
    m.add_function("FerrersBar3D", True)
    m.finish_functions()
    m.setup_model_image(n, n)
    m.create_model_image([101.0, 100.0] + list(params))
    return m.get_model_image()


# unit_tests/unittest_funcs.t.h:2068-2116 (centre (100, 100) there), shifted by +1 in x
KNOWN = [
    ([0, 0, 0, 1, 100, 1, 1, 2], [((101, 100), 106.666666573), ((101, 150), 51.9615240239), ((1, 100), 0.0),
                                  ((202, 100), 0.0)]),
    ([0, 0, 0, 1, 100, 0.5, 1, 2], [((101, 100), 106.666666573), ((101, 50), 51.9615240239),
                                    ((126, 100), 51.9615240239), ((151, 100), 0.0)]),
]


@pytest.mark.parametrize("params,cases", KNOWN)
def test_plain_ferrers_known_answers(gpu, params, cases):
    img = _ferrers_model(gpu, params)
    for (x, y), want in cases:
        got = img[int(y) - 1, int(x) - 1]  # IRAF pixel (x, y) with no PSF padding
        assert abs(got - want) <= 1e-9, (x, y, got, want)


def _c3_small(oracle_mod, psf=True, size=96):
    from imfit_gb300 import workloads
    wl = workloads.c3(size=size, psf_size=15)
    if not psf:
        wl.psf = None
    workloads.synthesize(wl, oracle_mod.OracleModel)
    return wl


def test_plain_los_image_matches_oracle_without_psf(gpu, oracle_mod):
    from imfit_gb300 import workloads
    wl = _c3_small(oracle_mod, psf=False)
    g = workloads.configure(gpu.ModelObject(), wl, with_data=False)
    o = workloads.configure(oracle_mod.OracleModel(), wl, with_data=False)
    for p in (wl.truth, wl.start):
        g.create_model_image(p)
        o.create_model_image(p)
        assert pixelwise(g.get_model_image(), o.get_model_image()) < 1e-12


def test_plain_los_image_and_statistic_match_oracle(gpu, oracle_mod):
    from imfit_gb300 import workloads
    wl = _c3_small(oracle_mod, psf=True)
    g = workloads.configure(gpu.ModelObject(), wl)
    o = workloads.configure(oracle_mod.OracleModel(), wl)
    for p in (wl.truth, wl.start):
        sg = g.get_fit_statistic(p)
        so = o.get_fit_statistic(p)
        assert relerr(sg, so) < 1e-10, (sg, so)
        assert normwise(g.get_model_image(), o.get_model_image()) < 1e-10


def test_plain_los_fd_gradient_matches_oracle(gpu, oracle_mod):
    from imfit_gb300 import workloads
    wl = _c3_small(oracle_mod, psf=True, size=64)
    g = workloads.configure(gpu.ModelObject(), wl)
    o = workloads.configure(oracle_mod.OracleModel(), wl)
    s, grad = g.statistic_and_gradient_fd(wl.start)
    assert relerr(s, o.get_fit_statistic(wl.start)) < 1e-10
    assert np.all(np.isfinite(grad))


# ---------------------------------------------------------------- fast form
@pytest.mark.parametrize("psf", [False, True])
def test_fast_los_model_image_close_to_exact_integrals(gpu, oracle_mod, psf):
    """The fast image against the oracle's integrals at QAGS epsrel 1e-11
    (near-exact).  The reference's own epsrel-1e-6 QAGS is off by up to 6e-5
    of the image maximum at the disk's centre pixel for these parameters, so
    the fast form is compared with the exact integral, and its statistic with
    the reference-tolerance oracle (test_fast_los_statistic_within_1e5)."""
    from imfit_gb300 import workloads
    wl = _c3_small(oracle_mod, psf=psf)
    g = workloads.configure(gpu.ModelObject(), wl)
    o = workloads.configure(oracle_mod.OracleModel(), wl)
    oracle_mod.set_los_epsrel(1e-11)
    try:
        for p in (wl.truth, wl.start):
            o.create_model_image(p)
            ref = o.get_model_image()
            fast = g.get_fast_model_image(p)
            assert np.max(np.abs(fast - ref)) / np.max(np.abs(ref)) < 2e-6
    finally:
        oracle_mod.set_los_epsrel(0)


def test_fast_los_statistic_within_1e5(gpu, oracle_mod):
    from imfit_gb300 import workloads
    wl = _c3_small(oracle_mod, psf=True)
    g = workloads.configure(gpu.ModelObject(), wl)
    o = workloads.configure(oracle_mod.OracleModel(), wl)
    for p in (wl.truth, wl.start):
        sf = g.fit_statistic_fast(p)
        so = o.get_fit_statistic(p)
        assert relerr(sf, so) < 1e-5, (sf, so)
        sg, grad = g.statistic_and_gradient(p)
        assert sg == sf
        assert np.all(np.isfinite(grad))


def test_fast_los_gradient_vs_central_fd(gpu, oracle_mod):
    from imfit_gb300 import workloads
    wl = _c3_small(oracle_mod, psf=True, size=64)
    g = workloads.configure(gpu.ModelObject(), wl)
    o = workloads.configure(oracle_mod.OracleModel(), wl)
    p = wl.start
    s, grad = g.statistic_and_gradient(p)
    fd = np.empty(len(p))
    for j in range(len(p)):
        h = 1e-4 * max(abs(p[j]), 1.0)
        a = np.array(p, dtype=float)
        b = a.copy()
        a[j] += h
        b[j] -= h
        fd[j] = (o.get_fit_statistic(a) - o.get_fit_statistic(b)) / (2 * h)
    scale = np.abs(fd) + 1e-3 * np.max(np.abs(fd))
    err = np.abs(grad - fd) / scale
    assert np.all(err < 2e-3), list(zip(g.parameter_names(), grad, fd, err))


def test_fast_los_batch_is_deterministic(gpu, oracle_mod):
    from imfit_gb300 import workloads
    wl = _c3_small(oracle_mod, psf=True, size=64)
    g = workloads.configure(gpu.ModelObject(), wl)
    P = np.stack([wl.start, wl.truth, 0.5 * (wl.start + wl.truth)])
    S1, G1 = g.batch_statistic_and_gradient(P)
    S2, G2 = g.batch_statistic_and_gradient(P)
    assert np.array_equal(S1, S2) and np.array_equal(G1, G2)
    s0, g0 = g.statistic_and_gradient(P[0])
    assert relerr(s0, S1[0]) < 2e-6


def test_jtwj_rejects_los_components(gpu, oracle_mod):
    from imfit_gb300 import workloads
    wl = _c3_small(oracle_mod, psf=True, size=64)
    g = workloads.configure(gpu.ModelObject(), wl)
    with pytest.raises(gpu.ImfitError) as e:
        g.jtwj(wl.start)
    assert e.value.code == -4


def test_fast_los_with_a_point_source(gpu, oracle_mod):
    """ExponentialDisk3D + PointSource (its own function set): the 3-D
    kernels integrate the disk only and the point source is added after the
    convolution -- fast statistic against the FP64 oracle, adjoint gradient
    against the oracle's central differences."""
    from imfit_gb300 import workloads
    size = 64
    truth = np.array([32.3, 31.8, 30.0, 85.0, 0.5, 5.0, 1.0, 0.75, 20.4, 40.6, 300.0])
    wl = workloads.Workload("los+ps", size, size, [("ExponentialDisk3D", True), ("PointSource", True)], truth,
                            psf=workloads.gaussian_psf(15, 1.5), seed=17, noise="gaussian", noise_sigma=2.0)
    wl.errors = np.full((size, size), 2.0)
    workloads.synthesize(wl, oracle_mod.OracleModel)
    g = workloads.configure(gpu.ModelObject(), wl)
    o = workloads.configure(oracle_mod.OracleModel(), wl)
    p = truth * np.array([1.0, 1.0, 1.03, 0.99, 1.05, 0.96, 1.0, 1.04, 1.0, 1.0, 1.1])
    # centres off the pixel grid: with the point source's centre on a pixel
    # centre every sample falls on a knot of the bicubic interpolant, where
    # its second derivative jumps and central differences are biased
    p[[0, 8, 9]] += [0.3, -0.37, 0.25]
    s, grad = g.statistic_and_gradient(p)
    so = o.get_fit_statistic(p)
    assert relerr(s, so) < 1e-5, (s, so)
    fd = np.empty(len(p))
    for j in range(len(p)):
        h = 1e-4 * max(abs(p[j]), 1.0)
        a = np.array(p, dtype=float)
        b = a.copy()
        a[j] += h
        b[j] -= h
        fd[j] = (o.get_fit_statistic(a) - o.get_fit_statistic(b)) / (2 * h)
    # the point source's derivatives come from the FP32 interpolant's slopes:
    # the point-source tests' bound 3e-3 |g_fd| + 3e-4 max|g_fd|
    bound = 3e-3 * np.abs(fd) + 3e-4 * np.max(np.abs(fd))
    assert np.all(np.abs(grad - fd) <= bound), [(n, a, b) for n, a, b in zip(g.parameter_names(), grad, fd)]
