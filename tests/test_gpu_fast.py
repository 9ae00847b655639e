"""GPU checks of the fast path (FP32 evaluation, FP64 reductions, adjoint
gradient) through the C ABI.

Tolerances:
  * statistic: relative 1e-5 against the FP64 oracle (the accuracy target of
    the fast form);
  * gradient: against FP64 central finite differences of the oracle's
    statistic, with subsampling off (the subsample count switches make the
    model only piecewise smooth): |g - g_fd| <= 2e-3 * (|g_fd| + 1e-3 max|g_fd|);
  * repeated calls are bit-identical; batched evaluation matches single-vector
    calls to 2e-6 relative (the autotuner may pick different CTA shapes for
    different batch sizes, which changes the FP32 per-CTA partial sums).
"""
import numpy as np
import pytest

from helpers import relerr

pytestmark = pytest.mark.gpu


def _wl(oracle_mod, stat="chi2", region=True, seed=7, subsample=True):
    from imfit_gb300 import workloads
    wl = workloads.small_case(seed=seed, stat=stat, region=region)
    if not subsample:
        wl.functions = list(wl.functions)
    workloads.synthesize(wl, oracle_mod.OracleModel)
    return wl


def _build(cls, wl, subsample=True):
    from imfit_gb300 import workloads
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


@pytest.mark.parametrize("stat", ["chi2", "cash", "pmlr"])
@pytest.mark.parametrize("region", [False, True])
def test_fast_statistic_within_1e5(gpu, oracle_mod, stat, region):
    wl = _wl(oracle_mod, stat=stat, region=region)
    g = _build(gpu.ModelObject, wl)
    o = _build(oracle_mod.OracleModel, wl)
    for p in (wl.truth, wl.start):
        sf = g.fit_statistic_fast(p)
        so = o.get_fit_statistic(p)
        assert relerr(sf, so) < 1e-5, (sf, so)
        sg, _ = g.statistic_and_gradient(p)
        assert sg == sf


def test_fast_model_image_close_to_fp64(gpu, oracle_mod):
    wl = _wl(oracle_mod)
    g = _build(gpu.ModelObject, wl)
    o = _build(oracle_mod.OracleModel, wl)
    o.create_model_image(wl.start)
    ref = o.get_model_image()
    fast = g.get_fast_model_image(wl.start)
    assert np.max(np.abs(fast - ref)) / np.max(np.abs(ref)) < 2e-6


def _central_fd(o, p, rel=1e-5):
    g = np.empty(len(p))
    for j in range(len(p)):
        h = rel * max(abs(p[j]), 1.0)
        a = np.array(p, dtype=float)
        b = a.copy()
        a[j] += h
        b[j] -= h
        g[j] = (o.get_fit_statistic(a) - o.get_fit_statistic(b)) / (2 * h)
    return g


@pytest.mark.parametrize("stat", ["chi2", "cash"])
@pytest.mark.parametrize("region", [False, True])
def test_adjoint_gradient_vs_central_fd(gpu, oracle_mod, stat, region):
    wl = _wl(oracle_mod, stat=stat, region=region, seed=13)
    g = _build(gpu.ModelObject, wl, subsample=False)
    o = _build(oracle_mod.OracleModel, wl, subsample=False)
    p = wl.start
    s, grad = g.statistic_and_gradient(p)
    fd = _central_fd(o, p)
    scale = np.abs(fd) + 1e-3 * np.max(np.abs(fd))
    err = np.abs(grad - fd) / scale
    assert np.all(err < 2e-3), list(zip(g.parameter_names(), grad, fd, err))


def test_adjoint_gradient_with_subsampling_near_fd(gpu, oracle_mod):
    """With subsampling on, the analytic gradient (subsample counts frozen)
    still tracks a small-step FD of the FP64 statistic."""
    wl = _wl(oracle_mod, seed=17, region=False)
    g = _build(gpu.ModelObject, wl)
    o = _build(oracle_mod.OracleModel, wl)
    s, grad = g.statistic_and_gradient(wl.start)
    fd = _central_fd(o, wl.start, rel=1e-6)
    scale = np.abs(fd) + 1e-2 * np.max(np.abs(fd))
    assert np.median(np.abs(grad - fd) / scale) < 1e-2


def test_batch_equals_single_calls(gpu, oracle_mod):
    wl = _wl(oracle_mod, region=True)
    g = _build(gpu.ModelObject, wl)
    rng = np.random.default_rng(2)
    P = np.array([wl.start * (1 + 0.02 * rng.standard_normal(len(wl.start))) for _ in range(5)])
    P[:, 3] = np.clip(P[:, 3], 0.05, 0.8)
    S, G = g.batch_statistic_and_gradient(P)
    S2, G2 = g.batch_statistic_and_gradient(P)
    assert np.array_equal(S, S2) and np.array_equal(G, G2)
    for b in range(len(P)):
        s1, g1 = g.statistic_and_gradient(P[b])
        assert relerr(s1, S[b]) < 2e-6
        scale = np.abs(G[b]) + 1e-3 * np.max(np.abs(G[b]))
        assert np.all(np.abs(g1 - G[b]) / scale < 1e-4)


def test_graph_replay_equals_direct_launch(gpu, oracle_mod):
    wl = _wl(oracle_mod, region=True)
    g = _build(gpu.ModelObject, wl)
    g.set_use_graphs(True)
    a = g.batch_statistic_and_gradient(np.stack([wl.start, wl.truth]))
    b = g.batch_statistic_and_gradient(np.stack([wl.start, wl.truth]))
    g.set_use_graphs(False)
    c = g.batch_statistic_and_gradient(np.stack([wl.start, wl.truth]))
    for x, y in ((a, b), (a, c)):
        assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])


def test_fast_bootstrap_matches_fp64(gpu, oracle_mod):
    wl = _wl(oracle_mod, region=False, seed=19)
    g = _build(gpu.ModelObject, wl)
    o = _build(oracle_mod.OracleModel, wl)
    g.use_bootstrap(99)
    o.use_bootstrap(99)
    assert relerr(g.fit_statistic_fast(wl.start), o.get_fit_statistic(wl.start)) < 1e-5
    assert relerr(g.get_fit_statistic(wl.start), o.get_fit_statistic(wl.start)) < 1e-10


def test_no_psf_fast_path(gpu, oracle_mod):
    from imfit_gb300 import workloads
    wl = _wl(oracle_mod, region=False, seed=23)
    wl.psf = None
    workloads.synthesize(wl, oracle_mod.OracleModel)
    g = workloads.configure(gpu.ModelObject(), wl)
    o = workloads.configure(oracle_mod.OracleModel(), wl)
    assert relerr(g.fit_statistic_fast(wl.start), o.get_fit_statistic(wl.start)) < 1e-5


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_oversampled_region_scales(gpu, oracle_mod, k):
    """Region scales whose subsample table uses the shared lattice (k = 2, 4,
    5: k divides the 20 x 20 count) and one that does not (k = 3): fast
    statistic and model image against the FP64 oracle, and the gradient with
    subsampling on (the lattice's derivative channels) against a small-step
    FD of the FP64 statistic."""
    from imfit_gb300 import workloads
    wl = workloads.small_case(seed=19, region=True)
    wl.regions = [(workloads.moffat_psf(15 * k | 1, k * 2.5, 3.0), k, (26, 33, 19, 26))]  # odd side
    workloads.synthesize(wl, oracle_mod.OracleModel)
    g = _build(gpu.ModelObject, wl)
    o = _build(oracle_mod.OracleModel, wl)
    for p in (wl.truth, wl.start):
        assert relerr(g.fit_statistic_fast(p), o.get_fit_statistic(p)) < 1e-5
    o.create_model_image(wl.start)
    ref = o.get_model_image()
    assert np.max(np.abs(g.get_fast_model_image(wl.start) - ref)) / np.max(np.abs(ref)) < 2e-6
    s, grad = g.statistic_and_gradient(wl.start)
    fd = _central_fd(o, wl.start, rel=1e-6)
    scale = np.abs(fd) + 1e-2 * np.max(np.abs(fd))
    assert np.median(np.abs(grad - fd) / scale) < 1e-2, list(zip(g.parameter_names(), grad, fd))
