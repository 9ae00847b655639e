"""GPU parity at the benchmark configurations' full sizes, through the C ABI.

Every other parity test runs on small images; these run C1 (256x256, 51x51
PSF), C2 (1024x1024, 63x63 PSF, 40x40 region at 5x with a 315x315 PSF, 10 %
mask), C3 (512x512 3-D disk + bar, 35x35 PSF) and C4 (512x512, Cash, four of
the 256 parameter vectors), so the padded FFT lengths, radix schedules and
launch shapes of the benchmark itself are covered.  Against two references:
the FP64 oracle run here on the same inputs, and the reference's own values
for the same inputs (tests/golden/bench_sizes.npz, written by the
reference's hot-path sources compiled from its checkout).

Tolerances (those of the small-image tests):
  * plain FP64: statistic 1e-10 relative; model image, deviates and the
    image digests 1e-10 normwise (max |d| / max |ref|);
  * fast form: statistic 1e-5 relative; model image 2e-6 of its maximum
    (not for C3, whose reference integrals are themselves only good to
    ~1e-4 of the maximum at the disk centre);
  * adjoint gradient against FP64 central differences of the oracle's
    statistic, subsampling off: |g - g_fd| <= 2e-3 (|g_fd| + 1e-3 max|g_fd|).
"""
import os

import numpy as np
import pytest

import bench_cases
from helpers import normwise, relerr

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_cache = {}


def _case(name):
    if name not in _cache:
        _cache[name] = bench_cases.build(name)
    return _cache[name]


def _golden():
    return np.load(os.path.join(GOLDEN, "bench_sizes.npz"))


@pytest.mark.parametrize("name", bench_cases.NAMES)
def test_plain_fp64_at_bench_size(gpu, oracle_mod, name):
    wl = _case(name)
    fx = _golden()
    assert np.allclose(bench_cases.data_digest(wl), fx[f"{name}_data"], rtol=1e-13, atol=0), \
        "synthesized data differ from the fixture's"
    g = bench_cases.configure(gpu.ModelObject, wl)
    o = bench_cases.configure(oracle_mod.OracleModel, wl)
    assert g.n_valid == o.n_valid
    assert np.array_equal(g.get_weights(), o.get_weights())
    for tag, p in bench_cases.vectors(wl):
        sg, so = g.get_fit_statistic(p), o.get_fit_statistic(p)
        want = float(fx[f"{name}_{tag}_stat"])
        assert relerr(sg, so) < 1e-10, (tag, sg, so)
        assert relerr(sg, want) < 1e-10, (tag, sg, want)
        mg = g.get_model_image()
        assert normwise(mg, o.get_model_image()) < 1e-10, tag
        for got, key in zip(bench_cases.digest(mg), ("rows", "cols", "sample")):
            assert normwise(got, fx[f"{name}_{tag}_{key}"]) < 1e-10, (tag, key)
        if wl.stat == "chi2":
            assert normwise(g.compute_deviates(p), o.compute_deviates(p)) < 1e-10, tag


@pytest.mark.parametrize("name", bench_cases.NAMES)
def test_fast_statistic_at_bench_size(gpu, oracle_mod, name):
    wl = _case(name)
    g = bench_cases.configure(gpu.ModelObject, wl)
    o = bench_cases.configure(oracle_mod.OracleModel, wl)
    vecs = bench_cases.vectors(wl)
    P = np.array([p for _, p in vecs])
    S, G = g.batch_statistic_and_gradient(P)
    for (tag, p), sb in zip(vecs, S):
        so = o.get_fit_statistic(p)
        sf = g.fit_statistic_fast(p)
        assert relerr(sf, so) < 1e-5, (tag, sf, so)
        assert relerr(sb, so) < 1e-5, (tag, sb, so)
        if name != "C3":
            o.create_model_image(p)
            ref = o.get_model_image()
            fast = g.get_fast_model_image(p)
            assert np.max(np.abs(fast - ref)) / np.max(np.abs(ref)) < 2e-6, tag
    assert np.all(np.isfinite(G))


def _central_fd(o, p, rel):
    fd = np.empty(len(p))
    for j in range(len(p)):
        h = rel * max(abs(p[j]), 1.0)
        a = np.array(p, dtype=float)
        b = a.copy()
        a[j] += h
        b[j] -= h
        fd[j] = (o.get_fit_statistic(a) - o.get_fit_statistic(b)) / (2 * h)
    return fd


@pytest.mark.parametrize("name", bench_cases.NAMES)
def test_adjoint_gradient_at_bench_size(gpu, oracle_mod, name):
    wl = _case(name)
    g = bench_cases.configure(gpu.ModelObject, wl, subsampling=False)
    o = bench_cases.configure(oracle_mod.OracleModel, wl, subsampling=False)
    p = bench_cases.vectors(wl)[-1][1] if wl.batch is None else wl.batch[0]
    s, grad = g.statistic_and_gradient(p)
    assert relerr(s, o.get_fit_statistic(p)) < 1e-5
    # 3-D integrals: a larger step keeps QAGS's panel changes out of the quotient
    fd = _central_fd(o, p, 1e-4 if name == "C3" else 1e-5)
    scale = np.abs(fd) + 1e-3 * np.max(np.abs(fd))
    err = np.abs(grad - fd) / scale
    assert np.all(err < 2e-3), list(zip(g.parameter_names(), grad, fd, err))
