"""GPU checks of the fast path's FFT plans (padded lengths x radix orders).

The autotuner chooses, per handle, among the three smallest 7-smooth even
padded lengths within 10 % of the window and three radix orders.  Every
candidate computes the same linear convolution (extra zero padding does not
change it) with a different FP32 rounding, so every candidate must give the
same statistic within 1e-6 relative, the same gradient within 1e-4 of its
largest entry, and the FP64 oracle's statistic within the fast path's 1e-5.
"""
import numpy as np
import pytest

from helpers import relerr

pytestmark = pytest.mark.gpu


def test_every_fft_plan_gives_the_same_statistic(gpu, oracle_mod):
    from imfit_gb300 import workloads
    wl = workloads.c1()  # 256x256, 51x51 PSF: window 306, candidates 320, 324, 336
    workloads.synthesize(wl, oracle_mod.OracleModel)
    g = workloads.configure(gpu.ModelObject(), wl)
    so = workloads.configure(oracle_mod.OracleModel(), wl).get_fit_statistic(wl.start)
    seen = {}
    for cand in range(3):
        for order in range(3):
            g.set_fft_plan(cand, order)
            s, grad = g.statistic_and_gradient(wl.start)
            lx, ly, o = g.fft_plan()
            assert o == order and lx >= 306 and ly >= 306 and lx <= 1.1 * 306
            assert gpu.radix_schedule(lx // 2, order) is not None and gpu.radix_schedule(ly, order) is not None
            seen[(lx, ly, o)] = (s, grad)
    assert len({k[0] for k in seen}) == 3  # three distinct padded lengths
    s0, g0 = next(iter(seen.values()))
    for (lx, ly, o), (s, grad) in seen.items():
        assert relerr(s, s0) < 1e-6, (lx, ly, o, s, s0)
        assert relerr(s, so) < 1e-5, (lx, ly, o, s, so)
        assert np.max(np.abs(grad - g0)) <= 1e-4 * np.max(np.abs(g0)), (lx, ly, o)
    # back to autotuning: the tuned plan is one of the candidates
    g.set_fft_plan(-1)
    g.statistic_and_gradient(wl.start)
    assert g.fft_plan() in seen
    shape = g.launch_shape()
    assert shape["Lx"] == g.fft_plan()[0] and shape["row_radices"] and shape["col_radices"]


def test_fft_plan_with_an_oversampled_region(gpu, oracle_mod):
    """The region's lengths follow the same candidate and order."""
    from imfit_gb300 import workloads
    wl = workloads.small_case(seed=5)
    workloads.synthesize(wl, oracle_mod.OracleModel)
    g = workloads.configure(gpu.ModelObject(), wl)
    so = workloads.configure(oracle_mod.OracleModel(), wl).get_fit_statistic(wl.start)
    stats = []
    for cand in range(3):
        for order in range(3):
            g.set_fft_plan(cand, order)
            stats.append(g.fit_statistic_fast(wl.start))
    assert max(relerr(s, stats[0]) for s in stats) < 1e-6
    assert all(relerr(s, so) < 1e-5 for s in stats)
