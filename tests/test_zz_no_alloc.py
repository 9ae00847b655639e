"""GPU tests of imfit_ChiSquaredDeviceNoAlloc, the allocation-free chi^2.

It exists for callers that may not allocate device memory when they need a
statistic (framework plug-ins whose host reserves all device memory, fixed
device budgets, solver loops that cannot pay for the allocator).  The tests
call it through the C ABI on device arrays:
  * against the existing entry point imfit_GetFitStatistic on the same model,
    data and weights, within the 1e-10 relative tolerance the plain-path
    statistic tests use, on two calls in a row -- the second on a smaller
    image, so partial sums left in the shared array by the first call's
    extra blocks would show if the second call read them;
  * at exactly the size limit (every slot of the fixed array in use) against a
    host FP64 sum, then a small call after it;
  * beyond the limit: rejected before any kernel runs (buffers sized for the
    rejected call, so a broken guard would give a wrong status, not a fault).
This file is collected last so a run that stops at the first failure has
already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 4096 * 2048  # IMFIT_NOALLOC_MAX_PIXELS


def _model_and_data(gpu, ncols, nrows, truth, seed):
    mk = gpu.ModelObject()
    mk.add_function("Sersic", True)
    mk.add_function("FlatSky")
    mk.finish_functions()
    mk.setup_model_image(ncols, nrows)
    mk.create_model_image(truth)
    img = mk.get_model_image()
    rng = np.random.default_rng(seed)
    data = img + rng.normal(0.0, 3.0, img.shape)
    sigma = np.sqrt(np.abs(data) + 9.0)
    mask = (rng.random(img.shape) < 0.05).astype(np.float64)  # 1 = bad (MASK_ZERO_IS_GOOD)
    m = gpu.ModelObject()
    m.add_function("Sersic", True)
    m.add_function("FlatSky")
    m.finish_functions()
    m.add_image_data(data)
    m.add_error_vector(sigma, gpu.WEIGHTS_ARE_SIGMAS)
    m.add_mask_vector(mask, gpu.MASK_ZERO_IS_GOOD)
    assert m.final_setup() == 0
    # internal weights exactly as AddErrorVector + ApplyMask form them
    good = (mask == 0).astype(np.float64)
    weights = good * (1.0 / sigma)
    return m, data, weights


def _call(lib, torch, model, data, weight, out, n):
    torch.cuda.synchronize()
    st = lib.imfit_ChiSquaredDeviceNoAlloc(model.data_ptr(), data.data_ptr(), weight.data_ptr(), n,
                                           out.data_ptr(), None)
    assert st == 0, lib.imfit_LastError(None)
    torch.cuda.synchronize()
    return float(out.item())


def test_no_alloc_chi2_matches_existing_entry_point(gpu):
    torch = pytest.importorskip("torch")
    lib = gpu.load_library()
    dev = torch.device("cuda", 0)
    d_out = torch.zeros(1, dtype=torch.float64, device=dev)
    # 170 x 130 = 22100 pixels (11 blocks of partial sums), then 90 x 70 = 6300 (4 blocks)
    cases = [(170, 130, [85.3, 64.6, 30.0, 0.3, 2.0, 20.0, 12.0, 50.0],
              [84.9, 65.2, 35.0, 0.25, 2.4, 18.0, 13.0, 51.0], 2024),
             (90, 70, [45.2, 35.1, 60.0, 0.2, 1.5, 30.0, 8.0, 40.0],
              [45.6, 34.7, 55.0, 0.22, 1.7, 28.0, 8.5, 41.0], 7)]
    for ncols, nrows, truth, p, seed in cases:
        m, data, weights = _model_and_data(gpu, ncols, nrows, truth, seed)
        want = m.get_fit_statistic(p)
        d_model = torch.tensor(m.get_model_image().ravel(), dtype=torch.float64, device=dev)
        d_data = torch.tensor(data.ravel(), dtype=torch.float64, device=dev)
        d_w = torch.tensor(weights.ravel(), dtype=torch.float64, device=dev)
        got = _call(lib, torch, d_model, d_data, d_w, d_out, data.size)
        assert abs(got - want) <= 1e-10 * abs(want), (ncols, nrows, got, want)


def test_no_alloc_chi2_at_the_size_limit(gpu):
    torch = pytest.importorskip("torch")
    lib = gpu.load_library()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    model = rng.normal(100.0, 10.0, LIMIT)
    data = model + rng.normal(0.0, 3.0, LIMIT)
    weight = 1.0 / rng.uniform(2.0, 4.0, LIMIT)
    weight[rng.random(LIMIT) < 0.05] = 0.0
    want = float(np.sum((weight * (data - model)) ** 2))
    d = [torch.tensor(a, dtype=torch.float64, device=dev) for a in (model, data, weight)]
    d_out = torch.zeros(1, dtype=torch.float64, device=dev)
    got = _call(lib, torch, d[0], d[1], d[2], d_out, LIMIT)
    assert abs(got - want) <= 1e-10 * abs(want), (got, want)
    # a one-block call right after: the other 4095 slots still hold the big call's sums
    n = 1000
    want = float(np.sum((weight[:n] * (data[:n] - model[:n])) ** 2))
    got = _call(lib, torch, d[0], d[1], d[2], d_out, n)
    assert abs(got - want) <= 1e-10 * abs(want), (got, want)


def test_no_alloc_rejects_inputs_beyond_its_fixed_scratch(gpu):
    torch = pytest.importorskip("torch")
    lib = gpu.load_library()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(LIMIT + 1, dtype=torch.float64, device=dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    st = lib.imfit_ChiSquaredDeviceNoAlloc(buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), LIMIT + 1,
                                           out.data_ptr(), None)
    assert st == -1
    assert b"scratch limit" in lib.imfit_LastError(None)
