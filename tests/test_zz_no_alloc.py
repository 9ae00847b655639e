"""GPU test of imfit_ChiSquaredDeviceNoAlloc, the allocation-free chi^2.

It exists for callers that may not allocate device memory when they need a
statistic (framework plug-ins whose host reserves all device memory, fixed
device budgets, solver loops that cannot pay for the allocator).  The test
calls it through the C ABI on device arrays and compares it with the existing
entry point imfit_GetFitStatistic on the same model, data and weights, within
the 1e-10 relative tolerance the plain-path statistic tests use, on two calls
in a row (the second with a different model, so stale partial sums left in
the shared array by the first call would show).  This file is collected last
so a run that stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model_and_data(gpu):
    ncols, nrows = 170, 130
    truth = [85.3, 64.6, 30.0, 0.3, 2.0, 20.0, 12.0, 50.0]
    mk = gpu.ModelObject()
    mk.add_function("Sersic", True)
    mk.add_function("FlatSky")
    mk.finish_functions()
    mk.setup_model_image(ncols, nrows)
    mk.create_model_image(truth)
    img = mk.get_model_image()
    rng = np.random.default_rng(2024)
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
    return m, data, weights, truth


def test_no_alloc_chi2_matches_existing_entry_point(gpu):
    torch = pytest.importorskip("torch")
    lib = gpu.load_library()
    m, data, weights, truth = _model_and_data(gpu)
    dev = torch.device("cuda", 0)
    d_data = torch.tensor(data.ravel(), dtype=torch.float64, device=dev)
    d_w = torch.tensor(weights.ravel(), dtype=torch.float64, device=dev)
    d_out = torch.zeros(1, dtype=torch.float64, device=dev)
    n = data.size
    for p in ([85.3, 64.6, 30.0, 0.3, 2.0, 20.0, 12.0, 50.0], [84.9, 65.2, 35.0, 0.25, 2.4, 18.0, 13.0, 51.0]):
        want = m.get_fit_statistic(p)
        d_model = torch.tensor(m.get_model_image().ravel(), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = lib.imfit_ChiSquaredDeviceNoAlloc(d_model.data_ptr(), d_data.data_ptr(), d_w.data_ptr(), n,
                                               d_out.data_ptr(), None)
        assert st == 0, lib.imfit_LastError(None)
        torch.cuda.synchronize()
        got = float(d_out.item())
        assert abs(got - want) <= 1e-10 * abs(want), (got, want)


def test_no_alloc_rejects_inputs_beyond_its_fixed_scratch(gpu):
    torch = pytest.importorskip("torch")
    lib = gpu.load_library()
    buf = torch.zeros(4, dtype=torch.float64, device=torch.device("cuda", 0))
    limit = 4096 * 2048  # IMFIT_NOALLOC_MAX_PIXELS
    st = lib.imfit_ChiSquaredDeviceNoAlloc(buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), limit + 1,
                                           buf.data_ptr(), None)
    assert st == -1
    assert b"scratch limit" in lib.imfit_LastError(None)
