"""GB300 model-image / fit-statistic library: Python mirror of ModelObject.

The compute path is the CUDA library ``_build/libimfit_gb300.so`` (built by
``imfit_gb300.build``) reached through its C ABI (include/imfit_gb300.h).
There is no CPU fallback: if the library cannot be loaded, or no GPU is
present, calls raise.

``ModelObject`` keeps the reference's method order and semantics
(core/model_object.h); method names are the reference's, in snake case.
"""
import ctypes
import os

import numpy as np

from . import build as _build

WEIGHTS_ARE_SIGMAS, WEIGHTS_ARE_VARIANCES, WEIGHTS_ARE_WEIGHTS = 100, 110, 120
MASK_ZERO_IS_GOOD, MASK_ZERO_IS_BAD = 10, 20

_lib = None

_D = ctypes.c_double
_I = ctypes.c_int
_L = ctypes.c_long
_P = ctypes.c_void_p
_DP = ctypes.POINTER(ctypes.c_double)

# (name, restype, argtypes) of every C-ABI entry point
# imfit_normal_eq_fn: (x, &statistic, A, b, user) -> status
NORMAL_EQ_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_void_p)

# imfit_normal_eq_batch_fn: (B, X, active, statistics, A, b, user) -> status
NORMAL_EQ_BATCH_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_ubyte), ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_void_p)

_SIGS = [
    ("imfit_ModelObject_new", _I, [_I, ctypes.POINTER(_P)]),
    ("imfit_ModelObject_delete", _I, [_P]),
    ("imfit_LastError", ctypes.c_char_p, [_P]),
    ("imfit_Version", ctypes.c_char_p, []),
    ("imfit_AddFunction", _I, [_P, ctypes.c_char_p]),
    ("imfit_SetSubsampling", _I, [_P, _I, _I]),
    ("imfit_DefineFunctionSets", _I, [_P, ctypes.POINTER(_I), _I]),
    ("imfit_PopulateParameterNames", _I, [_P]),
    ("imfit_GetParameterName", _I, [_P, _I, ctypes.c_char_p, _I]),
    ("imfit_AddPSFVector", _I, [_P, _L, _I, _I, _DP, _I]),
    ("imfit_SetupModelImage", _I, [_P, _I, _I]),
    ("imfit_AddImageDataVector", _I, [_P, _DP, _I, _I]),
    ("imfit_AddImageCharacteristics", _I, [_P, _D, _D, _D, _I, _D]),
    ("imfit_AddOversampledPsfInfo", _I, [_P, _DP, _I, _I, _I, _I, _I, _I, _I, _I]),
    ("imfit_AddErrorVector", _I, [_P, _L, _I, _I, _DP, _I]),
    ("imfit_AddMaskVector", _I, [_P, _L, _I, _I, _DP, _I]),
    ("imfit_UseCashStatistic", _I, [_P]),
    ("imfit_UsePoissonMLR", _I, [_P]),
    ("imfit_UseModelErrors", _I, [_P]),
    ("imfit_FinalSetupForFitting", _I, [_P]),
    ("imfit_SetMaxThreads", _I, [_P, _I]),
    ("imfit_SetOMPChunkSize", _I, [_P, _I]),
    ("imfit_GetNParams", _I, [_P]),
    ("imfit_GetNDataValues", _L, [_P]),
    ("imfit_GetNValidPixels", _L, [_P]),
    ("imfit_GetNFunctions", _I, [_P]),
    ("imfit_WhichFitStatistic", _I, [_P, _I]),
    ("imfit_GetModelImageSize", _I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("imfit_CreateModelImage", _I, [_P, _DP]),
    ("imfit_ComputeModelImage", _I, [_P, _DP]),
    ("imfit_ComputeDeviates", _I, [_P, _DP, _DP]),
    ("imfit_GetFitStatistic", _I, [_P, _DP, _DP]),
    ("imfit_ChiSquared", _I, [_P, _DP, _DP]),
    ("imfit_CashStatistic", _I, [_P, _DP, _DP]),
    ("imfit_GetModelImageVector", _I, [_P, _DP]),
    ("imfit_GetExpandedModelImageVector", _I, [_P, _DP]),
    ("imfit_GetResidualImageVector", _I, [_P, _DP]),
    ("imfit_GetWeightImageVector", _I, [_P, _DP]),
    ("imfit_GetDataVector", _I, [_P, _DP]),
    ("imfit_GetSingleFunctionImage", _I, [_P, _DP, _I, _DP]),
    ("imfit_FindTotalFluxes", _I, [_P, _DP, _I, _I, _DP, _DP]),
    ("imfit_UseBootstrap", _I, [_P, ctypes.c_ulong]),
    ("imfit_MakeBootstrapSample", _I, [_P]),
    ("imfit_GetFitStatisticAndGradientFD", _I, [_P, _DP, _DP, _DP]),
    ("imfit_GetFitStatisticAndGradient", _I, [_P, _DP, _DP, _DP]),
    ("imfit_GetFitStatisticFast", _I, [_P, _DP, _DP]),
    ("imfit_BatchFitStatisticAndGradient", _I, [_P, _I, _DP, _DP, _DP]),
    ("imfit_BatchFitStatisticAndGradientDevice", _I, [_P, _I, _P, _P, _P]),
    ("imfit_GetJtWJ", _I, [_P, _DP, _DP, _DP, _DP]),
    ("imfit_GetJacobian", _I, [_P, _DP, _DP, _DP]),
    ("imfit_BatchJtWJDevice", _I, [_P, _I, _P, _P, _P, _P]),
    ("imfit_FitLM", _I, [_P, _DP, ctypes.POINTER(_I), _DP, _DP, _D, _I, _DP, ctypes.POINTER(_I),
                         ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("imfit_FitLMBatch", _I, [_P, _I, _DP, ctypes.POINTER(_I), _DP, _DP, _D, _I, _DP, ctypes.POINTER(_I),
                              ctypes.POINTER(_I)]),
    ("imfit_GetLMBatchStats", _I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_L), _DP, _DP]),
    ("imfit_BootstrapFitBatch", _I, [_P, _I, _DP, ctypes.POINTER(_I), _DP, _DP, _D, _I, _DP, _DP,
                                     ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("imfit_SetupImageStack", _I, [_P, _I, _I, _I, _DP, _DP, _DP, _I, _I]),
    ("imfit_SetupCutouts", _I, [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), _DP, _DP, ctypes.POINTER(_I),
                                ctypes.POINTER(_I), _DP]),
    ("imfit_CutoutsJtWJ", _I, [_P, _I, ctypes.POINTER(_I), _DP, _DP, _DP, _DP]),
    ("imfit_MinimizeNormalEquations", _I, [_I, _DP, ctypes.POINTER(_I), _DP, _DP, _D, _I, NORMAL_EQ_FN, _P, _DP,
                                           ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("imfit_MinimizeNormalEquationsBatch", _I, [_I, _I, _DP, ctypes.POINTER(_I), _DP, _DP, _D, _I,
                                                NORMAL_EQ_BATCH_FN, _P, _DP, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("imfit_GetTuning", _I, [_P] + [ctypes.POINTER(_I)] * 6),
    ("imfit_SetFunctionOptionalParam", _I, [_P, _I, ctypes.c_char_p, ctypes.c_char_p]),
    ("imfit_Synchronize", _I, [_P]),
    ("imfit_GetStream", _I, [_P, ctypes.POINTER(_P)]),
    ("imfit_SetUseGraphs", _I, [_P, _I]),
    ("imfit_GetFastModelImageVector", _I, [_P, _DP, _DP]),
    ("imfit_SetKernelTiming", _I, [_P, _I]),
    ("imfit_GetKernelTimes", _I, [_P, _DP, ctypes.c_char_p, _I, _I]),
    ("imfit_SetKernelTimingStage", _I, [_P, ctypes.c_char_p]),
    ("imfit_SetConcurrentRegions", _I, [_P, _I]),
    ("imfit_SetAutotune", _I, [_P, _I]),
    ("imfit_GetLaunchShape", _I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("imfit_SetLaunchShape", _I, [_P, _I, _I, _I, _I]),
    ("imfit_SetFFTPlan", _I, [_P, _I, _I]),
    ("imfit_GetFFTPlan", _I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("imfit_MeasureSfuRate", _I, [_I, _DP]),
    ("imfit_HostAlloc", _I, [ctypes.c_ulong, ctypes.POINTER(_P)]),
    ("imfit_HostFree", _I, [_P]),
    ("imfit_ChiSquaredDeviceNoAlloc", _I, [_P, _P, _P, _L, _P, _P]),
]


class ImfitError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"imfit_gb300 error {code}: {msg}")
        self.code = code


def library_path():
    return _build.LIB


def load_library(build_if_missing=True):
    """Load the CUDA library (building it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} missing: run python -m imfit_gb300.build")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, res, args in _SIGS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return [s[0] for s in _SIGS]


def radix_schedule(n, order=0):
    """The radices of an n-point transform in the library's order `order`
    (0: 8, 9, 4, 2 then 3, 5, 7; 1: 7, 5, 9, 3 then 8, 4, 2; 2: 4, 2, 9 then
    3, 5, 7)."""
    seq = {0: (8, 9, 4, 2, 3, 5, 7), 1: (7, 5, 9, 3, 8, 4, 2), 2: (4, 2, 9, 3, 5, 7)}[order]
    out = []
    for p in seq:
        while n % p == 0:
            out.append(p)
            n //= p
    return out if n == 1 else None


def measure_sfu_rate(device=0):
    """Measured MUFU throughput of the device (transcendental ops/s)."""
    lib = load_library()
    v = ctypes.c_double()
    st = lib.imfit_MeasureSfuRate(device, ctypes.byref(v))
    if st != 0:
        raise ImfitError(st, "imfit_MeasureSfuRate failed")
    return v.value


def minimize_normal_equations(fun, x0, fixed=None, lower=None, upper=None, ftol=1e-8, max_iter=0):
    """The library's Levenberg-Marquardt driver (imfit_MinimizeNormalEquations)
    on a caller's normal equations: fun(x) -> (S, A, b) with S = sum dev^2,
    A = J^T J, b = J^T dev.  Limits are used where lower < upper.  Returns a
    dict with the parameters, S there, iterations, evaluations and the status
    (1 ftol, 2 xtol, 3 no step, 4 stalled, 5 iteration limit)."""
    lib = load_library()
    x = np.array(x0, dtype=float)
    n = x.size
    fx = (_I * n)(*([0] * n if fixed is None else [int(v) for v in fixed]))
    lo = _f64(lower) if lower is not None else None
    hi = _f64(upper) if upper is not None else None
    errors = []

    @NORMAL_EQ_FN
    def cb(xp, sp, ap, bp, user):
        try:
            s, A, b = fun(np.ctypeslib.as_array(xp, shape=(n,)).copy())
            sp[0] = s
            np.ctypeslib.as_array(ap, shape=(n * n,))[:] = np.asarray(A, dtype=float).ravel()
            np.ctypeslib.as_array(bp, shape=(n,))[:] = b
            return 0
        except Exception as e:  # reported after the driver returns
            errors.append(e)
            return -1

    stat = _D()
    it, nev, st = _I(), _I(), _I()
    rc = lib.imfit_MinimizeNormalEquations(n, _dp(x), fx, _dp(lo) if lo is not None else None,
                                           _dp(hi) if hi is not None else None, ftol, int(max_iter), cb, None,
                                           ctypes.byref(stat), ctypes.byref(it), ctypes.byref(nev), ctypes.byref(st))
    if errors:
        raise errors[0]
    if rc != 0:
        raise RuntimeError(lib.imfit_LastError(None).decode())
    return dict(params=x, statistic=stat.value, niter=it.value, nev=nev.value, status=st.value)


def minimize_normal_equations_batch(fun, X0, fixed=None, lower=None, upper=None, ftol=1e-8, max_iter=0):
    """imfit_MinimizeNormalEquationsBatch: B independent problems stepped in
    lockstep.  fun(X, active) -> (S, A, b) for the trial vectors X (B x n) and
    the mask of running problems: S (B), A (B x n x n), b (B x n); rows of
    inactive problems are ignored.  lower / upper: (B x n) or None.  Returns a
    dict of arrays: params, statistic, niter, status."""
    lib = load_library()
    X = np.array(X0, dtype=float)
    B, n = X.shape
    fx = (_I * n)(*([0] * n if fixed is None else [int(v) for v in fixed]))
    lo = _f64(np.asarray(lower, dtype=float).reshape(B, n)) if lower is not None else None
    hi = _f64(np.asarray(upper, dtype=float).reshape(B, n)) if upper is not None else None
    errors = []

    @NORMAL_EQ_BATCH_FN
    def cb(bb, xp, ap_, sp, ap, bp, user):
        try:
            act = np.ctypeslib.as_array(ap_, shape=(bb,)).astype(bool)
            S, A, b = fun(np.ctypeslib.as_array(xp, shape=(bb, n)).copy(), act)
            s_out = np.ctypeslib.as_array(sp, shape=(bb,))
            a_out = np.ctypeslib.as_array(ap, shape=(bb, n * n))
            b_out = np.ctypeslib.as_array(bp, shape=(bb, n))
            s_out[act] = np.asarray(S, dtype=float)[act]
            a_out[act] = np.asarray(A, dtype=float).reshape(bb, n * n)[act]
            b_out[act] = np.asarray(b, dtype=float).reshape(bb, n)[act]
            return 0
        except Exception as e:  # reported after the driver returns
            errors.append(e)
            return -1

    stats = np.zeros(B)
    it = (_I * B)()
    st = (_I * B)()
    rc = lib.imfit_MinimizeNormalEquationsBatch(B, n, _dp(X), fx, _dp(lo) if lo is not None else None,
                                                _dp(hi) if hi is not None else None, ftol, int(max_iter), cb, None,
                                                _dp(stats), it, st)
    if errors:
        raise errors[0]
    if rc != 0:
        raise RuntimeError(lib.imfit_LastError(None).decode())
    return dict(params=X, statistic=stats, niter=np.array(it[:]), status=np.array(st[:]))


def _dp(a):
    return a.ctypes.data_as(_DP)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class ModelObject:
    """One model + data image on one GPU (the reference's ModelObject)."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = _P()
        st = self.lib.imfit_ModelObject_new(device, ctypes.byref(h))
        if st != 0:
            raise ImfitError(st, self.lib.imfit_LastError(None).decode())
        self.h = h
        self.ncols = self.nrows = 0
        self._funcs = []
        self._set_starts = []

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.imfit_ModelObject_delete(h)
            self.h = None

    def _ck(self, st, allow_negative=False):
        if st != 0 and not allow_negative:
            raise ImfitError(st, self.lib.imfit_LastError(self.h).decode())
        return st

    @property
    def last_error(self):
        return self.lib.imfit_LastError(self.h).decode()

    # --- functions ---
    def add_function(self, name, new_set=False, subsampling=True, optional=None):
        """optional: {name: value} optional parameters (e.g. {"method": "lanczos2"}
        for PointSource)."""
        self._ck(self.lib.imfit_AddFunction(self.h, name.encode()))
        idx = len(self._funcs)
        self._funcs.append(name)
        if new_set or idx == 0:
            self._set_starts.append(idx)
        self._ck(self.lib.imfit_SetSubsampling(self.h, idx, int(subsampling)))
        for k, v in (optional or {}).items():
            self._ck(self.lib.imfit_SetFunctionOptionalParam(self.h, idx, str(k).encode(), str(v).encode()))

    def set_subsampling(self, index, flag):
        self._ck(self.lib.imfit_SetSubsampling(self.h, index, int(flag)))

    def define_function_sets(self, starts):
        arr = (ctypes.c_int * len(starts))(*starts)
        self._ck(self.lib.imfit_DefineFunctionSets(self.h, arr, len(starts)))

    def finish_functions(self):
        self.define_function_sets(self._set_starts)
        self._ck(self.lib.imfit_PopulateParameterNames(self.h))

    def parameter_names(self):
        buf = ctypes.create_string_buffer(64)
        out = []
        for i in range(self.n_params):
            self.lib.imfit_GetParameterName(self.h, i, buf, 64)
            out.append(buf.value.decode())
        return out

    # --- image setup ---
    def add_psf(self, psf, normalize=True):
        psf = _f64(psf)
        return self._ck(self.lib.imfit_AddPSFVector(self.h, psf.size, psf.shape[1], psf.shape[0], _dp(psf),
                                                    int(normalize)))

    def setup_model_image(self, ncols, nrows):
        self.ncols, self.nrows = ncols, nrows
        return self._ck(self.lib.imfit_SetupModelImage(self.h, ncols, nrows))

    def add_image_data(self, img):
        img = _f64(img)
        self.nrows, self.ncols = img.shape
        return self._ck(self.lib.imfit_AddImageDataVector(self.h, _dp(img), img.shape[1], img.shape[0]))

    def add_image_characteristics(self, gain=1.0, read_noise=0.0, exp_time=1.0, n_combined=1,
                                  original_sky=0.0):
        return self._ck(self.lib.imfit_AddImageCharacteristics(self.h, gain, read_noise, exp_time,
                                                               n_combined, original_sky))

    def add_oversampled_psf(self, psf, scale, region, normalize=True):
        psf = _f64(psf)
        x1, x2, y1, y2 = region
        return self._ck(self.lib.imfit_AddOversampledPsfInfo(self.h, _dp(psf), psf.shape[1], psf.shape[0],
                                                             scale, x1, x2, y1, y2, int(normalize)))

    def add_error_vector(self, err, input_type=WEIGHTS_ARE_SIGMAS):
        err = _f64(err)
        return self._ck(self.lib.imfit_AddErrorVector(self.h, err.size, err.shape[1], err.shape[0], _dp(err),
                                                      input_type))

    def add_mask_vector(self, mask, input_type=MASK_ZERO_IS_GOOD):
        mask = _f64(mask)
        return self._ck(self.lib.imfit_AddMaskVector(self.h, mask.size, mask.shape[1], mask.shape[0],
                                                     _dp(mask), input_type))

    def use_cash(self):
        return self._ck(self.lib.imfit_UseCashStatistic(self.h))

    def use_pmlr(self):
        return self._ck(self.lib.imfit_UsePoissonMLR(self.h))

    def use_model_errors(self):
        return self._ck(self.lib.imfit_UseModelErrors(self.h))

    def final_setup(self):
        """Returns FinalSetupForFitting's status (0, -1, -2, -3) like the reference."""
        return self.lib.imfit_FinalSetupForFitting(self.h)

    # --- queries ---
    @property
    def n_params(self):
        return self.lib.imfit_GetNParams(self.h)

    @property
    def n_data(self):
        return self.lib.imfit_GetNDataValues(self.h)

    @property
    def n_valid(self):
        return self.lib.imfit_GetNValidPixels(self.h)

    def which_statistic(self, verbose=True):
        return self.lib.imfit_WhichFitStatistic(self.h, int(verbose))

    def model_size(self):
        a, b = _I(), _I()
        self.lib.imfit_GetModelImageSize(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    # --- plain FP64 path ---
    def create_model_image(self, params):
        p = _f64(params)
        self._ck(self.lib.imfit_CreateModelImage(self.h, _dp(p)))

    def get_model_image(self):
        out = np.empty((self.nrows, self.ncols))
        self._ck(self.lib.imfit_GetModelImageVector(self.h, _dp(out)))
        return out

    def get_expanded_model_image(self):
        nc, nr = self.model_size()
        out = np.empty((nr, nc))
        self._ck(self.lib.imfit_GetExpandedModelImageVector(self.h, _dp(out)))
        return out

    def get_residual_image(self):
        out = np.empty((self.nrows, self.ncols))
        self._ck(self.lib.imfit_GetResidualImageVector(self.h, _dp(out)))
        return out

    def get_weights(self):
        out = np.empty((self.nrows, self.ncols))
        self._ck(self.lib.imfit_GetWeightImageVector(self.h, _dp(out)))
        return out

    def get_data(self):
        out = np.empty((self.nrows, self.ncols))
        self._ck(self.lib.imfit_GetDataVector(self.h, _dp(out)))
        return out

    def compute_deviates(self, params, n=None):
        p = _f64(params)
        out = np.empty(n if n is not None else self.n_data)
        self._ck(self.lib.imfit_ComputeDeviates(self.h, _dp(out), _dp(p)))
        return out

    def get_fit_statistic(self, params):
        p = _f64(params)
        s = _D()
        self._ck(self.lib.imfit_GetFitStatistic(self.h, _dp(p), ctypes.byref(s)))
        return s.value

    def get_single_function_image(self, params, function_index):
        p = _f64(params)
        out = np.empty((self.nrows, self.ncols))
        self._ck(self.lib.imfit_GetSingleFunctionImage(self.h, _dp(p), int(function_index), _dp(out)))
        return out

    def find_total_fluxes(self, params, xsize, ysize):
        """(total, per-function fluxes) as ModelObject::FindTotalFluxes."""
        p = _f64(params)
        nf = self.lib.imfit_GetNFunctions(self.h)
        ind = np.empty(nf)
        tot = _D()
        self._ck(self.lib.imfit_FindTotalFluxes(self.h, _dp(p), int(xsize), int(ysize), _dp(ind),
                                                ctypes.byref(tot)))
        return tot.value, ind

    def use_bootstrap(self, seed):
        return self._ck(self.lib.imfit_UseBootstrap(self.h, seed))

    def make_bootstrap_sample(self):
        return self._ck(self.lib.imfit_MakeBootstrapSample(self.h))

    # --- gradients ---
    def statistic_and_gradient_fd(self, params):
        p = _f64(params)
        s = _D()
        g = np.empty(self.n_params)
        self._ck(self.lib.imfit_GetFitStatisticAndGradientFD(self.h, _dp(p), ctypes.byref(s), _dp(g)))
        return s.value, g

    def statistic_and_gradient(self, params):
        p = _f64(params)
        s = _D()
        g = np.empty(self.n_params)
        self._ck(self.lib.imfit_GetFitStatisticAndGradient(self.h, _dp(p), ctypes.byref(s), _dp(g)))
        return s.value, g

    def fit_statistic_fast(self, params):
        p = _f64(params)
        s = _D()
        self._ck(self.lib.imfit_GetFitStatisticFast(self.h, _dp(p), ctypes.byref(s)))
        return s.value

    def batch_statistic_and_gradient(self, params, want_grad=True):
        p = _f64(np.atleast_2d(params))
        B = p.shape[0]
        s = np.empty(B)
        g = np.empty((B, self.n_params)) if want_grad else None
        self._ck(self.lib.imfit_BatchFitStatisticAndGradient(self.h, B, _dp(p), _dp(s),
                                                             _dp(g) if want_grad else None))
        return (s, g) if want_grad else s

    def batch_device(self, n_batch, d_params, d_stats, d_grads):
        """Device-pointer batch call (ints: raw device addresses); enqueues only."""
        return self._ck(self.lib.imfit_BatchFitStatisticAndGradientDevice(self.h, n_batch, d_params, d_stats,
                                                                          d_grads))

    def jtwj(self, params):
        """(statistic, J^T J, J^T dev) of the deviates by the forward-mode fast path."""
        p = _f64(params)
        n = self.n_params
        s = _D()
        a = np.empty((n, n))
        b = np.empty(n)
        self._ck(self.lib.imfit_GetJtWJ(self.h, _dp(p), ctypes.byref(s), _dp(a), _dp(b)))
        return s.value, a, b

    def jacobian(self, params):
        """(J, deviates): J[j] = d dev / d param_j over the data pixels (analytic, FP32-evaluated)."""
        p = _f64(params)
        n = self.n_params
        nd = self.nrows * self.ncols
        J = np.empty((n, nd))
        dev = np.empty(nd)
        self._ck(self.lib.imfit_GetJacobian(self.h, _dp(p), _dp(J), _dp(dev)))
        return J, dev

    def batch_jtwj_device(self, n_batch, d_params, d_stats, d_jtj, d_jtdev):
        """Device-pointer batched JtWJ (ints: raw device addresses); enqueues only."""
        return self._ck(self.lib.imfit_BatchJtWJDevice(self.h, n_batch, d_params, d_stats, d_jtj, d_jtdev))

    def fit_lm(self, params, fixed=None, lower=None, upper=None, ftol=1e-8, max_iter=0):
        """Levenberg-Marquardt fit on the normal equations (FP64 host solve,
        JtWJ from the GPU).  Returns a dict with the fitted parameters, the
        fast-path statistic, iteration and evaluation counts and the status."""
        p = _f64(params).copy()
        n = p.size
        fx = (_I * n)(*([0] * n if fixed is None else [int(v) for v in fixed]))
        lo = _f64(lower) if lower is not None else None
        hi = _f64(upper) if upper is not None else None
        s, it, ne, st = _D(), _I(), _I(), _I()
        self._ck(self.lib.imfit_FitLM(self.h, _dp(p), fx, _dp(lo) if lo is not None else None,
                                      _dp(hi) if hi is not None else None, ftol, int(max_iter),
                                      ctypes.byref(s), ctypes.byref(it), ctypes.byref(ne), ctypes.byref(st)))
        return dict(params=p, statistic=s.value, niter=it.value, nev=ne.value, status=st.value)

    def fit_lm_batch(self, params, fixed=None, lower=None, upper=None, ftol=1e-8, max_iter=0):
        """Lockstep Levenberg-Marquardt on the rows of params (B x nParams)."""
        P = _f64(np.atleast_2d(params)).copy()
        B, n = P.shape
        fx = (_I * n)(*([0] * n if fixed is None else [int(v) for v in fixed]))
        lo = _f64(np.broadcast_to(lower, P.shape)).copy() if lower is not None else None
        hi = _f64(np.broadcast_to(upper, P.shape)).copy() if upper is not None else None
        S = np.empty(B)
        it = (_I * B)()
        st = (_I * B)()
        self._ck(self.lib.imfit_FitLMBatch(self.h, B, _dp(P), fx, _dp(lo) if lo is not None else None,
                                           _dp(hi) if hi is not None else None, ftol, int(max_iter), _dp(S),
                                           it, st))
        return dict(params=P, statistic=S, niter=np.array(it[:]), status=np.array(st[:]))

    def lm_batch_stats(self):
        """Timing of the last fit_lm_batch: rounds, problem evaluations, seconds
        in the J^T W J evaluations and in the whole call."""
        r, ev, te, tt = _I(), _L(), ctypes.c_double(), ctypes.c_double()
        self._ck(self.lib.imfit_GetLMBatchStats(self.h, ctypes.byref(r), ctypes.byref(ev), ctypes.byref(te),
                                                ctypes.byref(tt)))
        return dict(rounds=r.value, evaluations=ev.value, eval_s=te.value, total_s=tt.value)

    def bootstrap_fit_batch(self, n_samples, bestfit, fixed=None, lower=None, upper=None, ftol=1e-8, max_iter=0):
        """The next n_samples bootstrap samples (after use_bootstrap(seed)), all
        refitted at once from bestfit; dict of params (n_samples x nParams),
        statistic, niter, status (> 0: success)."""
        x = _f64(bestfit)
        n = x.size
        fx = (_I * n)(*([0] * n if fixed is None else [int(v) for v in fixed]))
        lo = _f64(lower) if lower is not None else None
        hi = _f64(upper) if upper is not None else None
        P = np.empty((n_samples, n))
        S = np.empty(n_samples)
        it = (_I * n_samples)()
        st = (_I * n_samples)()
        self._ck(self.lib.imfit_BootstrapFitBatch(self.h, int(n_samples), _dp(x), fx,
                                                  _dp(lo) if lo is not None else None,
                                                  _dp(hi) if hi is not None else None, ftol, int(max_iter),
                                                  _dp(P), _dp(S), it, st))
        return dict(params=P, statistic=S, niter=np.array(it[:]), status=np.array(st[:]))

    def setup_image_stack(self, images, sigmas, psfs):
        """images, sigmas: (n, rows, cols); psfs: (n, prows, pcols)."""
        im = _f64(images)
        sg = _f64(np.broadcast_to(sigmas, im.shape)).copy()
        ps = _f64(psfs)
        n, nr, nc = im.shape
        return self._ck(self.lib.imfit_SetupImageStack(self.h, n, nc, nr, _dp(im), _dp(sg), _dp(ps),
                                                       ps.shape[2], ps.shape[1]))

    def setup_cutouts(self, images, sigmas, psfs):
        """A cutout set: lists of images (rows x cols, each its own size), their
        sigma images (or scalars) and their odd-sized PSFs."""
        n = len(images)
        ims = [_f64(im) for im in images]
        sgs = [_f64(np.broadcast_to(sg, im.shape)) for im, sg in zip(ims, sigmas)]
        pss = [_f64(p) for p in psfs]
        IA = ctypes.c_int * n
        cols = IA(*[im.shape[1] for im in ims])
        rows = IA(*[im.shape[0] for im in ims])
        pc = IA(*[p.shape[1] for p in pss])
        pr = IA(*[p.shape[0] for p in pss])
        pix = np.concatenate([im.ravel() for im in ims])
        sig = np.concatenate([sg.ravel() for sg in sgs])
        psf = np.concatenate([p.ravel() for p in pss])
        self._n_cutouts = n
        return self._ck(self.lib.imfit_SetupCutouts(self.h, n, cols, rows, _dp(pix), _dp(sig), pc, pr, _dp(psf)))

    def cutouts_jtwj(self, cutouts, params):
        """(statistics, J^T J, J^T dev) of the given cutouts at params (K x nParams)."""
        idx = np.ascontiguousarray(cutouts, dtype=np.int32)
        P = _f64(np.atleast_2d(params))
        K, n = P.shape[0], self.n_params
        S = np.empty(K)
        A = np.empty((K, n, n))
        B = np.empty((K, n))
        self._ck(self.lib.imfit_CutoutsJtWJ(self.h, K, idx.ctypes.data_as(ctypes.POINTER(_I)), _dp(P), _dp(S),
                                            _dp(A), _dp(B)))
        return S, A, B

    def synchronize(self):
        return self._ck(self.lib.imfit_Synchronize(self.h))

    def stream(self):
        """Raw cudaStream_t (int) of this handle."""
        s = _P()
        self._ck(self.lib.imfit_GetStream(self.h, ctypes.byref(s)))
        return s.value

    def set_use_graphs(self, flag):
        return self._ck(self.lib.imfit_SetUseGraphs(self.h, int(flag)))

    def set_kernel_timing(self, flag):
        return self._ck(self.lib.imfit_SetKernelTiming(self.h, int(flag)))

    def set_kernel_timing_stage(self, name=None):
        return self._ck(self.lib.imfit_SetKernelTimingStage(self.h, name.encode() if name else None))

    def set_concurrent_regions(self, flag):
        return self._ck(self.lib.imfit_SetConcurrentRegions(self.h, int(flag)))

    def set_autotune(self, flag):
        return self._ck(self.lib.imfit_SetAutotune(self.h, int(flag)))

    def set_launch_shape(self, rows_per_cta=-1, row_threads=256, cols_per_cta=0, col_threads=0):
        """Pin the fast path's launch shape (rows_per_cta < 0: autotune again)."""
        return self._ck(self.lib.imfit_SetLaunchShape(self.h, rows_per_cta, row_threads, cols_per_cta, col_threads))

    def set_fft_plan(self, candidate=-1, radix_order=0):
        """Pin the fast path's padded-length candidate (0..2) and radix order
        (0..2), or return to autotuning (candidate < 0)."""
        self._ck(self.lib.imfit_SetFFTPlan(self.h, candidate, radix_order))

    def fft_plan(self):
        """(Lx, Ly, radix order) of the fast path's main window."""
        lx, ly, v = _I(), _I(), _I()
        self._ck(self.lib.imfit_GetFFTPlan(self.h, ctypes.byref(lx), ctypes.byref(ly), ctypes.byref(v)))
        return lx.value, ly.value, v.value

    def launch_shape(self):
        """Launch shape and FFT plan the fast path uses (after its first call)."""
        a, b, c = _I(), _I(), _I()
        self._ck(self.lib.imfit_GetLaunchShape(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        lx, ly, order = self.fft_plan()
        t = [_I() for _ in range(6)]
        self._ck(self.lib.imfit_GetTuning(self.h, *[ctypes.byref(v) for v in t]))
        return {"rows_per_cta": a.value, "row_threads": b.value, "cols_per_cta": c.value,
                "col_threads": t[5].value, "Lx": lx, "Ly": ly, "fft_candidate": t[0].value,
                "radix_order": order, "row_radices": radix_schedule(lx // 2, order) if lx else [],
                "col_radices": radix_schedule(ly, order) if ly else [],
                "pin": {"fft_plan": f"{t[0].value},{t[1].value}",
                        "launch_shape": f"{t[2].value},{t[3].value},{t[4].value},{t[5].value}"}}

    def kernel_times(self):
        """[(kernel name, ms)] of the most recent fast evaluation."""
        ms = np.zeros(64)
        buf = ctypes.create_string_buffer(4096)
        n = self.lib.imfit_GetKernelTimes(self.h, _dp(ms), buf, 4096, 64)
        if n < 0:
            raise ImfitError(n, self.last_error)
        names = buf.value.decode().split(",") if n else []
        return list(zip(names, ms[:n].tolist()))

    def get_fast_model_image(self, params):
        p = _f64(params)
        out = np.empty((self.nrows, self.ncols))
        self._ck(self.lib.imfit_GetFastModelImageVector(self.h, _dp(p), _dp(out)))
        return out
