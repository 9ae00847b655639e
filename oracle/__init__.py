"""CPU oracle for the model-image / fit-statistic path (TEST INFRASTRUCTURE ONLY).

Two CPU implementations sit behind one Python interface:

* ``OracleModel`` -- the project's C restatement of the reference algorithm
  (``oracle/imfit_oracle.c``), built by ``make -C oracle restatement`` into
  ``oracle/_build/liboracle.so``.  It builds anywhere from this repository.
* ``RefModel`` -- the reference's OWN hot-path sources compiled unmodified
  against the project's FFTW/GSL shims (``make -C oracle ref`` ->
  ``oracle/_ref/libimfit_ref.so``).  It exists only where the reference
  checkout is present; it pins the restatement.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this package; the product library never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RESTATEMENT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libimfit_ref.so")


def _reference_dir():
    """The reference checkout: IMFIT_REFERENCE_DIR, else the build recipe's
    default (REFDIR in oracle/Makefile)."""
    d = os.environ.get("IMFIT_REFERENCE_DIR")
    if d:
        return d
    try:
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-refdir"],
                           capture_output=True, text=True, timeout=30)
        return r.stdout.strip() if r.returncode == 0 else ""
    except (OSError, subprocess.SubprocessError):
        return ""


REFERENCE_DIR = _reference_dir()


def reference_checkout():
    """True where the reference's sources are present (never on a host that
    only received this repository)."""
    return bool(REFERENCE_DIR) and os.path.isdir(os.path.join(REFERENCE_DIR, "core"))

# input-type codes (core/definitions.h)
WEIGHTS_ARE_SIGMAS, WEIGHTS_ARE_VARIANCES, WEIGHTS_ARE_WEIGHTS = 100, 110, 120
MASK_ZERO_IS_GOOD, MASK_ZERO_IS_BAD = 10, 20

_libs = {}


def build_restatement():
    subprocess.run(["make", "-s", "-C", HERE, "restatement"], check=True)


def build_reference():
    """Compile the reference's own sources (needs the reference checkout)."""
    if not reference_checkout():
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFDIR={REFERENCE_DIR}"], check=True)
    return True


def reference_available():
    return os.path.exists(REF_SO)


_D = ctypes.c_double
_I = ctypes.c_int
_L = ctypes.c_long
_P = ctypes.c_void_p
_DP = ctypes.POINTER(ctypes.c_double)
_S = ctypes.c_char_p


def _bind(lib, prefix):
    sig = {
        "create": (_P, []),
        "destroy": (None, [_P]),
        "set_max_threads": (None, [_P, _I]),
        "add_function": (_I, [_P, _S, _I, _I]),
        "finish_functions": (_I, [_P]),
        "add_psf": (_I, [_P, _I, _I, _DP, _I]),
        "setup_model_image": (_I, [_P, _I, _I]),
        "add_image_data": (_I, [_P, _DP, _I, _I]),
        "add_image_characteristics": (None, [_P, _D, _D, _D, _I, _D]),
        "add_error_vector": (_I, [_P, _DP, _I, _I, _I]),
        "add_mask_vector": (_I, [_P, _DP, _I, _I, _I]),
        "use_cash": (_I, [_P]),
        "use_pmlr": (None, [_P]),
        "use_model_errors": (_I, [_P]),
        "final_setup": (_I, [_P]),
        "n_params": (_I, [_P]),
        "n_data": (_L, [_P]),
        "n_valid": (_L, [_P]),
        "which_statistic": (_I, [_P]),
        "create_model_image": (None, [_P, _DP]),
        "get_model_image": (_I, [_P, _DP]),
        "get_expanded_model_image": (_I, [_P, _DP, _L]),
        "compute_deviates": (None, [_P, _DP, _DP]),
        "get_fit_statistic": (_D, [_P, _DP]),
        "get_weights": (_I, [_P, _DP]),
        "get_mask": (_I, [_P, _DP]),
        "get_data": (_I, [_P, _DP]),
        "function_value": (_D, [_S, _DP, _D, _D, _D, _D, _I]),
        "function_total_flux": (_D, [_S, _DP]),
        "use_bootstrap": (_I, [_P, ctypes.c_ulong]),
        "make_bootstrap_sample": (_I, [_P]),
        "fd_jacobian": (_I, [_P, _DP, _DP]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, f"{prefix}_{name}")
        fn.restype = res
        fn.argtypes = args
    if prefix == "orc":
        lib.orc_add_oversampled_psf.restype = _I
        lib.orc_add_oversampled_psf.argtypes = [_P, _I, _I, _DP, _I, _I, _I, _I, _I, _I]
        lib.orc_model_size.argtypes = [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)]
        lib.orc_fft_size.argtypes = [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)]
        lib.orc_get_internal_weights.argtypes = [_P, _DP]
        lib.orc_get_extra_cash_terms.argtypes = [_P, _DP]
        lib.orc_get_bootstrap_indices.restype = _L
        lib.orc_get_bootstrap_indices.argtypes = [_P, ctypes.POINTER(ctypes.c_long)]
        lib.orc_function_qags_nsub.restype = _I
        lib.orc_function_qags_nsub.argtypes = [_S, _DP, _D, _D, _D, _D]
        lib.orc_function_nparams.restype = _I
        lib.orc_function_nparams.argtypes = [_S]
        lib.orc_set_fft_smooth.restype = None
        lib.orc_set_fft_smooth.argtypes = [_P, _I]
        lib.orc_set_point_source_method.restype = _I
        lib.orc_set_point_source_method.argtypes = [_P, _I, _I]
        lib.orc_get_single_function_image.restype = _I
        lib.orc_get_single_function_image.argtypes = [_P, _DP, _I, _DP]
        lib.orc_interpolate_psf.restype = _I
        lib.orc_interpolate_psf.argtypes = [_I, _DP, _I, _I, _DP, _DP, _L, _DP]
        lib.orc_lanczos.restype = _D
        lib.orc_lanczos.argtypes = [_D, _I]
    else:
        lib.ref_add_oversampled_psf.restype = _I
        lib.ref_add_oversampled_psf.argtypes = [_P, _I, _I, _DP, _I, _S, _I]
        lib.ref_lm_fit.restype = _I
        lib.ref_lm_fit.argtypes = [_P, _DP, ctypes.POINTER(_I), _DP, _DP, _D, _I,
                                   ctypes.POINTER(_I), ctypes.POINTER(_I), _DP, _DP]


def _load(which):
    if which in _libs:
        return _libs[which]
    if which == "orc":
        if not os.path.exists(RESTATEMENT_SO):
            build_restatement()
        lib = ctypes.CDLL(RESTATEMENT_SO)
    else:
        if not os.path.exists(REF_SO) and not build_reference():
            raise RuntimeError("reference sources not available; cannot build oracle/_ref")
        lib = ctypes.CDLL(REF_SO)
    _bind(lib, which)
    _libs[which] = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(_DP)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class _CModel:
    """Common ModelObject-shaped interface over either CPU library."""

    prefix = None

    def __init__(self):
        self.lib = _load(self.prefix)
        self._fn = lambda n: getattr(self.lib, f"{self.prefix}_{n}")
        self.h = self._fn("create")()
        self.ncols = self.nrows = 0
        self._keep = []

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self._fn("destroy")(h)
            self.h = None

    # --- setup, in the reference's required order ---
    def set_max_threads(self, n):
        self._fn("set_max_threads")(self.h, int(n))

    def add_function(self, name, new_set=False, subsampling=True):
        st = self._fn("add_function")(self.h, name.encode(), int(new_set), int(subsampling))
        if st != 0:
            raise ValueError(f"unknown function {name}")

    def finish_functions(self):
        return self._fn("finish_functions")(self.h)

    def add_psf(self, psf, normalize=True):
        psf = _f64(psf)
        return self._fn("add_psf")(self.h, psf.shape[1], psf.shape[0], _dp(psf), int(normalize))

    def setup_model_image(self, ncols, nrows):
        self.ncols, self.nrows = ncols, nrows
        return self._fn("setup_model_image")(self.h, ncols, nrows)

    def add_image_data(self, img):
        img = _f64(img)
        self.nrows, self.ncols = img.shape
        return self._fn("add_image_data")(self.h, _dp(img), img.shape[1], img.shape[0])

    def add_image_characteristics(self, gain=1.0, read_noise=0.0, exp_time=1.0, n_combined=1,
                                  original_sky=0.0):
        self._fn("add_image_characteristics")(self.h, gain, read_noise, exp_time, n_combined,
                                              original_sky)

    def add_error_vector(self, err, input_type=WEIGHTS_ARE_SIGMAS):
        err = _f64(err)
        return self._fn("add_error_vector")(self.h, _dp(err), err.shape[1], err.shape[0], input_type)

    def add_mask_vector(self, mask, input_type=MASK_ZERO_IS_GOOD):
        mask = _f64(mask)
        return self._fn("add_mask_vector")(self.h, _dp(mask), mask.shape[1], mask.shape[0], input_type)

    def use_cash(self):
        return self._fn("use_cash")(self.h)

    def use_pmlr(self):
        self._fn("use_pmlr")(self.h)

    def use_model_errors(self):
        return self._fn("use_model_errors")(self.h)

    def final_setup(self):
        return self._fn("final_setup")(self.h)

    # --- queries ---
    @property
    def n_params(self):
        return self._fn("n_params")(self.h)

    @property
    def n_data(self):
        return self._fn("n_data")(self.h)

    @property
    def n_valid(self):
        return self._fn("n_valid")(self.h)

    def which_statistic(self):
        return self._fn("which_statistic")(self.h)

    # --- evaluation ---
    def create_model_image(self, params):
        p = _f64(params)
        self._fn("create_model_image")(self.h, _dp(p))

    def get_model_image(self):
        out = np.empty((self.nrows, self.ncols))
        if self._fn("get_model_image")(self.h, _dp(out)) != 0:
            raise RuntimeError("model image not computed")
        return out

    def compute_deviates(self, params, n=None):
        p = _f64(params)
        out = np.empty(n if n is not None else self.n_data)
        self._fn("compute_deviates")(self.h, _dp(out), _dp(p))
        return out

    def get_fit_statistic(self, params):
        p = _f64(params)
        return self._fn("get_fit_statistic")(self.h, _dp(p))

    def get_weights(self):
        out = np.empty(self.n_data)
        self._fn("get_weights")(self.h, _dp(out))
        return out.reshape(self.nrows, self.ncols)

    def get_mask(self):
        out = np.empty(self.n_data)
        if self._fn("get_mask")(self.h, _dp(out)) != 0:
            return None
        return out.reshape(self.nrows, self.ncols)

    def get_data(self):
        out = np.empty(self.n_data)
        self._fn("get_data")(self.h, _dp(out))
        return out.reshape(self.nrows, self.ncols)

    def use_bootstrap(self, seed):
        return self._fn("use_bootstrap")(self.h, seed)

    def make_bootstrap_sample(self):
        return self._fn("make_bootstrap_sample")(self.h)

    def fd_jacobian(self, params, n_rows=None):
        p = _f64(params)
        m = n_rows if n_rows is not None else self.n_data
        out = np.empty((self.n_params, m))
        self._fn("fd_jacobian")(self.h, _dp(p), _dp(out))
        return out


class OracleModel(_CModel):
    prefix = "orc"

    def set_fft_smooth(self, flag=True):
        self.lib.orc_set_fft_smooth(self.h, int(flag))

    def add_oversampled_psf(self, psf, scale, region, normalize=True):
        psf = _f64(psf)
        x1, x2, y1, y2 = region
        self._keep.append(psf)
        return self.lib.orc_add_oversampled_psf(self.h, psf.shape[1], psf.shape[0], _dp(psf), scale,
                                                x1, x2, y1, y2, int(normalize))

    def model_size(self):
        a, b = _I(), _I()
        self.lib.orc_model_size(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def get_expanded_model_image(self):
        nc, nr = self.model_size()
        out = np.empty((nr, nc))
        self.lib.orc_get_expanded_model_image(self.h, _dp(out), nc * nr)
        return out

    def get_internal_weights(self):
        out = np.empty(self.n_data)
        self.lib.orc_get_internal_weights(self.h, _dp(out))
        return out.reshape(self.nrows, self.ncols)

    def get_extra_cash_terms(self):
        out = np.empty(self.n_data)
        if self.lib.orc_get_extra_cash_terms(self.h, _dp(out)) != 0:
            return None
        return out.reshape(self.nrows, self.ncols)

    def set_point_source_method(self, index, method):
        """method: 'bicubic', 'lanczos2' or 'lanczos3' (PointSource's optional parameter)."""
        return self.lib.orc_set_point_source_method(self.h, int(index), INTERPOLATORS[method.lower()])

    def get_single_function_image(self, params, function_index):
        p = _f64(params)
        out = np.empty((self.nrows, self.ncols))
        st = self.lib.orc_get_single_function_image(self.h, _dp(p), int(function_index), _dp(out))
        if st != 0:
            raise ValueError(f"GetSingleFunctionImage failed ({st})")
        return out

    def get_bootstrap_indices(self):
        out = np.empty(self.n_valid, dtype=np.int64)
        n = self.lib.orc_get_bootstrap_indices(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
        return out[:n] if n >= 0 else None


class RefModel(_CModel):
    prefix = "ref"

    def add_oversampled_psf(self, psf, scale, region, normalize=True):
        psf = _f64(psf)
        x1, x2, y1, y2 = region
        reg = f"[{x1}:{x2},{y1}:{y2}]".encode()
        return self.lib.ref_add_oversampled_psf(self.h, psf.shape[1], psf.shape[0], _dp(psf), scale,
                                                reg, int(normalize))

    def get_expanded_model_image(self, ncols, nrows):
        out = np.empty((nrows, ncols))
        self.lib.ref_get_expanded_model_image(self.h, _dp(out), ncols * nrows)
        return out

    def lm_fit(self, params, fixed=None, lo=None, hi=None, ftol=1e-8, maxiter=200):
        p = _f64(params).copy()
        n = p.size
        fx = (ctypes.c_int * n)(*([0] * n if fixed is None else [int(v) for v in fixed]))
        lo_a = _f64(lo) if lo is not None else None
        hi_a = _f64(hi) if hi is not None else None
        niter, nfev = _I(), _I()
        chi2, chi2i = _D(), _D()
        st = self.lib.ref_lm_fit(self.h, _dp(p), fx, _dp(lo_a) if lo_a is not None else None,
                                 _dp(hi_a) if hi_a is not None else None, ftol, maxiter,
                                 ctypes.byref(niter), ctypes.byref(nfev), ctypes.byref(chi2),
                                 ctypes.byref(chi2i))
        return dict(status=st, params=p, niter=niter.value, nfev=nfev.value, chi2=chi2.value,
                    chi2_init=chi2i.value)


INTERPOLATORS = {"bicubic": 1, "lanczos2": 2, "lanczos3": 3}


def interpolate_psf(kind, psf, dx, dy):
    """PsfInterpolator::GetValue (function_objects/psf_interpolators.cpp) of
    the given kind on psf at offsets (dx, dy) from its centre."""
    lib = _load("orc")
    psf = _f64(psf)
    dx = _f64(np.atleast_1d(dx))
    dy = _f64(np.broadcast_to(dy, dx.shape))
    out = np.empty(dx.shape)
    st = lib.orc_interpolate_psf(INTERPOLATORS[kind], _dp(psf), psf.shape[1], psf.shape[0], _dp(dx), _dp(dy),
                                 dx.size, _dp(out))
    if st != 0:
        raise ValueError(f"PSF interpolator setup failed ({st})")
    return out


def lanczos(x, n):
    return _load("orc").orc_lanczos(float(x), int(n))


def set_los_epsrel(epsrel):
    """Relative tolerance of the oracle restatement's line-of-sight QAGS
    (the reference's 1e-6 by default; <= 0 restores it)."""
    lib = _load("orc")
    lib.orc_set_los_epsrel.restype = None
    lib.orc_set_los_epsrel.argtypes = [_D]
    lib.orc_set_los_epsrel(float(epsrel))


def function_value(name, params, x0, y0, x, y, subsampling=True, which="orc"):
    lib = _load(which)
    p = _f64(params)
    return getattr(lib, f"{which}_function_value")(name.encode(), _dp(p), x0, y0, x, y, int(subsampling))


def function_total_flux(name, params, which="orc"):
    lib = _load(which)
    p = _f64(params)
    return getattr(lib, f"{which}_function_total_flux")(name.encode(), _dp(p))


def qags_nsub(name, params, x0, y0, x, y):
    lib = _load("orc")
    p = _f64(params)
    return lib.orc_function_qags_nsub(name.encode(), _dp(p), x0, y0, x, y)
