"""Simultaneous fits of several images of one object (multimfit).

MultiImageModel restates ModelObjectMultImage (core/model_object_multimage.cpp,
core/param_holder.cpp, core/paramvector_processing.cpp) on top of one GPU
ModelObject per image.  The global parameter vector is

    [PIXEL_SCALE, IMAGE_PA, FLUX_SCALE, X0, Y0] of images 2..N,
    followed by the model's parameters as the reference image sees them,
    followed by the parameters of each image's own (per-image) functions,
    image 1's first (ParamHolder::AssembleParametersForImage,
    core/param_holder.cpp:257-268).

Image i > 0 gets the model with the first function set centred at its own
(X0, Y0), every later set's centre moved by the set's offset from the first,
rotated by IMAGE_PA and scaled by PIXEL_SCALE (CalculateOffset_X0Y0,
paramvector_processing.cpp:80-104), and each function's position angle,
intensity and size parameters turned into that image's by PA - IMAGE_PA,
FLUX_SCALE * I and size / PIXEL_SCALE (the Setup of every function class with
SetImageParameters, function_object.cpp:105-110).  The statistic is the sum of
the images' statistics, the deviates their concatenation.  Gradients and normal
equations chain each image's (fast path) with T_i = d(image parameters) /
d(global parameters); the LM driver is the library's own
(imfit_MinimizeNormalEquations).

Per-image functions (a FUNCTIONS_START section inside an image's block of the
image-info file, core/imageparams_file_parser.cpp:538-649) are appended to
that image's model after the global functions, each section opening new
function sets (core/multimfit_main.cpp:407-420).  Their parameters are that
image's own: copied unchanged into its parameter vector after the global
model's, neither moved by the image's X0/Y0 nor scaled by its description
parameters (ModelObject::SetImageParameters touches global functions only,
core/model_object.cpp:1088-1097).
"""
from dataclasses import dataclass, field

import numpy as np

from . import ModelObject

N_IMAGE_PARAMS = 5
IMAGE_PARAM_NAMES = ["PIXEL_SCALE", "IMAGE_PA", "FLUX_SCALE", "X0", "Y0"]

# per function: index of PA (or None), intensity indices, size indices
# (each class's Setup, e.g. func_sersic.cpp:109-117, func_exp.cpp, func_flatsky.cpp ...)
ADJUST = {
    "Sersic": (0, [3], [4]),
    "Exponential": (0, [2], [3]),
    "FlatSky": (None, [0], []),
    "GaussianRing": (0, [2], [3, 4]),
    "Moffat": (0, [2], [3]),
    "Gaussian": (0, [2], [3]),
    "ExponentialDisk3D": (0, [2], [3, 5]),
    "FerrersBar3D": (0, [3], [4]),
    "PointSource": (None, [0], []),
    "PointSourceRot": (0, [1], []),
    "TiltedSkyPlane": (None, [0], []),  # slopes unscaled (func_tilted-sky-plane.cpp:74-80)
}


@dataclass
class ImageInfo:
    """One IMAGE_START block of an image-info file
    (core/imageparams_file_parser.cpp:51-78)."""
    data: str = None
    error: str = None
    mask: str = None
    psf: str = None
    options: dict = field(default_factory=dict)        # GAIN, READNOISE, ...
    flags: set = field(default_factory=set)            # ERRORS_ARE_*, MASK_ZERO_IS_BAD
    params: dict = field(default_factory=dict)         # PIXEL_SCALE ... Y0 -> (value, lo, hi, fixed)
    local: object = None                               # per-image functions: a config.ModelConfig

    @property
    def local_functions(self):
        return list(self.local.functions) if self.local is not None else []


def parse_image_info(text):
    """Blocks opened by IMAGE_START: file names (DATA, ERROR, MASK, PSF),
    image characteristics, flags, and the image-description parameters with
    optional limits or 'fixed' (same grammar as configuration files).  A
    FUNCTIONS_START line ends the block's own lines; what follows it, up to
    the next IMAGE_START, is a function section of that image's per-image
    functions in configuration-file grammar (X0/Y0 lines opening function
    sets, FUNCTION blocks, limits), read as ParseFunctionSection reads it
    (core/imageparams_file_parser.cpp:531-547, 626-650)."""
    from .config import parse_config
    images = []
    functions_text = None
    raw_lines = text.splitlines()

    def close_functions():
        if functions_text is not None:
            if not any(t.split("#", 1)[0].strip() for t in functions_text):
                raise ValueError("FUNCTIONS_START without functions")
            images[-1].local = parse_config("\n".join(functions_text))

    for k, raw in enumerate(raw_lines, 1):
        line = raw.split("#", 1)[0].strip()
        if not line:
            if functions_text is not None:
                functions_text.append(raw)
            continue
        parts = line.split()
        key = parts[0]
        if key == "IMAGE_START":
            close_functions()
            functions_text = None
            images.append(ImageInfo())
            continue
        if not images:
            raise ValueError(f"line {k}: {key} before the first IMAGE_START")
        if functions_text is not None:
            functions_text.append(raw)
            continue
        if key == "FUNCTIONS_START":
            functions_text = []
            continue
        im = images[-1]
        if key in ("DATA", "ERROR", "MASK", "PSF"):
            setattr(im, key.lower(), parts[1])
        elif key in ("ERRORS_ARE_SIGMAS", "ERRORS_ARE_VARIANCES", "ERRORS_ARE_WEIGHTS", "MASK_ZERO_IS_GOOD",
                     "MASK_ZERO_IS_BAD"):
            im.flags.add(key)
        elif key in IMAGE_PARAM_NAMES:
            v = float(parts[1])
            lo = hi = np.nan
            fixed = False
            if len(parts) > 2:
                if parts[2].lower() == "fixed":
                    fixed = True
                else:
                    lo, hi = (float(x) for x in parts[2].split(","))
            im.params[key] = (v, lo, hi, fixed)
        else:
            im.options[key] = parts[1]
    if not images:
        raise ValueError("no IMAGE_START lines found")
    close_functions()
    return images


class MultiImageModel:
    """ModelObject-like view of several images fitted with one model.

    functions: [(name, starts_new_set)] as for ModelObject.add_function;
    handles: one configured ModelObject per image (functions added, images,
    PSF, errors, mask and statistic set, final_setup done), the reference
    image first."""

    def __init__(self, functions, handles, local_functions=None):
        self.functions = list(functions)
        self.handles = list(handles)
        self.n_images = len(self.handles)
        self.n_image_params = N_IMAGE_PARAMS * (self.n_images - 1)
        self.local_functions = [list(f) for f in (local_functions or [[] for _ in self.handles])]
        if len(self.local_functions) != self.n_images:
            raise ValueError("one list of per-image functions per image")
        for name, _ in self.functions:
            if name not in ADJUST:
                raise ValueError(f"function {name} has no image adjustment rule")
        # parameter layout of the model vector
        self._set_x0, self._blocks, self.n_model = self._layout(self.functions)
        # per-image parameters: X0/Y0 of each per-image set plus the functions'
        # (ModelObject::FinalModelSetup, core/model_object.cpp:323-334)
        self.n_local = []
        for i, funcs in enumerate(self.local_functions):
            if funcs and not funcs[0][1]:
                raise ValueError(f"image {i + 1}: per-image functions must open a function set")
            self.n_local.append(self._layout(funcs)[2])
        for i, h in enumerate(self.handles):
            if h.n_params != self.n_model + self.n_local[i]:
                raise ValueError("function list does not match the handles' parameter count")
        self.local_start = list(np.cumsum([self.n_image_params + self.n_model] + self.n_local[:-1]))
        self.n_params = self.n_image_params + self.n_model + sum(self.n_local)

    @classmethod
    def _layout(cls, functions):
        set_x0, blocks, off = [], [], 0
        for k, (name, new_set) in enumerate(functions):
            if new_set or k == 0:
                set_x0.append(off)
                off += 2
            blocks.append((name, off))
            off += cls._nparams(name)
        return set_x0, blocks, off

    @staticmethod
    def _nparams(name):
        from .config import _NPARAMS
        return _NPARAMS[name]

    # ---------------------------------------------------- parameter transform
    def image_vector(self, params, i):
        """Parameters of image i (ParamHolder::AssembleParametersForImage,
        core/param_holder.cpp:215-270, then each function's Setup scaling)."""
        p = np.asarray(params, dtype=float)
        model = p[self.n_image_params:self.n_image_params + self.n_model].copy()
        if i == 0:
            ps, rot, fs = 1.0, 0.0, 1.0
        else:
            ps, rot, fs, x0i, y0i = p[N_IMAGE_PARAMS * (i - 1):N_IMAGE_PARAMS * i]
            x0r, y0r = model[0], model[1]
            model[0], model[1] = x0i, y0i
            if ps <= 0:
                raise ValueError("zero or negative PIXEL_SCALE")
            t = np.deg2rad(rot)  # DEG2RAD * rotation (paramvector_processing.cpp:89)
            c, s = np.cos(t), np.sin(t)
            for k in self._set_x0[1:]:
                dx, dy = model[k] - x0r, model[k + 1] - y0r
                model[k] = x0i + ps * (dx * c + dy * s)
                model[k + 1] = y0i + ps * (-dx * s + dy * c)
        scaling = 1.0 / ps  # FunctionObject::SetImageParameters: pixelScaling = 1 / pixScale
        for name, off in self._blocks:
            pa, inten, size = ADJUST[name]
            if pa is not None:
                model[off + pa] = model[off + pa] - rot
            for j in inten:
                model[off + j] = model[off + j] * fs
            for j in size:
                model[off + j] = model[off + j] * scaling
        if self.n_local[i]:
            a = self.local_start[i]
            model = np.concatenate([model, p[a:a + self.n_local[i]]])
        return model

    def local_slice(self, i):
        """Slice of the global vector holding image i's per-image parameters."""
        return slice(self.local_start[i], self.local_start[i] + self.n_local[i])

    def transform_jacobian(self, params, i):
        """T_i = d image_vector(params, i) / d params: central differences on
        the global part of the transform (which is smooth), the identity on
        image i's per-image parameters, zero on the other images'."""
        p = np.asarray(params, dtype=float)
        ng = self.n_image_params + self.n_model
        T = np.zeros((self.n_model + self.n_local[i], self.n_params))
        for j in range(ng):
            h = 1e-6 * max(1.0, abs(p[j]))
            a, b = p.copy(), p.copy()
            a[j] += h
            b[j] -= h
            T[:self.n_model, j] = (self.image_vector(a, i)[:self.n_model] -
                                   self.image_vector(b, i)[:self.n_model]) / (2 * h)
        if self.n_local[i]:
            a = self.local_start[i]
            T[self.n_model:, a:a + self.n_local[i]] = np.eye(self.n_local[i])
        return T

    # ---------------------------------------------------- ModelObject surface
    def get_fit_statistic(self, params):
        """ModelObjectMultImage::GetFitStatistic (model_object_multimage.cpp:359-405):
        the sum over images, FP64 plain path."""
        return float(sum(m.get_fit_statistic(self.image_vector(params, i)) for i, m in enumerate(self.handles)))

    def compute_deviates(self, params):
        return np.concatenate([m.compute_deviates(self.image_vector(params, i)) for i, m in enumerate(self.handles)])

    def statistic_and_gradient(self, params):
        S, g = 0.0, np.zeros(self.n_params)
        for i, m in enumerate(self.handles):
            s_i, g_i = m.statistic_and_gradient(self.image_vector(params, i))
            S += s_i
            g += self.transform_jacobian(params, i).T @ g_i
        return S, g

    def batch_statistic_and_gradient(self, P, want_grad=True):
        P = np.atleast_2d(np.asarray(P, dtype=float))
        B = P.shape[0]
        S = np.zeros(B)
        G = np.zeros((B, self.n_params)) if want_grad else None
        for i, m in enumerate(self.handles):
            Pi = np.array([self.image_vector(P[b], i) for b in range(B)])
            r = m.batch_statistic_and_gradient(Pi, want_grad=want_grad)
            if want_grad:
                s_i, g_i = r
                for b in range(B):
                    G[b] += self.transform_jacobian(P[b], i).T @ g_i[b]
            else:
                s_i = r
            S += s_i
        return (S, G) if want_grad else S

    def jtwj(self, params):
        """S, A = sum T_i^T A_i T_i, b = sum T_i^T b_i."""
        S, A, b = 0.0, np.zeros((self.n_params, self.n_params)), np.zeros(self.n_params)
        for i, m in enumerate(self.handles):
            s_i, A_i, b_i = m.jtwj(self.image_vector(params, i))
            T = self.transform_jacobian(params, i)
            S += s_i
            A += T.T @ A_i @ T
            b += T.T @ b_i
        return S, A, b

    def fit_lm(self, params, fixed=None, lower=None, upper=None, ftol=1e-8, max_iter=0):
        """Levenberg-Marquardt on the summed normal equations with the library's
        driver (the same one imfit_FitLM runs)."""
        from . import minimize_normal_equations
        return minimize_normal_equations(self.jtwj, params, fixed, lower, upper, ftol, max_iter)




def build_handles(functions, images, device=0, subsampling=True, statistic="chi2", model_errors=False,
                  read_image=None):
    """One configured ModelObject per ImageInfo (multimfit_main.cpp's setup
    of each image: the global functions, then the image's per-image functions,
    PSF, data, characteristics, errors, mask, statistic)."""
    from . import fits
    read_image = read_image or (lambda path: fits.read_image(path)[0])
    handles = []
    for im in images:
        m = ModelObject(device)
        for name, new_set in list(functions) + im.local_functions:
            m.add_function(name, new_set, subsampling=subsampling)
        m.finish_functions()
        if im.psf:
            m.add_psf(read_image(im.psf))
        m.add_image_data(read_image(im.data))
        o = im.options
        m.add_image_characteristics(float(o.get("GAIN", 1.0)), float(o.get("READNOISE", 0.0)),
                                    float(o.get("EXPTIME", 1.0)), int(float(o.get("NCOMBINED", 1))),
                                    float(o.get("ORIGINAL_SKY", 0.0)))
        if im.error:
            kind = 110 if "ERRORS_ARE_VARIANCES" in im.flags else (120 if "ERRORS_ARE_WEIGHTS" in im.flags else 100)
            m.add_error_vector(read_image(im.error), kind)
        if im.mask:
            m.add_mask_vector(read_image(im.mask), 20 if "MASK_ZERO_IS_BAD" in im.flags else 10)
        if statistic == "cash":
            m.use_cash()
        elif statistic == "pmlr":
            m.use_pmlr()
        if model_errors:
            m.use_model_errors()
        if m.final_setup() != 0:
            raise RuntimeError("FinalSetupForFitting failed for " + str(im.data))
        handles.append(m)
    return handles


def section_offsets(cfg, images):
    """CorrectForImageOffsets (core/utilities_multimfit.cpp:34-95): the vector
    to subtract from the global vector's values and limits (and to add back
    to fitted values) when images are image sections -- each later image's
    X0/Y0 description parameters by that image's (x1 - 1, y1 - 1), the
    model's X0/Y0 by the reference image's.  A per-image function set's
    X0/Y0 lie in its own image's frame and move by that image's offset (the
    reference's loop over parameter names does not reach them: it indexes
    the global parameter names only)."""
    from . import fits
    nip = N_IMAGE_PARAMS * (len(images) - 1)
    n_local = [len(im.local.values) if im.local is not None else 0 for im in images]
    off = np.zeros(nip + len(cfg.values) + sum(n_local))
    for i, im in enumerate(images[1:], start=1):
        off[N_IMAGE_PARAMS * (i - 1) + 3:N_IMAGE_PARAMS * i] = fits.image_offset(im.data)
    dx, dy = fits.image_offset(images[0].data)
    for j, name in enumerate(cfg.param_names):
        if name == "X0":
            off[nip + j] = dx
        elif name == "Y0":
            off[nip + j] = dy
    start = nip + len(cfg.values)
    for im, n in zip(images, n_local):
        if n:
            ix, iy = fits.image_offset(im.data)
            for j, name in enumerate(im.local.param_names):
                if name == "X0":
                    off[start + j] = ix
                elif name == "Y0":
                    off[start + j] = iy
        start += n
    return off


def global_vector(cfg, images):
    """(values, lower, upper, fixed) of the global vector: the image-description
    parameters of images 2..N (defaults 1, 0, 1 and the reference model's X0,
    Y0), then the configuration's parameters, then each image's per-image
    parameters in image order."""
    vals, lo, hi, fx = [], [], [], []
    defaults = {"PIXEL_SCALE": 1.0, "IMAGE_PA": 0.0, "FLUX_SCALE": 1.0, "X0": cfg.values[0], "Y0": cfg.values[1]}
    for im in images[1:]:
        for name in IMAGE_PARAM_NAMES:
            v, l, h, f = im.params.get(name, (defaults[name], np.nan, np.nan, name in ("PIXEL_SCALE", "IMAGE_PA",
                                                                                     "FLUX_SCALE")))
            vals.append(v)
            lo.append(l)
            hi.append(h)
            fx.append(int(f))
    vals += list(cfg.values)
    lo += list(cfg.lower)
    hi += list(cfg.upper)
    fx += list(cfg.fixed)
    for im in images:
        if im.local is not None:
            vals += list(im.local.values)
            lo += list(im.local.lower)
            hi += list(im.local.upper)
            fx += list(im.local.fixed)
    return np.array(vals), np.array(lo), np.array(hi), np.array(fx, dtype=int)


def parameter_names(cfg, images):
    """Names of the global vector's entries, in order (image-description
    names carry their image number, per-image names their image's)."""
    names = [f"{n}_{i + 1}" for i in range(1, len(images)) for n in IMAGE_PARAM_NAMES]
    names += list(cfg.param_names)
    for i, im in enumerate(images):
        if im.local is not None:
            names += [f"{n}_{i + 1}" for n in im.local.param_names]
    return names
