"""Fitting many cutouts of uneven sizes with one model on the GPU.

Default ("set"): all cutouts go into ONE handle as a cutout set
(``ModelObject.setup_cutouts``): each cutout keeps its own size, PSF and FFT
plan, and every stage of each Levenberg-Marquardt round is one kernel launch
over all cutouts still being fitted (``fit_lm_batch``).

Alternative ("buckets"): cutouts are grouped into size buckets; each bucket becomes one image stack
(``ModelObject.setup_image_stack``): every cutout is padded to the bucket's
size with masked pixels (sigma 0) at the bottom and right, so its pixel
coordinates are unchanged, and its PSF is padded with zeros around its centre
to the bucket's PSF size (odd sizes, so the centre stays the centre pixel).
Each bucket is fitted by the lockstep batched Levenberg-Marquardt
(``fit_lm_batch``): one batched forward-mode J^T J evaluation per round for
all of its cutouts.  Buckets run concurrently, each on its own handle and
CUDA stream, from a pool of host threads (the C calls release the GIL).
"""
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

import imfit_gb300

# bucket ladders: cutout sides (ratio ~1.1 from 48 px) and odd PSF sizes
SIDE_LADDER = [48, 53, 58, 64, 70, 77, 85, 93, 103, 113, 124, 137, 150, 165, 182, 200, 220, 242, 266, 293,
               322, 354, 390, 430, 474, 522, 576]
PSF_LADDER = [15, 25, 31, 37, 43, 51, 57, 63, 71, 81, 101]


@dataclass
class Cutout:
    data: np.ndarray      # rows x cols
    sigma: np.ndarray     # rows x cols (or a scalar broadcast to the cutout)
    psf: np.ndarray       # odd x odd


def _ceil_ladder(v, ladder):
    for x in ladder:
        if x >= v:
            return x
    return v if v % 2 else v + 1


def bucket_of(c):
    nr, nc = c.data.shape
    return (_ceil_ladder(nr, SIDE_LADDER), _ceil_ladder(nc, SIDE_LADDER), _ceil_ladder(c.psf.shape[0], PSF_LADDER))


def _pad_psf(psf, P):
    p = psf.shape[0]
    out = np.zeros((P, P))
    o = (P - p) // 2
    out[o:o + p, o:o + p] = psf
    return out


def build_stack(functions, cutouts, key, device=0, autotune=False):
    """ModelObject holding the cutouts of one bucket as an image stack."""
    NR, NC, P = key
    n = len(cutouts)
    img = np.zeros((n, NR, NC))
    sig = np.zeros((n, NR, NC))
    psf = np.zeros((n, P, P))
    for i, c in enumerate(cutouts):
        nr, nc = c.data.shape
        img[i, :nr, :nc] = c.data
        sig[i, :nr, :nc] = np.broadcast_to(c.sigma, c.data.shape)
        psf[i] = _pad_psf(c.psf, P)
    m = imfit_gb300.ModelObject(device)
    for name, new_set in functions:
        m.add_function(name, new_set)
    m.finish_functions()
    m.set_autotune(autotune)
    m.setup_image_stack(img, sig, psf)
    return m


def build_set(functions, cutouts, device=0):
    """ModelObject holding every cutout as one cutout set (each at its own size)."""
    m = imfit_gb300.ModelObject(device)
    for name, new_set in functions:
        m.add_function(name, new_set)
    m.finish_functions()
    m.setup_cutouts([c.data for c in cutouts], [c.sigma for c in cutouts], [c.psf for c in cutouts])
    return m


class CutoutFitter:
    """The cutouts of a list set up once and fitted many times: one cutout set
    (mode "set", default) or size buckets of image stacks fitted from host
    threads (mode "buckets")."""

    def __init__(self, functions, cutouts, device=0, threads=8, mode="set"):
        self.functions = functions
        self.n = len(cutouts)
        self.mode = mode
        if mode == "set":
            self.model = build_set(functions, cutouts, device)
            self.buckets = []
            return
        groups = {}
        for i, c in enumerate(cutouts):
            groups.setdefault(bucket_of(c), []).append(i)
        # largest buckets (by pixels) first, so the pool finishes together
        self.buckets = sorted(groups.items(), key=lambda kv: -kv[0][0] * kv[0][1] * len(kv[1]))
        self.threads = threads
        self.models = [None] * len(self.buckets)

        def setup(k):
            key, idx = self.buckets[k]
            self.models[k] = build_stack(functions, [cutouts[i] for i in idx], key, device)

        with ThreadPoolExecutor(self.threads) as ex:
            list(ex.map(setup, range(len(self.buckets))))

    def fit(self, starts, lower=None, upper=None, fixed=None, ftol=1e-8, max_iter=0):
        """Fit every cutout from starts (n x nParams); returns dict of arrays in cutout order."""
        starts = np.asarray(starts, dtype=np.float64)
        if self.mode == "set":
            r = self.model.fit_lm_batch(starts, fixed=fixed, lower=lower, upper=upper, ftol=ftol, max_iter=max_iter)
            return dict(params=r["params"], statistic=r["statistic"], niter=r["niter"], status=r["status"])
        out_p = np.empty_like(starts)
        out_s = np.empty(self.n)
        out_it = np.empty(self.n, dtype=int)
        out_st = np.empty(self.n, dtype=int)

        def run(k):
            key, idx = self.buckets[k]
            lo = None if lower is None else np.asarray(lower)[idx]
            hi = None if upper is None else np.asarray(upper)[idx]
            r = self.models[k].fit_lm_batch(starts[idx], fixed=fixed, lower=lo, upper=hi, ftol=ftol,
                                            max_iter=max_iter)
            out_p[idx] = r["params"]
            out_s[idx] = r["statistic"]
            out_it[idx] = r["niter"]
            out_st[idx] = r["status"]

        with ThreadPoolExecutor(self.threads) as ex:
            list(ex.map(run, range(len(self.buckets))))
        return dict(params=out_p, statistic=out_s, niter=out_it, status=out_st)
