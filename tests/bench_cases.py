"""The benchmark configurations at their full sizes, as parity cases.

Shared by tests/golden/make_golden.py (which stores the reference's own
values for them, computed by the reference's hot-path sources compiled here)
and the GPU tests at benchmark sizes.  Data are synthesized from the seeded
workloads with the oracle, so every machine builds the same images; a model
image is compared through digests (row sums, column sums and a fixed sample
of pixels) because the full images are too large to commit.

  C1  256x256   Sersic + FlatSky, 51x51 Moffat, chi^2 with data-based errors
  C2  1024x1024 Sersic + Exponential + FlatSky, 63x63 Moffat, 40x40 region at
                5x with a 315x315 PSF, 10 % mask, chi^2 (padded FFT 1150+63-1)
  C3  512x512   ExponentialDisk3D + FerrersBar3D, 35x35 Gaussian, chi^2 with
                an error image
  C4  512x512   Sersic + Exponential + GaussianRing + FlatSky, 51x51 Moffat,
                Cash; the first four of the 256 parameter vectors
"""
import numpy as np

from imfit_gb300 import workloads

NAMES = ("C1", "C2", "C3", "C4")
N_SAMPLE = 512


def build(name):
    """The workload with its data synthesized by the FP64 oracle."""
    import oracle
    wl = {"C1": workloads.c1, "C2": workloads.c2, "C3": workloads.c3, "C4": workloads.c4}[name]()
    workloads.synthesize(wl, oracle.OracleModel)
    return wl


def vectors(wl):
    """(tag, parameter vector) pairs checked for a workload."""
    if wl.batch is not None:
        return [(f"b{k}", wl.batch[k]) for k in range(4)]
    return [("truth", wl.truth), ("start", wl.start)]


def sample_index(shape):
    return np.sort(np.random.default_rng(99).choice(shape[0] * shape[1], N_SAMPLE, replace=False))


def digest(img):
    """Row sums, column sums and the fixed pixel sample of a model image."""
    img = np.asarray(img, dtype=np.float64)
    return img.sum(axis=1), img.sum(axis=0), img.ravel()[sample_index(img.shape)]


def data_digest(wl):
    d = np.asarray(wl.data, dtype=np.float64)
    return np.array([d.sum(), (d * d).sum(), d.ravel()[::997].sum()])


def configure(cls, wl, subsampling=True):
    """workloads.configure with the per-function subsampling flag."""
    m = cls()
    if subsampling:
        return workloads.configure(m, wl)
    for name, new_set in wl.functions:
        m.add_function(name, new_set, subsampling=False)
    m.finish_functions()
    m.add_psf(wl.psf)
    m.add_image_data(wl.data)
    m.add_image_characteristics(wl.gain, wl.read_noise, 1.0, 1, wl.original_sky)
    for psf, scale, reg in wl.regions:
        m.add_oversampled_psf(psf, scale, reg)
    if wl.errors is not None:
        m.add_error_vector(wl.errors, workloads.WEIGHTS_ARE_SIGMAS)
    if wl.mask is not None:
        m.add_mask_vector(wl.mask)
    if wl.stat == "cash":
        m.use_cash()
    assert m.final_setup() == 0
    return m
