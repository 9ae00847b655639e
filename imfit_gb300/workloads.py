"""Synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: every image is generated from a fixed seed.
Each workload lists the model functions (config-file names), the true
parameter vector, the PSF(s), the image characteristics, the mask and the
statistic, and is turned into a configured model object by ``configure`` for
any implementation that offers the ModelObject-shaped interface (the GPU
``imfit_gb300.ModelObject`` or the CPU oracle).

  C1  256x256  Sersic + FlatSky, 51x51 Moffat PSF (fwhm 4, beta 3), chi^2 with
      data-based errors (gain 4, read noise 5 e-), 8 parameters.
  C2  1024x1024 Sersic + Exponential + FlatSky, 63x63 Moffat (fwhm 4.5, beta 3.5),
      central 40x40 region oversampled 5x with a 315x315 Moffat, 10% random mask,
      Poisson noise, chi^2, 12 parameters.
  C3  512x512 edge-on ExponentialDisk3D (h 40, n 1, z_0 6, inc U[80,90]) +
      FerrersBar3D (R_bar 30, q 0.4, q_z 0.2667, n 2, random bar PA), 35x35
      Gaussian PSF (sigma 1.5), Gaussian noise sigma 5 given as an error image,
      chi^2, 16 parameters.
  C4  512x512 Poisson counts, Sersic + Exponential + GaussianRing (R 60, sigma 8)
      + FlatSky, 51x51 Moffat, Cash statistic, 256 parameter vectors drawn
      within +-30% boxes around the truth (positions +-3 px), 17 parameters.
"""
from dataclasses import dataclass, field

import numpy as np

WEIGHTS_ARE_SIGMAS = 100


def moffat_psf(n, fwhm, beta, sub=5):
    """Circular Moffat sampled on an n x n grid centred at pixel (n-1)/2, sub x sub subsampled, sum 1."""
    alpha = fwhm / (2.0 * np.sqrt(2.0 ** (1.0 / beta) - 1.0))
    c = (n - 1) / 2.0
    off = (np.arange(sub) + 0.5) / sub - 0.5
    y, x = np.mgrid[0:n, 0:n].astype(np.float64)
    acc = np.zeros((n, n))
    for oy in off:
        for ox in off:
            r2 = (x + ox - c) ** 2 + (y + oy - c) ** 2
            acc += (1.0 + r2 / alpha ** 2) ** (-beta)
    return acc / acc.sum()


def gaussian_psf(n, sigma, sub=5):
    c = (n - 1) / 2.0
    off = (np.arange(sub) + 0.5) / sub - 0.5
    y, x = np.mgrid[0:n, 0:n].astype(np.float64)
    acc = np.zeros((n, n))
    for oy in off:
        for ox in off:
            acc += np.exp(-((x + ox - c) ** 2 + (y + oy - c) ** 2) / (2 * sigma ** 2))
    return acc / acc.sum()


@dataclass
class Workload:
    name: str
    ncols: int
    nrows: int
    functions: list                # [(name, starts_new_set)]
    truth: np.ndarray
    psf: np.ndarray = None
    regions: list = field(default_factory=list)  # [(psf, scale, (x1, x2, y1, y2))]
    gain: float = 1.0
    read_noise: float = 0.0
    original_sky: float = 0.0
    stat: str = "chi2"             # chi2 | cash | pmlr
    mask: np.ndarray = None        # 0 = good (MASK_ZERO_IS_GOOD)
    errors: np.ndarray = None      # sigma image, or None for data-based errors
    data: np.ndarray = None
    start: np.ndarray = None
    batch: np.ndarray = None
    seed: int = 0
    noise: str = "poisson+read"    # poisson+read | poisson | gaussian
    noise_sigma: float = 0.0

    @property
    def n_params(self):
        return len(self.truth)


def configure(model, wl, with_data=True):
    """Apply the reference's setup order (core/setup_model_object.cpp:36-157)."""
    for name, new_set in wl.functions:
        model.add_function(name, new_set)
    model.finish_functions()
    if wl.psf is not None:
        model.add_psf(wl.psf)
    if with_data:
        model.add_image_data(wl.data)
    else:
        model.setup_model_image(wl.ncols, wl.nrows)
    model.add_image_characteristics(wl.gain, wl.read_noise, 1.0, 1, wl.original_sky)
    for psf, scale, reg in wl.regions:
        model.add_oversampled_psf(psf, scale, reg)
    if not with_data:
        return model
    if wl.errors is not None:
        model.add_error_vector(wl.errors, WEIGHTS_ARE_SIGMAS)
    if wl.mask is not None:
        model.add_mask_vector(wl.mask)
    if wl.stat == "cash":
        model.use_cash()
    elif wl.stat == "pmlr":
        model.use_pmlr()
    st = model.final_setup()
    if st != 0:
        raise RuntimeError(f"FinalSetupForFitting returned {st}")
    return model


def synthesize(wl, model_cls):
    """Fill wl.data from the true model (computed by model_cls) plus seeded noise."""
    m = configure(model_cls(), wl, with_data=False)
    m.create_model_image(wl.truth)
    img = m.get_model_image()
    rng = np.random.default_rng(wl.seed)
    if wl.noise == "poisson+read":
        e = rng.poisson(np.clip(img + wl.original_sky, 0, None) * wl.gain).astype(np.float64)
        e += rng.normal(0.0, wl.read_noise, img.shape)
        wl.data = e / wl.gain - wl.original_sky
    elif wl.noise == "poisson":
        wl.data = rng.poisson(np.clip(img * wl.gain, 0, None)).astype(np.float64) / wl.gain
    else:
        wl.data = img + rng.normal(0.0, wl.noise_sigma, img.shape)
    return wl


def _perturb(rng, truth, names, frac=0.1, pos=1.0):
    p = truth.copy()
    for i, n in enumerate(names):
        if n in ("X0", "Y0"):
            p[i] += rng.uniform(-pos, pos)
        else:
            p[i] *= 1.0 + rng.uniform(-frac, frac)
    return p


def param_names(functions):
    table = {"Sersic": ["PA", "ell", "n", "I_e", "r_e"], "Exponential": ["PA", "ell", "I_0", "h"],
             "FlatSky": ["I_sky"], "GaussianRing": ["PA", "ell", "A", "R_ring", "sigma_r"],
             "Moffat": ["PA", "ell", "I_0", "fwhm", "beta"], "Gaussian": ["PA", "ell", "I_0", "sigma"],
             "ExponentialDisk3D": ["PA", "inc", "J_0", "h", "n", "z_0"],
             "FerrersBar3D": ["PA", "inc", "barPA", "J_0", "R_bar", "q", "q_z", "n"],
             "PointSource": ["I_tot"], "PointSourceRot": ["PA", "I_tot"], "TiltedSkyPlane": ["I_0", "m_x", "m_y"]}
    out = []
    for i, (name, new_set) in enumerate(functions):
        if new_set or i == 0:
            out += ["X0", "Y0"]
        out += table[name]
    return out


def c1(size=256, psf_size=51, seed=1001):
    s = size / 256.0
    truth = np.array([size / 2 + 0.5, size / 2 + 0.5, 20.0, 0.3, 2.5, 20.0, 25.0 * s, 100.0])
    wl = Workload("C1", size, size, [("Sersic", True), ("FlatSky", False)], truth,
                  psf=moffat_psf(psf_size, 4.0, 3.0), gain=4.0, read_noise=5.0, seed=seed)
    rng = np.random.default_rng(seed + 7)
    wl.start = _perturb(rng, truth, param_names(wl.functions))
    return wl


def c2(size=1024, psf_size=63, region=40, scale=5, os_psf_size=315, seed=1002):
    rng = np.random.default_rng(seed)
    cx = size / 2 + 0.5 + rng.uniform(-0.5, 0.5)
    cy = size / 2 + 0.5 + rng.uniform(-0.5, 0.5)
    n = rng.uniform(1, 4)
    r_e = rng.uniform(5, 30) * size / 1024
    ell_s = rng.uniform(0, 0.4)
    h = rng.uniform(20, 80) * size / 1024
    ell_d = rng.uniform(0.2, 0.6)
    truth = np.array([cx, cy, rng.uniform(0, 180), ell_s, n, 50.0, r_e,
                      rng.uniform(0, 180), ell_d, 20.0, h, 100.0])
    half = region // 2
    c = size // 2
    reg = (c - half + 1, c + half, c - half + 1, c + half)
    wl = Workload("C2", size, size, [("Sersic", True), ("Exponential", False), ("FlatSky", False)], truth,
                  psf=moffat_psf(psf_size, 4.5, 3.5),
                  regions=[(moffat_psf(os_psf_size, 4.5 * scale, 3.5), scale, reg)],
                  gain=4.0, read_noise=5.0, seed=seed)
    wl.mask = (rng.random((size, size)) < 0.10).astype(np.float64)
    wl.start = _perturb(rng, truth, param_names(wl.functions))
    return wl


def c3(size=512, psf_size=35, seed=1003):
    rng = np.random.default_rng(seed)
    s = size / 512.0
    c = size / 2 + 0.5
    pa = rng.uniform(0, 180)
    inc = rng.uniform(80, 90)
    truth = np.array([c + rng.uniform(-0.5, 0.5), c + rng.uniform(-0.5, 0.5),
                      pa, inc, 0.5, 40.0 * s, 1.0, 6.0 * s,
                      pa, inc, rng.uniform(0, 180), 0.2, 30.0 * s, 0.4, 0.2667, 2.0])
    wl = Workload("C3", size, size, [("ExponentialDisk3D", True), ("FerrersBar3D", False)], truth,
                  psf=gaussian_psf(psf_size, 1.5), seed=seed, noise="gaussian", noise_sigma=5.0)
    wl.errors = np.full((size, size), 5.0)
    names = param_names(wl.functions)
    p = truth.copy()
    for i, nm in enumerate(names):
        if nm in ("X0", "Y0"):
            p[i] += rng.uniform(-1, 1)
        elif nm == "inc":
            p[i] = min(p[i] + rng.uniform(-2, 2), 90.0)
        elif nm in ("PA", "barPA"):
            p[i] += rng.uniform(-3, 3)
        else:
            p[i] *= 1.0 + rng.uniform(-0.05, 0.05)
    wl.start = p
    return wl


def c4(size=512, psf_size=51, batch=256, seed=1004):
    rng = np.random.default_rng(seed)
    s = size / 512.0
    c = size / 2 + 0.5
    truth = np.array([c, c, 30.0, 0.2, 2.0, 40.0, 15.0 * s,
                      60.0, 0.4, 15.0, 40.0 * s,
                      60.0, 0.4, 10.0, 60.0 * s, 8.0 * s,
                      5.0])
    wl = Workload("C4", size, size,
                  [("Sersic", True), ("Exponential", False), ("GaussianRing", False), ("FlatSky", False)],
                  truth, psf=moffat_psf(psf_size, 4.0, 3.0), gain=1.0, stat="cash", seed=seed,
                  noise="poisson")
    names = param_names(wl.functions)
    B = np.empty((batch, len(truth)))
    for b in range(batch):
        for i, nm in enumerate(names):
            if nm in ("X0", "Y0"):
                B[b, i] = truth[i] + rng.uniform(-3, 3)
            elif nm == "ell":
                B[b, i] = np.clip(truth[i] * (1 + rng.uniform(-0.3, 0.3)), 0.0, 0.9)
            else:
                B[b, i] = truth[i] * (1 + rng.uniform(-0.3, 0.3))
    wl.batch = B
    wl.start = B[0].copy()
    return wl


def small_case(seed=7, ncols=64, nrows=48, psf=15, region=True, mask=True, stat="chi2"):
    """A small image exercising every setup feature (used by the parity tests)."""
    rng = np.random.default_rng(seed)
    truth = np.array([30.3, 22.7, 35.0, 0.35, 1.8, 30.0, 6.0,
                      110.0, 0.5, 12.0, 9.0,
                      20.0, 0.1, 3.0, 15.0, 2.5, 5.0])
    fns = [("Sersic", True), ("Exponential", False), ("GaussianRing", False), ("FlatSky", False)]
    regs = []
    if region:
        regs = [(moffat_psf(3 * psf, 3 * 2.5, 3.0), 3, (26, 33, 19, 26))]
    wl = Workload("small", ncols, nrows, fns, truth, psf=moffat_psf(psf, 2.5, 3.0), regions=regs,
                  gain=3.0, read_noise=4.0, original_sky=20.0, stat=stat, seed=seed)
    if mask:
        m = (rng.random((nrows, ncols)) < 0.1).astype(np.float64)
        m[0, 0] = np.nan  # non-finite mask values count as masked
        wl.mask = m
    wl.start = _perturb(rng, truth, param_names(fns), frac=0.05, pos=0.5)
    return wl


def sersic_total_flux(n, I_e, r_e, ell):
    """Sersic::TotalFlux (function_objects/func_sersic.cpp:246-251)."""
    import math
    bn = _sersic_bn(n)
    return 2.0 * math.pi * n * math.exp(bn) * bn ** (-2.0 * n) * math.gamma(2.0 * n) * (1.0 - ell) * r_e * r_e * I_e


def exp_total_flux(I_0, h, ell):
    """Exponential::TotalFlux (function_objects/func_exp.cpp:210-213)."""
    import math
    return 2.0 * math.pi * I_0 * h * h * (1.0 - ell)


def _sersic_bn(n):
    # function_objects/helper_funcs.cpp:14-29
    n2 = n * n
    if n > 0.36:
        return (2 * n - 0.333333333333333 + 0.009876543209876543 / n + 0.0018028610621203215 / n2
                + 0.00011409410586365319 / (n2 * n) - 7.1510122958919723e-05 / (n2 * n2))
    return 0.01945 + -0.8902 * n + 10.95 * n2 + -19.67 * n2 * n + 13.43 * n2 * n2


C5_FUNCTIONS = [("Sersic", True), ("Exponential", False)]


def c5(count=4096, seed=1005, min_side=48, max_side=384):
    """Uneven batch of cutouts: side log-uniform [min_side, max_side], Sersic
    (n U[0.5,6], r_e U[2,60] capped by the side, ell U[0,0.7]) + Exponential
    with B/T U[0,1] through the TotalFlux formulas, per-cutout Moffat PSF
    (odd 25..63 px, fwhm U[2.5,6], beta U[2.5,4.5]), sky s U[30,70] subtracted
    and Gaussian noise sigma = sqrt(s).  Returns a dict with the per-cutout
    geometry, truth, start and limits; the images are made by synthesize_c5."""
    rng = np.random.default_rng(seed)
    items = []
    for k in range(count):
        side = int(np.floor(np.exp(rng.uniform(np.log(min_side), np.log(max_side)))))
        side = max(min_side, min(side, max_side))
        P = int(rng.integers(12, 32)) * 2 + 1  # odd 25..63
        fwhm = rng.uniform(2.5, 6.0)
        beta = rng.uniform(2.5, 4.5)
        c = side / 2 + 0.5
        x0, y0 = c + rng.uniform(-1, 1), c + rng.uniform(-1, 1)
        n = rng.uniform(0.5, 6.0)
        r_e = min(rng.uniform(2.0, 60.0), side / 4)
        ell_b = rng.uniform(0.0, 0.7)
        h = min(rng.uniform(3.0, 40.0), side / 5)
        ell_d = rng.uniform(0.0, 0.7)
        bt = rng.uniform(0.0, 1.0)
        flux = np.exp(rng.uniform(np.log(3e4), np.log(3e5)))
        sky = rng.uniform(30.0, 70.0)
        fb, fd = max(bt, 0.02) * flux, max(1.0 - bt, 0.02) * flux
        I_e = fb / sersic_total_flux(n, 1.0, r_e, ell_b)
        I_0 = fd / exp_total_flux(1.0, h, ell_d)
        truth = np.array([x0, y0, rng.uniform(0, 180), ell_b, n, I_e, r_e, rng.uniform(0, 180), ell_d, I_0, h])
        start = truth.copy()
        for i in range(len(truth)):
            if i < 2:
                start[i] += rng.uniform(-1, 1)
            elif i in (2, 7):
                start[i] += rng.uniform(-5, 5)
            else:
                start[i] *= 1.0 + rng.uniform(-0.1, 0.1)
        start[3] = min(start[3], 0.9)
        start[8] = min(start[8], 0.9)
        lower = np.array([x0 - 10, y0 - 10, -360, 0.0, 0.3, 0.0, 0.3, -360, 0.0, 0.0, 0.3])
        upper = np.array([x0 + 10, y0 + 10, 360, 0.95, 10.0, 1e9, 4.0 * side, 360, 0.95, 1e9, 4.0 * side])
        items.append(dict(side=side, psf_size=P, fwhm=fwhm, beta=beta, sky=sky, truth=truth, start=start,
                          lower=lower, upper=upper, seed=seed * 7919 + k))
    return items


def synthesize_c5(items, model_cls, sub=5):
    """Images for c5() items: model (model_cls, FP64) + Gaussian noise, and the PSFs."""
    out = []
    for it in items:
        psf = moffat_psf(it["psf_size"], it["fwhm"], it["beta"], sub=sub)
        m = model_cls()
        for name, new_set in C5_FUNCTIONS:
            m.add_function(name, new_set)
        m.finish_functions()
        m.add_psf(psf)
        m.setup_model_image(it["side"], it["side"])
        m.create_model_image(it["truth"])
        img = m.get_model_image()
        rng = np.random.default_rng(it["seed"])
        sigma = np.sqrt(it["sky"])
        data = img + rng.normal(0.0, sigma, img.shape)
        out.append((data, np.full(img.shape, sigma), psf))
    return out
