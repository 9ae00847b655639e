"""An imfit-style command line on the GPU path.

    python -m imfit_gb300.cli CONFIG IMAGE [--psf F] [--mask F] [--noise F] ...

Reads an Imfit configuration file and FITS images, sets the model up in the
reference's order (core/setup_model_object.cpp:36-157), and either prints the
fit statistic at the initial parameters (--chisquare-only) or fits with the
Levenberg-Marquardt driver on the GPU's J^T J (chi^2 or Poisson-MLR; the Cash
statistic has no deviates to fit by least squares).  The option names follow
imfit.s (core/imfit_main.cpp, core/options_imfit.h); only the ones that matter
for the model-image path are accepted.
"""
import argparse
import sys

import numpy as np

from . import ModelObject
from . import fits as fitsio
from .config import ConfigError, format_params, read_config

WEIGHTS_ARE_SIGMAS, WEIGHTS_ARE_VARIANCES, WEIGHTS_ARE_WEIGHTS = 100, 110, 120
MASK_ZERO_IS_GOOD, MASK_ZERO_IS_BAD = 10, 20


def build_parser():
    ap = argparse.ArgumentParser(prog="imfit_gb300.cli", description=__doc__.splitlines()[0])
    ap.add_argument("config")
    ap.add_argument("image")
    ap.add_argument("--psf")
    ap.add_argument("--mask")
    ap.add_argument("--noise")
    ap.add_argument("--errors-are-variances", action="store_true")
    ap.add_argument("--errors-are-weights", action="store_true")
    ap.add_argument("--mask-zero-is-bad", action="store_true")
    ap.add_argument("--gain", type=float)
    ap.add_argument("--readnoise", type=float)
    ap.add_argument("--exptime", type=float)
    ap.add_argument("--ncombined", type=int)
    ap.add_argument("--sky", type=float, help="original sky level (ORIGINAL_SKY)")
    ap.add_argument("--cashstat", action="store_true")
    ap.add_argument("--poisson-mlr", action="store_true")
    ap.add_argument("--model-errors", action="store_true")
    ap.add_argument("--nosubsampling", action="store_true")
    ap.add_argument("--chisquare-only", action="store_true")
    ap.add_argument("--ftol", type=float, default=1e-8)
    ap.add_argument("--max-iter", type=int, default=0)
    ap.add_argument("--save-params", default="bestfit_parameters_imfit_gb300.dat")
    ap.add_argument("--save-model")
    ap.add_argument("--save-residual")
    ap.add_argument("--device", type=int, default=0)
    return ap


def setup_model(cfg, args, image):
    m = ModelObject(args.device)
    for name, new_set in cfg.functions:
        m.add_function(name, new_set, subsampling=not args.nosubsampling)
    m.finish_functions()
    if args.psf:
        m.add_psf(fitsio.read_image(args.psf)[0])
    m.add_image_data(image)
    gain = args.gain if args.gain is not None else cfg.gain
    rn = args.readnoise if args.readnoise is not None else cfg.read_noise
    et = args.exptime if args.exptime is not None else cfg.exp_time
    nc = args.ncombined if args.ncombined is not None else cfg.n_combined
    sky = args.sky if args.sky is not None else cfg.original_sky
    m.add_image_characteristics(gain, rn, et, nc, sky)
    if args.noise:
        kind = WEIGHTS_ARE_VARIANCES if args.errors_are_variances else (
            WEIGHTS_ARE_WEIGHTS if args.errors_are_weights else WEIGHTS_ARE_SIGMAS)
        m.add_error_vector(fitsio.read_image(args.noise)[0], kind)
    if args.mask:
        m.add_mask_vector(fitsio.read_image(args.mask)[0], MASK_ZERO_IS_BAD if args.mask_zero_is_bad
                          else MASK_ZERO_IS_GOOD)
    if args.cashstat:
        m.use_cash()
    elif args.poisson_mlr:
        m.use_pmlr()
    if args.model_errors:
        m.use_model_errors()
    st = m.final_setup()
    if st != 0:
        raise RuntimeError(f"FinalSetupForFitting returned {st}")
    return m


def run(argv=None, out=sys.stdout):
    """Returns (fitted parameters, statistic)."""
    args = build_parser().parse_args(argv)
    try:
        cfg = read_config(args.config)
    except ConfigError as e:
        raise SystemExit(f"error in {args.config}: {e}")
    image = fitsio.read_image(args.image)[0]
    m = setup_model(cfg, args, image)
    p0 = np.array(cfg.values, dtype=float)
    if args.chisquare_only:
        s = m.get_fit_statistic(p0)
        out.write(f"fit statistic = {s:.6f}\n")
        return p0, s
    if args.cashstat:
        raise SystemExit("the Cash statistic has no deviates: use --chisquare-only, or fit chi^2 / "
                         "--poisson-mlr")
    limited = ~np.isnan(cfg.lower)
    lo = np.where(limited, cfg.lower, 0.0)
    hi = np.where(limited, cfg.upper, 0.0)  # lower >= upper means no limit
    r = m.fit_lm(p0, fixed=cfg.fixed, lower=lo, upper=hi, ftol=args.ftol, max_iter=args.max_iter)
    p = r["params"]
    s = m.get_fit_statistic(p)  # FP64 statistic at the fitted point
    n_free = int(np.sum(cfg.fixed == 0))
    dof = m.n_valid - n_free
    out.write(f"status {r['status']} after {r['niter']} iterations ({r['nev']} J^T J evaluations)\n")
    out.write(f"fit statistic = {s:.6f}, reduced = {s / dof:.6f} ({dof} degrees of freedom)\n")
    for name, v in zip(cfg.param_names, p):
        out.write(f"  {name:8s} {v:.6f}\n")
    if args.save_params:
        with open(args.save_params, "w") as f:
            f.write(format_params(cfg, p, s))
    if args.save_model or args.save_residual:
        m.create_model_image(p)
        model = m.get_model_image()
        if args.save_model:
            fitsio.write_image(args.save_model, model)
        if args.save_residual:
            fitsio.write_image(args.save_residual, image - model)
    return p, s


if __name__ == "__main__":
    run()
