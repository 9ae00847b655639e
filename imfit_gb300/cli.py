"""imfit- and makeimage-style command lines on the GPU path.

    python -m imfit_gb300.cli CONFIG IMAGE [--psf F] [--mask F] [--noise F] ...
    python -m imfit_gb300.cli makeimage CONFIG [--ncols N --nrows M | --refimage F] ...
    python -m imfit_gb300.cli mcmc CONFIG IMAGE [--nchains N] [--max-chain-length N] ...
    python -m imfit_gb300.cli multimfit CONFIG --image-info FILE [--nm | --de] ...

Reads an Imfit configuration file and FITS images and sets the model up in
the reference's order (core/setup_model_object.cpp:36-157).  The fitting
command either prints the fit statistic at the initial parameters
(--chisquare-only) or fits: Levenberg-Marquardt on the GPU's J^T J (chi^2 or
Poisson-MLR; the Cash statistic has no deviates to fit by least squares), or,
with --de, generation-synchronous differential evolution on the batched
statistic.  mcmc runs DREAM (imfit-mcmc) with one batched GPU evaluation per
generation.  makeimage follows core/makeimage_main.cpp:99-380: the model image,
optionally the expanded (PSF-padded) image, single-function images and the
component-flux table.  Option names follow core/imfit_main.cpp and
core/makeimage_main.cpp; only the ones that matter for the model-image path
are accepted.
"""
import argparse
import math
import os
import sys
import time

import numpy as np

from . import ImfitError, ModelObject
from . import fits as fitsio
from .config import ConfigError, format_params, read_config

WEIGHTS_ARE_SIGMAS, WEIGHTS_ARE_VARIANCES, WEIGHTS_ARE_WEIGHTS = 100, 110, 120
MASK_ZERO_IS_GOOD, MASK_ZERO_IS_BAD = 10, 20


def _add_psf_options(ap):
    ap.add_argument("--psf")
    ap.add_argument("--no-normalize", action="store_true", help="do not normalise the PSF images")
    ap.add_argument("--overpsf", action="append", default=[])
    ap.add_argument("--overpsf_scale", action="append", type=int, default=[])
    ap.add_argument("--overpsf_region", action="append", default=[])
    ap.add_argument("--nosubsampling", "--no-subsampling", dest="nosubsampling", action="store_true")
    ap.add_argument("--device", type=int, default=0)


def build_parser():
    ap = argparse.ArgumentParser(prog="imfit_gb300.cli", description=__doc__.splitlines()[0])
    ap.add_argument("config")
    ap.add_argument("image")
    _add_psf_options(ap)
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
    ap.add_argument("--poisson-mlr", "--mlr", dest="poisson_mlr", action="store_true")
    ap.add_argument("--model-errors", action="store_true")
    ap.add_argument("--chisquare-only", "--fitstat-only", dest="chisquare_only", action="store_true")
    ap.add_argument("--de", action="store_true", help="differential evolution instead of LM")
    ap.add_argument("--de-lhs", action="store_true", help="--de with a Latin-hypercube initial population")
    ap.add_argument("--nm", action="store_true", help="Nelder-Mead simplex instead of LM")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--bootstrap", type=int, default=0, help="number of bootstrap resampling iterations")
    ap.add_argument("--save-bootstrap", help="file for the bootstrap best-fit parameters")
    ap.add_argument("--ftol", type=float, default=1e-8)
    ap.add_argument("--max-iter", type=int, default=0)
    ap.add_argument("--save-params", default="bestfit_parameters_imfit_gb300.dat")
    ap.add_argument("--save-model")
    ap.add_argument("--save-residual")
    ap.add_argument("--save-weights", help="file for the weight image (1/sigma^2, masked pixels 0)")
    return ap


def build_makeimage_parser():
    ap = argparse.ArgumentParser(prog="imfit_gb300.cli makeimage",
                                 description="model image from a configuration file")
    ap.add_argument("config")
    _add_psf_options(ap)
    ap.add_argument("-o", "--output", default="modelimage.fits")
    ap.add_argument("--refimage")
    ap.add_argument("--ncols", type=int, default=0)
    ap.add_argument("--nrows", type=int, default=0)
    ap.add_argument("--save-expanded", action="store_true")
    ap.add_argument("--output-functions", help="root name of single-function images")
    ap.add_argument("--nosave", action="store_true")
    ap.add_argument("--print-fluxes", action="store_true")
    ap.add_argument("--save-fluxes")
    ap.add_argument("--zero-point", type=float)
    ap.add_argument("--estimation-size", type=int, default=5000)
    ap.add_argument("--timing", type=int, default=0)
    return ap


def parse_region(text):
    """'x1:x2,y1:y2' (1-based, inclusive) -> (x1, x2, y1, y2)."""
    try:
        xs, ys = text.split(",")
        x1, x2 = (int(v) for v in xs.split(":"))
        y1, y2 = (int(v) for v in ys.split(":"))
    except ValueError:
        raise SystemExit(f"bad oversampled-PSF region {text!r} (want x1:x2,y1:y2)")
    return x1, x2, y1, y2


def _add_psf(m, args):
    if args.psf:
        m.add_psf(_read(args.psf, "PSF image"), normalize=not args.no_normalize)


def _section_offsets(cfg, image_name):
    """X0/Y0 shifts of an image section (core/imfit_main.cpp:211, 288-309,
    350-356): the vector to subtract from the configuration's values and
    limits, and to add back to fitted values."""
    dx, dy = fitsio.image_offset(image_name)
    off = np.zeros(len(cfg.values))
    for j, name in enumerate(cfg.param_names):
        if name == "X0":
            off[j] = dx
        elif name == "Y0":
            off[j] = dy
    return off, (dx, dy)


def _add_oversampled_psfs(m, args, offset=(0, 0)):
    """Oversampled PSFs as core/getimages.cpp:138-200 (after the image size is
    known): one image and scale serve every region, or one per region."""
    if not args.overpsf:
        return
    if not args.overpsf_region:
        raise SystemExit("an oversampled PSF needs at least one --overpsf_region")
    if len(args.overpsf) != len(args.overpsf_scale):
        raise SystemExit("the number of --overpsf_scale values differs from the number of --overpsf images")
    if len(args.overpsf) > 1 and len(args.overpsf) != len(args.overpsf_region):
        raise SystemExit("give one oversampled PSF image, or one per region")
    for k, region in enumerate(args.overpsf_region):
        j = k if len(args.overpsf) > 1 else 0
        if args.overpsf_scale[j] < 1:
            raise SystemExit("--overpsf_scale must be a positive integer")
        x1, x2, y1, y2 = parse_region(region)
        m.add_oversampled_psf(_read(args.overpsf[j], "oversampled PSF image"), args.overpsf_scale[j],
                              (x1 - offset[0], x2 - offset[0], y1 - offset[1], y2 - offset[1]),
                              normalize=not args.no_normalize)


def _add_functions(m, cfg, args):
    for (name, new_set), opt in zip(cfg.functions, cfg.optional):
        try:
            m.add_function(name, new_set, subsampling=not args.nosubsampling, optional=opt)
        except ImfitError as e:  # e.g. SetExtraParams on a function without optional parameters
            raise SystemExit(f"function {name}: {e}")
    m.finish_functions()
    if m.n_params != len(cfg.values):
        raise SystemExit(f"the configuration gives {len(cfg.values)} parameters, the functions need "
                         f"{m.n_params}")


def setup_model(cfg, args, image, offset=(0, 0)):
    m = ModelObject(args.device)
    _add_functions(m, cfg, args)
    _add_psf(m, args)
    m.add_image_data(image)
    _add_oversampled_psfs(m, args, offset)
    gain = args.gain if args.gain is not None else cfg.gain
    rn = args.readnoise if args.readnoise is not None else cfg.read_noise
    et = args.exptime if args.exptime is not None else cfg.exp_time
    nc = args.ncombined if args.ncombined is not None else cfg.n_combined
    sky = args.sky if args.sky is not None else cfg.original_sky
    m.add_image_characteristics(gain, rn, et, nc, sky)
    if args.noise:
        kind = WEIGHTS_ARE_VARIANCES if args.errors_are_variances else (
            WEIGHTS_ARE_WEIGHTS if args.errors_are_weights else WEIGHTS_ARE_SIGMAS)
        m.add_error_vector(_matching_image(args.noise, "noise", image, args.image), kind)
    if args.mask:
        m.add_mask_vector(_matching_image(args.mask, "mask", image, args.image),
                          MASK_ZERO_IS_BAD if args.mask_zero_is_bad else MASK_ZERO_IS_GOOD)
    if args.cashstat:
        m.use_cash()
    elif args.poisson_mlr:
        m.use_pmlr()
    if args.model_errors:
        m.use_model_errors()
    st = m.final_setup()
    if st != 0:  # too few valid pixels, or non-finite weights (core/imfit_main.cpp:279-283)
        raise SystemExit(f"*** ERROR: Failure in ModelObject::FinalSetupForFitting! ({m.last_error})")
    return m


def _read(path, kind):
    """An input image; an unreadable one stops the command with the
    reference's messages (core/image_io.cpp:169-170, core/getimages.cpp:41-45,
    core/imfit_main.cpp:200-204)."""
    try:
        return fitsio.read_image(path)[0]
    except (OSError, ValueError) as e:
        raise SystemExit(f"*** WARNING: {e}!\n*** ERROR: Unable to read {kind} file \"{path}\"!")


def _matching_image(path, kind, image, image_path):
    """A noise or mask image, which must have the data image's dimensions
    (GetImageAndCheckSize, core/getimages.cpp:34-58)."""
    arr = _read(path, kind)
    if arr.shape != image.shape:
        raise SystemExit(f"*** ERROR: Dimensions of {kind} image ({path}: {arr.shape[1]} columns, {arr.shape[0]} "
                         f"rows)\ndo not match dimensions of data image ({image.shape[1]} columns, "
                         f"{image.shape[0]} rows)!")
    return arr


def fit_statistic_lines(statistic, kind, n_free, n_valid):
    """The lines imfit prints for --chisquare-only (PrintFitStatistic,
    core/print_results.cpp:160-181); kind: "chi2", "cash" or "pmlr"."""
    dof = n_valid - n_free
    aic, bic = information_criteria(statistic, n_free, n_valid)
    if kind == "cash":
        lines = [f"  CASH STATISTIC = {statistic:f}"]
    elif kind == "pmlr":
        lines = [f"  POISSON-MLR STATISTIC = {statistic:f}", "", f"Reduced Chi^2 equivalent = {statistic / dof:f}"]
    else:
        lines = [f"  CHI-SQUARE = {statistic:f}    ({dof} DOF)", "", f"Reduced Chi^2 = {statistic / dof:f}"]
    return lines + [f"AIC = {aic:f}, BIC = {bic:f}"]


def information_criteria(statistic, n_free, n_valid):
    """Bias-corrected AIC (Burnham & Anderson 2002, p. 66) and BIC of a fit,
    the statistic standing for -2 ln L (core/statistics.cpp:139-175)."""
    k = float(n_free)
    aic = statistic + 2.0 * k + 2.0 * k * (k + 1.0) / (n_valid - k - 1.0)
    bic = statistic + k * math.log(n_valid)
    return aic, bic


def parameter_errors(m, p, fixed, lower, upper):
    """One-sigma parameter errors as mpfit reports them after an LM fit
    (solvers/mpfit.cpp:1016-1047): the square roots of the diagonal of the
    inverse of J^T J over the free parameters, J the Jacobian of the
    deviates; a parameter held at one of its limits, fixed, or without
    influence on the deviates (a zero column) gets 0.  None when the model
    has no J^T J (3-D line-of-sight components)."""
    try:
        A = m.jtwj(p)[1]
    except ImfitError:
        return None
    p = np.asarray(p, dtype=float)
    limited = ~np.isnan(lower)
    pegged = limited & ((p == lower) | (p == upper))
    use = (np.asarray(fixed) == 0) & ~pegged & (np.diag(A) > 0)
    err = np.zeros(len(p))
    if np.any(use):
        cov = np.linalg.inv(A[np.ix_(use, use)])
        err[use] = np.sqrt(np.clip(np.diag(cov), 0.0, None))
    return err


def run(argv=None, out=sys.stdout, details=None):
    """The fitting command; returns (fitted parameters, statistic).  A dict
    passed as details receives n_valid, n_free, aic, bic and, after an LM
    fit, the parameter errors."""
    details = {} if details is None else details
    args = build_parser().parse_args(argv)
    try:
        cfg = read_config(args.config)
    except ConfigError as e:
        raise SystemExit(f"error in {args.config}: {e}")
    image = _read(args.image, "image")
    off, shift = _section_offsets(cfg, args.image)
    m = setup_model(cfg, args, image, shift)
    p0 = np.array(cfg.values, dtype=float) - off
    cfg_lower, cfg_upper = cfg.lower - off, cfg.upper - off  # NaN (no limit) stays NaN
    n_free = int(np.sum(cfg.fixed == 0))
    if args.chisquare_only:
        s = m.get_fit_statistic(p0)
        kind = "cash" if args.cashstat else ("pmlr" if args.poisson_mlr else "chi2")
        out.write("\n".join(fit_statistic_lines(s, kind, n_free, m.n_valid)) + "\n")
        return p0 + off, s
    if args.de or args.de_lhs:
        from .solvers import differential_evolution
        try:
            r = differential_evolution(m, p0, cfg_lower, cfg_upper, fixed=cfg.fixed.astype(bool),
                                       ftol=args.ftol, seed=args.seed, latin_hypercube=args.de_lhs)
        except ValueError as e:
            raise SystemExit(str(e))
        p = r["params"]
        out.write(f"differential evolution: {r['generations']} generations of {r['population']} "
                  f"({'converged' if r['converged'] else 'generation limit'})\n")
    elif args.nm:
        from .solvers import nelder_mead
        lo = np.where(np.isnan(cfg_lower), -np.inf, cfg_lower)
        hi = np.where(np.isnan(cfg_upper), np.inf, cfg_upper)
        r = nelder_mead(m, p0, lo, hi, fixed=cfg.fixed.astype(bool), ftol=args.ftol)
        p = r["params"]
        out.write(f"Nelder-Mead simplex: {r['evaluations']} evaluations "
                  f"({'converged' if r['converged'] else 'evaluation limit'})\n")
    else:
        if args.cashstat:
            raise SystemExit("the Cash statistic has no deviates: use --chisquare-only, --de, --nm, or fit "
                             "chi^2 / --poisson-mlr")
        limited = ~np.isnan(cfg_lower)
        lo = np.where(limited, cfg_lower, 0.0)
        hi = np.where(limited, cfg_upper, 0.0)  # lower >= upper means no limit
        r = m.fit_lm(p0, fixed=cfg.fixed, lower=lo, upper=hi, ftol=args.ftol, max_iter=args.max_iter)
        p = r["params"]
        out.write(f"status {r['status']} after {r['niter']} iterations ({r['nev']} J^T J evaluations)\n")
    s = m.get_fit_statistic(p)  # FP64 statistic at the fitted point
    p_section = p
    p = p + off  # reported in the full image's coordinates
    dof = m.n_valid - n_free
    aic, bic = information_criteria(s, n_free, m.n_valid)
    errors = None
    if not (args.de or args.de_lhs or args.nm):
        errors = parameter_errors(m, p_section, cfg.fixed, cfg_lower, cfg_upper)
    details.update(n_valid=m.n_valid, n_free=n_free, aic=aic, bic=bic, errors=errors)
    out.write(f"fit statistic = {s:.6f}, reduced = {s / dof:.6f} ({dof} degrees of freedom)\n")
    out.write(f"AIC = {aic:f}, BIC = {bic:f}\n")
    for k, (name, v) in enumerate(zip(cfg.param_names, p)):
        out.write(f"  {name:8s} {v:.6f}" + (f"  +/- {errors[k]:.6g}" if errors is not None else "") + "\n")
    if args.save_params:
        with open(args.save_params, "w") as f:
            f.write(format_params(cfg, p, s))
    if args.save_weights:  # GetWeightImageVector: 1/sigma^2 at the fitted model (core/imfit_main.cpp:466-476)
        fitsio.write_image(args.save_weights, m.get_weights(), bitpix=-64)
    if args.bootstrap > 0:
        run_bootstrap(m, cfg, args, p_section, out, off)
    if args.save_model or args.save_residual:
        m.create_model_image(p_section)
        model = m.get_model_image()
        if args.save_model:
            fitsio.write_image(args.save_model, model)
        if args.save_residual:
            fitsio.write_image(args.save_residual, image - model)
    return p, s


def run_bootstrap(m, cfg, args, bestfit, out, off=None):
    """Bootstrap resampling errors (core/bootstrap_errors.cpp:86-160), all
    refits of a chunk at once on the GPU; off: image-section shifts added back
    to the reported values."""
    off = np.zeros(len(bestfit)) if off is None else off
    from .config import _NPARAMS
    from .solvers import bootstrap_errors, bootstrap_file_lines, bootstrap_summary
    if args.cashstat:
        raise SystemExit("bootstrap refits use the LM driver: chi^2 or --poisson-mlr")
    limited = ~np.isnan(cfg.lower)
    lo = np.where(limited, cfg.lower - off, 0.0)
    hi = np.where(limited, cfg.upper - off, 0.0)
    seed = args.seed if args.seed > 0 else int(time.time())
    samples, status = bootstrap_errors(m, bestfit, args.bootstrap, seed, fixed=cfg.fixed, lower=lo, upper=hi,
                                       ftol=args.ftol, max_iter=args.max_iter)
    samples = samples + off
    bestfit = np.asarray(bestfit) + off
    if samples.shape[0] < 3:  # MIN_ITERATIONS_FOR_STATISTICS
        out.write(f"\nNot enough successful bootstrap iterations ({samples.shape[0]}) for meaningful "
                  "statistics!\n")
    else:
        out.write("\n".join(bootstrap_summary(bestfit, samples, cfg.param_names, cfg.fixed.astype(bool))) + "\n")
    if args.save_bootstrap:
        with open(args.save_bootstrap, "w") as f:
            f.write("\n".join(bootstrap_file_lines(cfg.functions, cfg.param_names, _NPARAMS, samples,
                                                   args.bootstrap)) + "\n")
    return samples, status


def flux_table(names, fluxes, total, zero_point=None, labels=None):
    """Lines of makeimage's component-flux table (core/makeimage_main.cpp:753-785):
    header, one line per function, an empty line, the total."""
    labels = labels or [""] * len(names)
    lines = ["Component                 Flux        Magnitude   Fraction   Label"]
    rows = [(n, f, f / total, lb) for n, f, lb in zip(names, fluxes, labels)] + [("Total", total, 1.0, "")]
    for k, (name, flux, frac, label) in enumerate(rows):
        if k == len(names):
            lines.append("")
        s = f"{name:<25s} {flux:10.4e}"
        s += f"   {zero_point - 2.5 * math.log10(flux):6.4f}" if zero_point is not None and flux > 0 \
            else "      ---"
        s += f"{frac:12.5f}" if frac >= 1e-4 or frac == 0.0 else f"{frac:12.3e}"
        if label:
            s += f"    {label}"
        lines.append(s)
    return lines


def makeimage(argv=None, out=sys.stdout):
    """The makeimage command; returns the model image (None when only fluxes
    were asked for) and the flux table (None when not asked for)."""
    args = build_makeimage_parser().parse_args(argv)
    try:
        cfg = read_config(args.config, check_limits=False)
    except ConfigError as e:
        raise SystemExit(f"error in {args.config}: {e}")
    fluxes_only = (args.print_fluxes or args.save_fluxes) and args.nosave
    ncols = args.ncols or int(float(cfg.options.get("NCOLS", 0)))
    nrows = args.nrows or int(float(cfg.options.get("NROWS", 0)))
    if not (ncols > 0 and nrows > 0):
        if args.refimage:
            nrows, ncols = fitsio.read_image(args.refimage)[0].shape
        elif not args.nosave:
            raise SystemExit("no image size: give --ncols and --nrows, or --refimage")
        else:
            ncols = nrows = 2  # fluxes only: the reference's minimal image
    m = ModelObject(args.device)
    _add_functions(m, cfg, args)
    _add_psf(m, args)
    m.setup_model_image(ncols, nrows)
    _add_oversampled_psfs(m, args)
    p = np.array(cfg.values, dtype=float)
    model = None
    if not fluxes_only:
        m.create_model_image(p)
        model = m.get_model_image()
        if not args.nosave:
            fitsio.write_image(args.output, model)
            out.write(f"saved {args.output} ({ncols} x {nrows})\n")
            if args.save_expanded:
                head, tail = os.path.split(args.output)
                fitsio.write_image(os.path.join(head, "expanded_" + tail), m.get_expanded_model_image())
            if args.output_functions:
                for k, (name, _) in enumerate(cfg.functions):
                    fitsio.write_image(f"{args.output_functions}{k + 1}_{name}.fits",
                                       m.get_single_function_image(p, k))
    table = None
    if args.print_fluxes or args.save_fluxes:
        total, ind = m.find_total_fluxes(p, args.estimation_size, args.estimation_size)
        table = flux_table([n for n, _ in cfg.functions], ind, total, args.zero_point, cfg.labels)
        if args.print_fluxes:
            out.write("\n".join(table) + "\n")
        if args.save_fluxes:
            with open(args.save_fluxes, "w") as f:
                f.write(f"# Fluxes estimated on {args.estimation_size} x {args.estimation_size} image\n")
                f.write("# " + table[0] + "\n" + "\n".join(table[1:]) + "\n")
    if args.timing > 0:
        t0 = time.perf_counter()
        for _ in range(args.timing):
            m.create_model_image(p)
        dt = (time.perf_counter() - t0) / args.timing
        out.write(f"mean time per image computation ({args.timing} iterations) = {dt:.7f} s\n")
    return model, table


def build_mcmc_parser():
    ap = build_parser()
    ap.prog = "imfit_gb300.cli mcmc"
    ap.description = "DREAM MCMC (imfit-mcmc) on the batched GPU statistic"
    ap.add_argument("-o", "--output", default="mcmc_out", help="root name of the chain files")
    ap.add_argument("--nchains", type=int, default=0)
    ap.add_argument("--max-chain-length", type=int, default=100000)
    ap.add_argument("--burnin-length", type=int, default=5000)
    ap.add_argument("--gelman-evals", type=int, default=5000)
    ap.add_argument("--gelman-rubin-limit", type=float, default=1.01)
    ap.add_argument("--uniform-offset", type=float, default=0.01)
    ap.add_argument("--gaussian-offset", type=float, default=1.0e-6)
    return ap


def mcmc(argv=None, out=sys.stdout):
    """The imfit-mcmc command (core/mcmc_main.cpp:150-460): chains written to
    OUTPUT.1.txt ... OUTPUT.<nchains>.txt; returns the sampler's result."""
    from .config import _NPARAMS
    from .solvers import chain_file_header, chain_file_row, dream
    args = build_mcmc_parser().parse_args(argv)
    try:
        cfg = read_config(args.config)
    except ConfigError as e:
        raise SystemExit(f"error in {args.config}: {e}")
    image = _read(args.image, "image")
    off, shift = _section_offsets(cfg, args.image)
    m = setup_model(cfg, args, image, shift)
    p0 = np.array(cfg.values, dtype=float) - off
    fixed = cfg.fixed.astype(bool)
    if np.any(np.isnan(cfg.lower[~fixed])):
        raise SystemExit("parameter limits must be supplied for all free parameters when using MCMC")
    head = chain_file_header(cfg.functions, cfg.param_names, _NPARAMS)
    files = []

    def write(t, states, liks, burn, pCR, accept):
        if not files:
            for i in range(states.shape[0]):
                f = open(f"{args.output}.{i + 1}.txt", "w")
                f.write(f"# imfit_gb300 mcmc, configuration file {args.config}, image {args.image}\n#\n")
                f.write("# Column Headers\n" + head + "\n")
                files.append(f)
        for i, f in enumerate(files):  # full-image coordinates, as PrintModelParamsHorizontalString writes
            f.write(chain_file_row(states[i] + off, liks[i], burn, pCR, accept[i]) + "\n")

    try:
        r = dream(m, p0, cfg.lower - off, cfg.upper - off, fixed=fixed, n_chains=args.nchains,
                  max_generations=args.max_chain_length, burn_in=args.burnin_length, gelman_evals=args.gelman_evals,
                  scale_reduction=args.gelman_rubin_limit, noise=args.uniform_offset, bstar=args.gaussian_offset,
                  seed=args.seed, callback=write)
    finally:
        for f in files:
            f.close()
    out.write(f"{r['generations']} generations of {r['n_chains']} chains, {r['evaluations']} likelihood "
              f"evaluations; {'converged' if r['converged'] else 'maximum chain length reached'}\n")
    out.write(f"chains written to {args.output}.1.txt through {args.output}.{r['n_chains']}.txt\n")
    return r


def build_multimfit_parser():
    ap = argparse.ArgumentParser(prog="imfit_gb300.cli multimfit",
                                 description="simultaneous fit of several images (multimfit)")
    ap.add_argument("config")
    ap.add_argument("-i", "--image-info", required=True)
    ap.add_argument("--nosubsampling", "--no-subsampling", dest="nosubsampling", action="store_true")
    ap.add_argument("--cashstat", action="store_true")
    ap.add_argument("--poisson-mlr", "--mlr", dest="poisson_mlr", action="store_true")
    ap.add_argument("--model-errors", action="store_true")
    ap.add_argument("--fitstat-only", "--chisquare-only", dest="fitstat_only", action="store_true")
    ap.add_argument("--nm", action="store_true")
    ap.add_argument("--de", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--ftol", type=float, default=1e-8)
    ap.add_argument("--max-iter", type=int, default=0)
    ap.add_argument("--device", type=int, default=0)
    return ap


def multimfit(argv=None, out=sys.stdout):
    """The multimfit command (core/multimfit_main.cpp): the configuration file
    gives the model, the image-info file the images and their description
    parameters; returns (fitted global parameters, statistic)."""
    from .multimage import (IMAGE_PARAM_NAMES, MultiImageModel, build_handles, global_vector, parse_image_info,
                            section_offsets)
    args = build_multimfit_parser().parse_args(argv)
    try:
        cfg = read_config(args.config)
    except ConfigError as e:
        raise SystemExit(f"error in {args.config}: {e}")
    with open(args.image_info) as f:
        images = parse_image_info(f.read())
    stat = "cash" if args.cashstat else ("pmlr" if args.poisson_mlr else "chi2")
    handles = build_handles(cfg.functions, images, args.device, not args.nosubsampling, stat, args.model_errors)
    mm = MultiImageModel(cfg.functions, handles, [im.local_functions for im in images])
    p0, lo, hi, fx = global_vector(cfg, images)
    off = section_offsets(cfg, images)  # image sections: X0/Y0 in the sections' pixel frames
    p0, lo, hi = p0 - off, lo - off, hi - off
    if args.fitstat_only:
        # PrintFitStatistic (core/multimfit_main.cpp:686-692 -> core/print_results.cpp:160-181),
        # the valid pixels summed over the images
        s = mm.get_fit_statistic(p0)
        n_free = int(np.sum(fx == 0))
        n_valid = int(sum(h.n_valid for h in handles))
        out.write("\n" + "\n".join(fit_statistic_lines(s, stat, n_free, n_valid)) + "\n\n")
        return p0 + off, s
    if args.de:
        from .solvers import differential_evolution
        r = differential_evolution(mm, p0, lo, hi, fixed=fx.astype(bool), ftol=args.ftol, seed=args.seed)
    elif args.nm:
        from .solvers import nelder_mead
        r = nelder_mead(mm, p0, np.where(np.isnan(lo), -np.inf, lo), np.where(np.isnan(hi), np.inf, hi),
                        fixed=fx.astype(bool), ftol=args.ftol)
    else:
        if args.cashstat:
            raise SystemExit("the Cash statistic has no deviates: use --nm or --de")
        r = mm.fit_lm(p0, fixed=fx, lower=np.where(np.isnan(lo), 0.0, lo), upper=np.where(np.isnan(hi), 0.0, hi),
                      ftol=args.ftol, max_iter=args.max_iter)
    s = mm.get_fit_statistic(r["params"])
    p = r["params"] + off  # reported in the full images' pixel frames
    out.write(f"fit statistic = {s:.6f}\n# Main model parameters (reference image)\n")
    for name, v in zip(cfg.param_names, p[mm.n_image_params:]):
        out.write(f"  {name:8s} {v:.6f}\n")
    for i in range(1, mm.n_images):
        out.write(f"# Image-description parameters for image {i + 1}\n")
        for j, name in enumerate(IMAGE_PARAM_NAMES):
            out.write(f"  {name:12s} {p[5 * (i - 1) + j]:.6f}\n")
    for i, im in enumerate(images):
        if im.local is not None:
            out.write(f"# Per-image function parameters for image {i + 1}\n")
            for name, v in zip(im.local.param_names, p[mm.local_slice(i)]):
                out.write(f"  {name:8s} {v:.6f}\n")
    return p, s


def makemultimages(argv=None, out=sys.stdout):
    """The makemultimages command (core/makemultimages_main.cpp): the model of
    the configuration file seen through each image of an image-info file
    (NCOLS/NROWS, optional PSF, image-description parameters), saved as
    OUTPUT_0.fits, OUTPUT_1.fits, ...; returns the images."""
    from .multimage import MultiImageModel, global_vector, parse_image_info
    ap = argparse.ArgumentParser(prog="imfit_gb300.cli makemultimages")
    ap.add_argument("config")
    ap.add_argument("-i", "--image-info", required=True)
    ap.add_argument("-o", "--output", default="modelimage_multi")
    ap.add_argument("--nosubsampling", "--no-subsampling", dest="nosubsampling", action="store_true")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    try:
        cfg = read_config(args.config, check_limits=False)
    except ConfigError as e:
        raise SystemExit(f"error in {args.config}: {e}")
    with open(args.image_info) as f:
        images = parse_image_info(f.read())
    handles = []
    for im in images:
        m = ModelObject(args.device)
        # global functions, then the image's own (core/makemultimages_main.cpp:266-300)
        for name, new_set in list(cfg.functions) + im.local_functions:
            m.add_function(name, new_set, subsampling=not args.nosubsampling)
        m.finish_functions()
        if im.psf:
            m.add_psf(fitsio.read_image(im.psf)[0])
        nc, nr = int(float(im.options.get("NCOLS", 0))), int(float(im.options.get("NROWS", 0)))
        if not (nc > 0 and nr > 0):
            if not im.data:
                raise SystemExit("an image needs NCOLS and NROWS (or a DATA image for its size)")
            nr, nc = fitsio.read_image(im.data)[0].shape
        m.setup_model_image(nc, nr)
        handles.append(m)
    mm = MultiImageModel(cfg.functions, handles, [im.local_functions for im in images])
    p, _, _, _ = global_vector(cfg, images)
    outs = []
    for i, m in enumerate(handles):
        m.create_model_image(mm.image_vector(p, i))
        img = m.get_model_image()
        fitsio.write_image(f"{args.output}_{i}.fits", img)
        outs.append(img)
    out.write(f"saved {len(outs)} model images as {args.output}_0.fits ... {args.output}_{len(outs) - 1}.fits\n")
    return outs


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if argv and argv[0] == "makeimage":
        makeimage(argv[1:])
    elif argv and argv[0] == "mcmc":
        mcmc(argv[1:])
    elif argv and argv[0] == "multimfit":
        multimfit(argv[1:])
    elif argv and argv[0] == "makemultimages":
        makemultimages(argv[1:])
    else:
        run(argv)


if __name__ == "__main__":
    main()
