"""Generate the committed golden fixtures from the reference.

Run where the reference checkout is present (IMFIT_REFERENCE_DIR, else the
oracle build recipe's REFDIR):  python tests/golden/make_golden.py [part ...]
(parts: n3073 makeimage ic3478 pointsource mcmc multimfit makemultimages small_case
imfit_regressions bench_sizes los3d; all by default)

Outputs (all small .npz files next to this script):
  n3073.npz          the reference regression inputs tests/n3073rss_small.fits,
                     tests/n3073rss_small_mask.fits, tests/psf_moffat_35_n4699z.fits
                     (float32 / int, exactly as stored), the printed goldens of
                     tests/imfit_reference/imfit_textout4c:24 and imfit_textout4d,
                     the full-precision values from the reference's own code
                     compiled here (oracle/_ref), and its mpfit LM fit.
  makeimage.npz      reference makeimage outputs tests/sersic+exp_orig.fits
                     (central 128x128 crop and four 16x16 corners),
                     tests/oversampled_orig.fits and oversampled2both_orig.fits
                     with their PSFs, tests/biggertest_orig.fits, and the
                     configurations of the last two (do_makeimage_tests:48,
                     51, 68-72).
  ic3478.npz         the reference regression input tests/ic3478rss_64x64.fits
                     (float32 as stored) with the configuration
                     tests/imfit_reference/imfit_config_ic3478_64x64b.dat and the
                     printed results of its mpfit fit (imfit_textout3) and its
                     Differential Evolution fit (imfit_textout3c_tail).
  pointsource.npz    unit_tests/psf_gauss_sigma0.5_5.fits (the PSF of
                     unittest_psf_interpolators.t.h) and the makeimage output
                     tests/oversampled_pointsource.fits (do_makeimage_tests:74).
  mcmc.npz           tests/faintstar.fits with
                     tests/imfit-mcmc_reference/config_imfit_faintstar.dat, and
                     summaries of the reference's DREAM chain 1 for it
                     (tests/imfit-mcmc_reference/mcmc_ref1.1.txt_skip3,
                     do_mcmc_tests:27): post-burn-in means, standard deviations
                     and 16/50/84 % quantiles per parameter, the number of
                     rows and the burn-in rows.
  multimfit.npz      tests/multimfit_reference/smallgauss_5x5_{0,1,sigma}.fits and
                     smallDataImage1{a,b}.fits with the printed results of
                     multimfit_textout3a (Nelder-Mead fit of
                     config_imfit_smallgauss.dat + imageinfo_multimfit3.txt) and
                     multimfit_textout1a (--fitstat-only, imageinfo_multimfit0.txt);
                     the configurations, image-info files and printed results
                     of multimfit_textout1b-1e and 3b-3f (do_multimfit_tests.sh:61-92:
                     Nelder-Mead and LM fits, limits on the image-description
                     parameters, image sections, no error images, model errors).
  makemultimages.npz the makemultimages outputs tests/makemultimages_reference/
                     multimagetest_{0,1,2,2b,2c,2d}.fits and multimagetest_2blocks_0 /
                     _offset_1 / _offset_2.fits (do_makemultimages_tests.sh:59-65),
                     64 x 64 each.
  small_case.npz     the reference's own outputs (oracle/_ref) for
                     imfit_gb300.workloads.small_case: model images, deviates and
                     statistics for chi^2 / Cash / PMLR.
  imfit_regressions.npz
                     inputs (images as stored, configuration files as text) and
                     printed results of the reference's imfit regression runs
                     do_imfit_tests:66, 87, 89, 97, 121-124, 147-162, 165-178
                     (imfit_textout2, 3e, 3e2, 4b, 5a/5b/5c_tail, 6, 6b-6h,
                     7a-7f, 8a; the linux_x86_64 copies where the reference keeps
                     per-platform outputs): per case the command's options, the
                     best-fit values and printed errors, the printed statistic
                     (or the one implied by the printed AIC), AIC, BIC, and the
                     error line of the runs that stop with an error; and the
                     saved bootstrap iterations of --seed 10 --bootstrap 5 on
                     ic3478rss_64x64.fits and its section [10:64,10:64]
                     (do_imfit_tests:133-134, bootstrap_output_seed10*_tail.dat).
  bench_sizes.npz    the reference's own values (oracle/_ref) for the benchmark
                     configurations C1-C4 at their full sizes (tests/bench_cases.py):
                     a digest of the synthesized data, and per parameter vector
                     the fit statistic and the model image's row sums, column
                     sums and a fixed sample of 512 pixels.
  los3d.npz          the reference's own values for a 96x96 ExponentialDisk3D +
                     FerrersBar3D model (the C3 workload at 96 px, 15x15 PSF):
                     the data, the model image without and with the PSF, and
                     the chi^2 at the true and start vectors.
"""
import re
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from imfit_gb300 import fits, workloads  # noqa: E402

REF = oracle.REFERENCE_DIR


def n3073():
    t = os.path.join(REF, "tests")
    data, _ = fits.read_image(os.path.join(t, "n3073rss_small.fits"))
    mask, _ = fits.read_image(os.path.join(t, "n3073rss_small_mask.fits"))
    psf, _ = fits.read_image(os.path.join(t, "psf_moffat_35_n4699z.fits"))
    # tests/imfit_reference/imfit_config_n3073.dat
    params = np.array([101.0, 97.0, 110.0, 0.2, 1.5, 150.0, 15.0, 55.0, 0.2, 70.0, 45.0])
    lo = np.array([90, 90, 0, 0, 0, 0, 0, 0, 0, 0, 0], dtype=float)
    hi = np.array([110, 110, 180, 1, 5, 500, 100, 90, 1, 600, 1000], dtype=float)
    out = {}
    for stat in ("chi2", "cash"):
        m = oracle.RefModel()
        m.add_function("Sersic", True)
        m.add_function("Exponential")
        m.finish_functions()
        m.add_psf(psf)
        m.add_image_data(data)
        m.add_image_characteristics(4.725, 4.3, 1.0, 1, 154.33)
        m.add_mask_vector(mask)
        if stat == "cash":
            m.use_cash()
        assert m.final_setup() == 0
        out[f"{stat}_ref"] = m.get_fit_statistic(params)
        if stat == "chi2":
            out["deviates_ref"] = m.compute_deviates(params)
            fit = m.lm_fit(params, lo=lo, hi=hi, ftol=1e-8, maxiter=10000)
            out["lm_params"] = fit["params"]
            out["lm_chi2"] = fit["chi2"]
            out["lm_niter"] = fit["niter"]
            out["lm_nfev"] = fit["nfev"]
    np.savez_compressed(os.path.join(HERE, "n3073.npz"), data=data.astype(np.float32),
                        mask=mask.astype(np.int16), psf=psf.astype(np.float32), params=params, lo=lo, hi=hi,
                        gain=4.725, read_noise=4.3, original_sky=154.33,
                        chi2_printed=235606.146670, cash_printed=-305659765.743167,
                        lm_chi2_printed=36828.577653, **out)


def makeimage():
    t = os.path.join(REF, "tests")
    se, _ = fits.read_image(os.path.join(t, "sersic+exp_orig.fits"))
    ov, _ = fits.read_image(os.path.join(t, "oversampled_orig.fits"))
    psf_std, _ = fits.read_image(os.path.join(t, "psf_standard.fits"))
    psf_os, _ = fits.read_image(os.path.join(t, "psf_oversamp.fits"))
    ov2, _ = fits.read_image(os.path.join(t, "oversampled2both_orig.fits"))
    big, _ = fits.read_image(os.path.join(t, "biggertest_orig.fits"))
    mref = os.path.join(t, "makeimage_reference")
    np.savez_compressed(
        os.path.join(HERE, "makeimage.npz"),
        # do_makeimage_tests:48 (--ncols 64 --nrows 64) and :70-72 (two oversampled
        # regions, one PSF image for both or one each): configurations as text
        big_config=np.array(open(os.path.join(mref, "config_biggertest_4c.dat")).read()),
        big_image=big.astype(np.float32),
        ov2_config=np.array(open(os.path.join(mref, "config_makeimage_gauss-oversample2.dat")).read()),
        ov2_image=ov2.astype(np.float32),
        # tests/makeimage_reference/config_makeimage_sersic+exp512.dat
        se_params=np.array([256.0, 256.0, 30.0, 0.5, 2.5, 100.0, 50.0, 30.0, 0.75, 10.0, 150.0]),
        se_center=se[192:320, 192:320].astype(np.float32),
        se_corners=np.stack([se[:16, :16], se[:16, -16:], se[-16:, :16], se[-16:, -16:]]).astype(np.float32),
        # tests/makeimage_reference/config_makeimage_gauss-oversample.dat
        ov_params=np.array([105.2377, 105.4582, 0.0, 0.0, 99.8787, 1.20062]),
        ov_image=ov.astype(np.float32), psf_standard=psf_std.astype(np.float32),
        psf_oversamp=psf_os.astype(np.float32), ov_region=np.array([100, 110, 100, 110]), ov_scale=3)


def ic3478():
    t = os.path.join(REF, "tests")
    data, _ = fits.read_image(os.path.join(t, "ic3478rss_64x64.fits"))
    np.savez_compressed(
        os.path.join(HERE, "ic3478.npz"), data=data.astype(np.float32),
        gain=4.725, read_noise=4.3, original_sky=130.1,
        # X0 Y0 PA ell n I_e r_e and their limits
        params=np.array([32.0, 32.0, 18.0, 0.2, 1.5, 15.0, 25.0]),
        lo=np.array([1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0]),
        hi=np.array([64.0, 64.0, 90.0, 1.0, 5.0, 500.0, 100.0]),
        # imfit_textout3: CHI-SQUARE, reduced chi^2, best-fit values and errors
        lm_chi2_printed=4555.947654, lm_reduced_printed=1.114196,
        lm_params_printed=np.array([32.9439, 34.0933, 18.2612, 0.235989, 2.40028, 20.0094, 60.7612]),
        lm_errors_printed=np.array([0.0128, 0.0156, 0.30986, 0.0023165, 0.018072, 0.40396, 0.86063]),
        # imfit_textout3c_tail: the same fit with --de
        de_reduced_printed=1.114196,
        de_params_printed=np.array([32.9439, 34.0933, 18.2613, 0.235989, 2.40028, 20.0094, 60.7612]))


def pointsource():
    psf5, _ = fits.read_image(os.path.join(REF, "unit_tests", "psf_gauss_sigma0.5_5.fits"))
    img, _ = fits.read_image(os.path.join(REF, "tests", "oversampled_pointsource.fits"))
    np.savez_compressed(os.path.join(HERE, "pointsource.npz"), psf5=psf5.astype(np.float32),
                        ps_image=img.astype(np.float32),
                        # config_makeimage_pointsource-oversample.dat: X0 Y0 I_tot
                        ps_params=np.array([100.0, 100.0, 1.0]), ps_region=np.array([80, 120, 80, 120]),
                        ps_scale=3)


def mcmc():
    t = os.path.join(REF, "tests")
    data, _ = fits.read_image(os.path.join(t, "faintstar.fits"))
    rows = np.loadtxt(os.path.join(t, "imfit-mcmc_reference", "mcmc_ref1.1.txt_skip3"), comments="#")
    post = rows[rows[:, 7] == 0][:, :6]
    np.savez_compressed(
        os.path.join(HERE, "mcmc.npz"), data=data.astype(np.float32), gain=4.72, read_noise=1.15,
        original_sky=124.94,
        # X0 Y0 PA ell I_0 sigma with their limits
        params=np.array([5.0, 6.0, 155.0, 0.1, 250.0, 1.0]),
        lo=np.array([3.0, 3.0, 140.0, 0.0, 220.0, 0.1]), hi=np.array([8.0, 8.0, 170.0, 0.3, 320.0, 1.5]),
        ref_rows=rows.shape[0], ref_burn_rows=int(np.sum(rows[:, 7] == 1)),
        ref_mean=post.mean(axis=0), ref_std=post.std(axis=0, ddof=1),
        ref_q=np.percentile(post, [16, 50, 84], axis=0), ref_best_loglik=rows[:, 6].max())


def multimfit():
    t = os.path.join(REF, "tests", "multimfit_reference")
    r = lambda n: fits.read_image(os.path.join(t, n))[0].astype(np.float32)
    np.savez_compressed(
        os.path.join(HERE, "multimfit.npz"), g0=r("smallgauss_5x5_0.fits"), g1=r("smallgauss_5x5_1.fits"),
        gsig=r("smallgauss_5x5_sigma.fits"), d1a=r("smallDataImage1a.fits"), d1b=r("smallDataImage1b.fits"),
        # multimfit_textout3a: CHI-SQUARE and the printed parameters (X0 Y0 PA ell I_0 sigma; image 2 X0 Y0)
        g_chi2_printed=36.070608, g_model_printed=np.array([2.5072, 2.5387, 18.9357, 0.293283, 995.047, 0.992441]),
        g_image2_printed=np.array([2.49082, 2.47557]),
        # multimfit_textout1a: CHI-SQUARE at the starting parameters
        d_chi2_printed=6.75, **_multimfit_cases(t))


# do_multimfit_tests.sh:61-92: (case, configuration, image-info file, options); the
# reference keeps 1b and 3f only as macOS printouts (macos_x86_64/)
MULTIMFIT_CASES = [
    ("1b", "config_imfit_smalldataimages.dat", "imageinfo_multimfit0.txt", []),
    ("1c", "config_imfit_smalldataimages.dat", "imageinfo_multimfit0.txt", ["--nm"]),
    ("1d", "config_imfit_smalldataimages_with-limits.dat", "imageinfo_multimfit0.txt", []),
    ("1e", "config_imfit_smalldataimages.dat", "imageinfo_multimfit0_with-limits.txt", []),
    ("3b", "config_imfit_smallgauss.dat", "imageinfo_multimfit3b.txt", ["--nm"]),
    ("3c", "config_imfit_smallgauss.dat", "imageinfo_multimfit3c.txt", ["--nm"]),
    ("3d", "config_imfit_smallgauss.dat", "imageinfo_multimfit3_noerror.txt", ["--nm"]),
    ("3e", "config_imfit_smallgauss.dat", "imageinfo_multimfit3_noerror.txt", ["--nm", "--model-errors"]),
    ("3f", "config_imfit_smallgauss.dat", "imageinfo_multimfit3_noerror.txt", ["--mlr"]),
]


def _multimfit_cases(t):
    """Configurations and image-info files as text, and the printed CHI-SQUARE
    and parameter values (model first, then image 2's description
    parameters, as multimfit prints them) of multimfit_textout<case>."""
    out = {"cases": np.array([c[0] for c in MULTIMFIT_CASES])}
    for case, cfg, info, opts in MULTIMFIT_CASES:
        name = f"multimfit_textout{case}"
        if not os.path.exists(os.path.join(t, name)):
            name = os.path.join("macos_x86_64", name)
        r = _parse_textout(os.path.join(t, name))
        out[f"{case}__config"] = np.array(open(os.path.join(t, cfg)).read())
        out[f"{case}__info"] = np.array(open(os.path.join(t, info)).read())
        out[f"{case}__options"] = np.array(opts if opts else [""])
        out[f"{case}__names"] = np.array(r["names"])
        out[f"{case}__values"] = np.array(r["values"])
        out[f"{case}__stat"] = np.float64(r["stat"])
    return out


def makemultimages():
    t = os.path.join(REF, "tests", "makemultimages_reference")
    names = {"img_0": "multimagetest_0", "img_1": "multimagetest_1", "img_2": "multimagetest_2",
             "img_2b": "multimagetest_2b", "img_2c": "multimagetest_2c", "img_2d": "multimagetest_2d",
             "blk_0": "multimagetest_2blocks_0", "blk_1": "multimagetest_2blocks_offset_1",
             "blk_2": "multimagetest_2blocks_offset_2"}
    out = {k: fits.read_image(os.path.join(t, v + ".fits"))[0].astype(np.float32) for k, v in names.items()}
    np.savez_compressed(os.path.join(HERE, "makemultimages.npz"), **out)


def small_case():
    out = {}
    for stat in ("chi2", "cash", "pmlr"):
        wl = workloads.small_case(stat=stat)
        workloads.synthesize(wl, oracle.RefModel)
        m = workloads.configure(oracle.RefModel(), wl)
        out[f"{stat}_data"] = wl.data
        for tag, p in (("truth", wl.truth), ("start", wl.start)):
            out[f"{stat}_{tag}_stat"] = m.get_fit_statistic(p)
            out[f"{stat}_{tag}_dev"] = m.compute_deviates(p)
            out[f"{stat}_{tag}_model"] = m.get_model_image()
    np.savez_compressed(os.path.join(HERE, "small_case.npz"), **out)


def bench_sizes():
    sys.path.insert(0, os.path.dirname(HERE))
    import bench_cases
    out = {}
    for name in bench_cases.NAMES:
        wl = bench_cases.build(name)
        out[f"{name}_data"] = bench_cases.data_digest(wl)
        m = workloads.configure(oracle.RefModel(), wl)
        for tag, p in bench_cases.vectors(wl):
            out[f"{name}_{tag}_params"] = np.asarray(p, dtype=np.float64)
            out[f"{name}_{tag}_stat"] = m.get_fit_statistic(p)
            rows, cols, sample = bench_cases.digest(m.get_model_image())
            out[f"{name}_{tag}_rows"] = rows
            out[f"{name}_{tag}_cols"] = cols
            out[f"{name}_{tag}_sample"] = sample
    np.savez_compressed(os.path.join(HERE, "bench_sizes.npz"), **out)


def los3d():
    wl = workloads.c3(size=96, psf_size=15)
    workloads.synthesize(wl, oracle.RefModel)
    out = {"data": wl.data, "truth": wl.truth, "start": wl.start, "psf": wl.psf}
    nopsf = workloads.c3(size=96, psf_size=15)
    nopsf.psf = None
    m0 = workloads.configure(oracle.RefModel(), nopsf, with_data=False)
    m = workloads.configure(oracle.RefModel(), wl)
    for tag, p in (("truth", wl.truth), ("start", wl.start)):
        m0.create_model_image(p)
        out[f"{tag}_model_nopsf"] = m0.get_model_image()
        out[f"{tag}_stat"] = m.get_fit_statistic(p)
        out[f"{tag}_model"] = m.get_model_image()
    np.savez_compressed(os.path.join(HERE, "los3d.npz"), **out)


# (case, configuration, image, options with fixture file names, printed output)
REGRESSIONS = [
    ("2", "imfit_config_ic3478_64x64.dat", "ic3478rss_64x64.fits", ["--gain=4.725", "--readnoise=4.3", "--sky=130.1"],
     "linux_x86_64/imfit_textout2"),
    ("3e", "imfit_config_ic3478_64x64c.dat", "ic3478rss_64x64.fits", ["--noise=ic3478rss_64x64_sigma.fits"],
     "linux_x86_64/imfit_textout3e"),
    ("3e2", "imfit_config_ic3478_64x64c.dat", "ic3478rss_64x64.fits",
     ["--noise=ic3478rss_64x64_variance.fits", "--errors-are-variances"], "linux_x86_64/imfit_textout3e2"),
    ("4b", "imfit_config_n3073.dat", "n3073rss_small_cps.fits",
     ["--mask", "n3073rss_small_mask.fits", "--psf", "psf_moffat_35_n4699z.fits", "--exptime=53.907456",
      "--sky=2.8628692847238053"], "linux_x86_64/imfit_textout4b"),
    ("5a", "config_imfit_poisson.dat", "testimage_poisson_lowsn20.fits", ["--cashstat", "--nm"],
     "imfit_textout5a_tail"),
    ("5b", "config_imfit_poisson.dat", "testimage_poisson_lowsn20.fits", ["--mlr", "--nm"], "imfit_textout5b_tail"),
    ("5c", "config_imfit_poisson.dat", "testimage_poisson_lowsn20.fits", ["--mlr"], "imfit_textout5c_tail"),
    ("6", "imfit_config_ic3478_64x64b.dat", "ic3478rss_64x64.fits", ["--mask", "totalmask_64x64.fits"],
     "imfit_textout6"),
    ("6b", "imfit_config_ic3478_64x64b.dat", "ic3478rss_64x64.fits", ["--mask", "n3073rss_small_mask.fits"],
     "imfit_textout6b"),
    ("6c", "imfit_config_ic3478_64x64b.dat", "test_emptyhdu.fits", [], "imfit_textout6c"),
    ("6d", "imfit_config_ic3478_64x64b.dat", "test_table.fits", [], "imfit_textout6d"),
    ("6e", "imfit_config_ic3478_64x64b.dat", "ic3478rss_64x64.fits", ["--mask", "test_emptyhdu.fits"],
     "imfit_textout6e"),
    ("6f", "imfit_config_ic3478_64x64b.dat", "test_multiextension_hdu0empty.fits[0]", [], "imfit_textout6f"),
    ("6g", "config_imfit_small-gaussian.dat", "test_multiextension_hdu0empty.fits[1]", [], "imfit_textout6g"),
    ("6h", "config_imfit_small-gaussian.dat", "test_multiextension_hdu0empty.fits[1][1:8,1:8]", [],
     "imfit_textout6h"),
    ("7a", "config_3x3_flatsky.dat", "testimage_3x3_nan.fits", [], "imfit_textout7a"),
    ("7b", "config_3x3_flatsky.dat", "testimage_3x3_ones.fits", ["--mask=testimage_3x3_mask-with-nan.fits"],
     "imfit_textout7b"),
    ("7c", "config_3x3_flatsky.dat", "testimage_3x3_ones.fits", ["--noise=testimage_3x3_nan.fits"],
     "imfit_textout7c"),
    ("7d", "config_3x3_flatsky.dat", "testimage_3x3_onezero.fits", [], "imfit_textout7d"),
    ("7e", "config_3x3_flatsky.dat", "testimage_3x3_onezero.fits", ["--mask=mask_for_onezero.fits"],
     "imfit_textout7e"),
    ("7f", "config_imfit_2gauss_small.dat", "testimage_2gauss_psf.fits", ["--nm"], "imfit_textout7f"),
    ("8a", "config_imfit_ptsource.dat", "psf_moffat_fwhm2.fits", ["--psf=psf_moffat_fwhm2_35x35.fits"],
     "linux_x86_64/imfit_textout8a"),
]


# regression inputs whose HDU layout matters (an empty primary HDU, a table)
RAW_FILES = {"test_emptyhdu.fits", "test_table.fits", "test_multiextension_hdu0empty.fits"}


def _parse_textout(path):
    """Printed statistic, AIC, BIC, parameter names / values / errors (NaN
    where none is printed) and the first ERROR line of an imfit printout."""
    lines = open(path).read().splitlines()
    res = dict(stat=np.nan, aic=np.nan, bic=np.nan, names=[], values=[], errors=[], error="")
    start = None
    for k, ln in enumerate(lines):
        m = re.match(r"\s*(CHI-SQUARE|CASH STATISTIC|POISSON-MLR STATISTIC) = (\S+)", ln)
        if m:
            res["stat"] = float(m.group(2))
        m = re.match(r"AIC = (\S+), BIC = (\S+)", ln)
        if m:
            res["aic"], res["bic"], start = float(m.group(1)), float(m.group(2)), k
        if "ERROR" in ln and not res["error"]:
            res["error"] = ln.strip()
    if start is not None:
        for ln in lines[start + 1:]:
            if ln.startswith("Saving") or ln.startswith("(Elapsed"):
                break
            t = ln.split()
            if not t or t[0] == "FUNCTION" or t[0].startswith("#"):
                continue
            res["names"].append(t[0])
            res["values"].append(float(t[1]))
            res["errors"].append(float(t[4]) if len(t) > 4 and t[2:4] == ["#", "+/-"] else np.nan)
    return res


def imfit_regressions():
    t = os.path.join(REF, "tests")
    cfg_dir = os.path.join(t, "imfit_reference")
    out = {"cases": np.array([c[0] for c in REGRESSIONS])}
    files = set()
    for case, cfg, img, opts, textout in REGRESSIONS:
        out[f"config__{cfg}"] = np.array(open(os.path.join(cfg_dir, cfg)).read())
        files.add(img.split("[")[0])
        for o in opts:
            v = o.split("=", 1)[1] if "=" in o else o
            if v.endswith(".fits"):
                files.add(v)
        r = _parse_textout(os.path.join(cfg_dir, textout))
        out[f"{case}__config"] = np.array(cfg)
        out[f"{case}__image"] = np.array(img)
        out[f"{case}__options"] = np.array(opts if opts else [""])
        out[f"{case}__names"] = np.array(r["names"] if r["names"] else [""])
        out[f"{case}__values"] = np.array(r["values"], dtype=float)
        out[f"{case}__errors"] = np.array(r["errors"], dtype=float)
        for k in ("stat", "aic", "bic"):
            out[f"{case}__{k}"] = np.float64(r[k])
        out[f"{case}__error"] = np.array(r["error"])
    # bootstrap refits with --seed 10 --bootstrap 5 on the whole image and on
    # its section [10:64,10:64] (do_imfit_tests:133-134, 312-323): the last 7
    # lines of the saved iterations
    for key, name in (("full", "bootstrap_output_seed10_tail.dat"), ("section", "bootstrap_output_seed10_2_tail.dat")):
        lines = open(os.path.join(cfg_dir, "linux_x86_64", name)).read().splitlines()
        out[f"boot__{key}__header"] = np.array(lines[:2])
        out[f"boot__{key}__rows"] = np.array([[float(v) for v in ln.split()] for ln in lines[2:]])
    out["config__imfit_config_ic3478_64x64b.dat"] = np.array(
        open(os.path.join(cfg_dir, "imfit_config_ic3478_64x64b.dat")).read())
    for f in sorted(files):
        if f in RAW_FILES:  # several HDUs, kept byte for byte
            out[f"raw__{f}"] = np.frombuffer(open(os.path.join(t, f), "rb").read(), dtype=np.uint8)
            continue
        data, hdr = fits.read_image(os.path.join(t, f))
        # float32 images as stored; integer masks and float64 images as float64
        out[f"file__{f}"] = data.astype(np.float32) if int(hdr["BITPIX"]) == -32 else data
    np.savez_compressed(os.path.join(HERE, "imfit_regressions.npz"), **out)


if __name__ == "__main__":
    if not os.path.isdir(os.path.join(REF, "core")):
        sys.exit(f"reference checkout not found at {REF}")
    oracle.build_reference()
    parts = {"n3073": n3073, "makeimage": makeimage, "ic3478": ic3478, "pointsource": pointsource,
             "mcmc": mcmc, "multimfit": multimfit, "makemultimages": makemultimages, "small_case": small_case,
             "imfit_regressions": imfit_regressions, "bench_sizes": bench_sizes, "los3d": los3d}
    for name in (sys.argv[1:] or parts):
        parts[name]()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
