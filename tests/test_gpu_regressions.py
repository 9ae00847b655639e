"""The reference's imfit regression runs (do_imfit_tests:66, 87, 89, 97,
121-124, 133-134, 147-162, 165-178) through the imfit-style command line on the GPU,
against the printed outputs held in tests/golden/imfit_regressions.npz
(imfit_textout2, 3e, 3e2, 4b, 5a-5c, 6, 6b-6h, 7a-7f, 8a):

* Levenberg-Marquardt runs: best-fit values within 0.05 of the printed
  one-sigma errors (plus the printing's rounding), the statistic to its six
  printed decimals, AIC and BIC as printed, and the parameter errors within
  1 % of mpfit's (0 where mpfit reports 0: fixed, pegged at a limit, or
  without influence on the model);
* Nelder-Mead runs (the reference's NLopt simplex, stood in by scipy's): the
  same minimum -- statistic within 2e-7 relative, values within 0.1 sigma
  (sigma from an LM fit of the same case);
* runs the reference stops with an error stop here with the same error."""
import io
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
D = np.load(os.path.join(GOLDEN, "imfit_regressions.npz"))

LM_CASES = ["2", "3e", "3e2", "4b", "5c", "6g", "6h", "7a", "7b", "7c", "7e", "8a"]
NM_CASES = ["5a", "5b", "7f"]
ERROR_CASES = {"6": "Failure in ModelObject::FinalSetupForFitting!",
               "6b": "Dimensions of mask image",
               "6c": "Unable to read image file",
               "6d": "Unable to read image file",
               "6e": "Unable to read mask file",
               "6f": "Unable to read image file",
               "7d": "Failure in ModelObject::FinalSetupForFitting!"}


def _args(tmp_path, case, drop=()):
    """The case's command line with its fixture files written to tmp_path."""
    from imfit_gb300 import fits

    def path(name):
        base, suffix = name.split("[")[0], name[len(name.split("[")[0]):]  # HDU / section suffix
        out = tmp_path / base
        if not out.exists():
            if f"raw__{base}" in D.files:
                out.write_bytes(D[f"raw__{base}"].tobytes())
            else:
                arr = D[f"file__{base}"]
                fits.write_image(str(out), arr, bitpix=-32 if arr.dtype == np.float32 else -64)
        return str(out) + suffix

    cfg = str(D[f"{case}__config"])
    (tmp_path / cfg).write_text(str(D[f"config__{cfg}"]))
    args = [str(tmp_path / cfg), path(str(D[f"{case}__image"]))]
    for o in (str(x) for x in D[f"{case}__options"]):
        if not o or o in drop:
            continue
        if "=" in o and o.endswith(".fits"):
            k, v = o.split("=", 1)
            args.append(f"{k}={path(v)}")
        elif o.endswith(".fits"):
            args.append(path(o))
        else:
            args.append(o)
    return args


def _printed(case):
    v, e = D[f"{case}__values"], D[f"{case}__errors"]
    stat = float(D[f"{case}__stat"])
    return v, e, stat, float(D[f"{case}__aic"]), float(D[f"{case}__bic"])


def _stat_from_aic(aic, k, n):
    return aic - 2.0 * k - 2.0 * k * (k + 1.0) / (n - k - 1.0)


@pytest.mark.parametrize("case", LM_CASES)
def test_lm_runs_match_printed_results(gpu, tmp_path, case):
    from imfit_gb300 import cli
    det = {}
    p, s = cli.run(_args(tmp_path, case), out=io.StringIO(), details=det)
    v, e, stat, aic, bic = _printed(case)
    if np.isnan(stat):
        stat = _stat_from_aic(aic, det["n_free"], det["n_valid"])
    assert abs(s - stat) <= 2e-7 * abs(stat) + 1e-6, (s, stat)
    assert abs(det["aic"] - aic) <= 2e-7 * abs(aic) + 2e-6 and abs(det["bic"] - bic) <= 2e-7 * abs(bic) + 2e-6
    rounding = 1e-5 * np.abs(v) + 1e-12
    assert np.all(np.abs(p - v) <= 0.05 * e + rounding), list(zip(p, v, e))
    err = det["errors"]
    assert err is not None
    assert np.all(np.abs(err - e) <= 0.01 * e + 1e-5 * np.abs(e) + 1e-12), list(zip(err, e))


@pytest.mark.parametrize("case", NM_CASES)
def test_simplex_runs_reach_the_printed_minimum(gpu, tmp_path, case):
    from imfit_gb300 import cli
    det = {}
    p, s = cli.run(_args(tmp_path, case), out=io.StringIO(), details=det)
    v, _, stat, aic, _ = _printed(case)
    if np.isnan(stat):
        stat = _stat_from_aic(aic, det["n_free"], det["n_valid"])
    assert stat - 1e-6 * abs(stat) <= s <= stat + 2e-7 * abs(stat) + 1e-6, (s, stat)
    # the parameters' scale: one-sigma errors of an LM fit of the same case
    # (Cash has no deviates: the Poisson-MLR fit of the same data stands in)
    lm = {}
    drop = ("--nm", "--cashstat")
    extra = ["--mlr"] if case == "5a" else []
    cli.run(_args(tmp_path, case, drop) + extra, out=io.StringIO(), details=lm)
    sigma = lm["errors"]
    # a parameter the LM fit holds at a limit has no sigma: 0.5 in its own units
    sigma = np.where(sigma > 0, sigma, 0.5)
    assert np.all(np.abs(p - v) <= 0.1 * sigma + 1e-5 * np.abs(v)), list(zip(p, v, sigma))


@pytest.mark.parametrize("case", sorted(ERROR_CASES))
def test_runs_the_reference_stops_stop_here(gpu, tmp_path, case):
    from imfit_gb300 import cli
    assert ERROR_CASES[case] in str(D[f"{case}__error"])
    with pytest.raises(SystemExit) as e:
        cli.run(_args(tmp_path, case), out=io.StringIO())
    assert ERROR_CASES[case] in str(e.value)


@pytest.mark.parametrize("key,section", [("full", ""), ("section", "[10:64,10:64]")])
def test_bootstrap_iterations_match_the_reference(gpu, tmp_path, key, section):
    """do_imfit_tests:133-134: --seed 10 --bootstrap 5 --save-bootstrap on
    ic3478rss_64x64.fits and on its section [10:64,10:64] (whose saved values
    carry the section's offsets added back).  The resampling indices are the
    reference's MT19937 stream, so each refit is of the same resampled image
    as the reference's: every saved value within 0.01 sigma (the printed
    errors of the full-image fit) of the reference's."""
    from imfit_gb300 import cli, fits
    cfg = "imfit_config_ic3478_64x64b.dat"
    (tmp_path / cfg).write_text(str(D[f"config__{cfg}"]))
    img = tmp_path / "ic3478rss_64x64.fits"
    fits.write_image(str(img), D["file__ic3478rss_64x64.fits"])
    out = tmp_path / "boot.dat"
    cli.run([str(tmp_path / cfg), str(img) + section, "--seed", "10", "--bootstrap", "5", "--save-bootstrap",
             str(out)], out=io.StringIO())
    lines = out.read_text().splitlines()
    header, rows = list(D[f"boot__{key}__header"]), D[f"boot__{key}__rows"]
    assert lines[-7:-5] == header
    got = np.array([[float(v) for v in ln.split()] for ln in lines[-5:]])
    sigma = D["2__errors"]
    assert np.all(np.abs(got - rows) <= 0.01 * sigma), (got - rows) / sigma


def test_saved_weight_images_data_and_model_errors(gpu, tmp_path):
    """do_imfit_tests:138-139: --save-weights after fitting a FlatSky to a
    constant image, once with data-based errors and once with --model-errors:
    the fitted model equals the data, so the two weight images (1/sigma^2)
    are the same, here 1 / (I / gain + read noise^2 / gain^2)."""
    from imfit_gb300 import cli, fits
    img = np.full((32, 40), 250.0)
    fits.write_image(str(tmp_path / "flat.fits"), img, bitpix=-64)
    (tmp_path / "c.dat").write_text("GAIN 4.0\nREADNOISE 2.0\nX0 20 1,40\nY0 16 1,32\nFUNCTION FlatSky\n"
                                    "I_sky 200 0,1000\n")
    out = {}
    for tag, extra in (("data", []), ("model", ["--model-errors"])):
        w = tmp_path / f"w_{tag}.fits"
        cli.run([str(tmp_path / "c.dat"), str(tmp_path / "flat.fits"), "--save-weights", str(w)] + extra,
                out=io.StringIO())
        out[tag] = fits.read_image(str(w))[0]
    want = 1.0 / (250.0 / 4.0 + 2.0 ** 2 / 4.0 ** 2)
    assert np.allclose(out["data"], want, rtol=1e-12)
    assert np.allclose(out["model"], out["data"], rtol=1e-7)


def test_chisquare_only_printouts(gpu, tmp_path):
    """do_imfit_tests:98-99 (imfit_textout4c, 4d): --chisquare-only on the
    n3073 case, with data-based chi^2 (the printed lines, character for
    character) and with --cashstat (the printed numbers)."""
    from imfit_gb300 import cli, fits
    d = np.load(os.path.join(GOLDEN, "n3073.npz"))
    names = ["X0", "Y0", "PA", "ell", "n", "I_e", "r_e", "PA", "ell", "I_0", "h"]
    lines = [f"GAIN {float(d['gain'])}", f"READNOISE {float(d['read_noise'])}",
             f"ORIGINAL_SKY {float(d['original_sky'])}"]
    for j, (nm, v, lo, hi) in enumerate(zip(names, d["params"], d["lo"], d["hi"])):
        if j in (2, 7):
            lines.append("FUNCTION Sersic" if j == 2 else "FUNCTION Exponential")
        lines.append(f"{nm} {float(v)!r} {float(lo)!r},{float(hi)!r}")
    (tmp_path / "c.dat").write_text("\n".join(lines) + "\n")
    for k, arr in (("data", d["data"]), ("mask", d["mask"]), ("psf", d["psf"])):
        fits.write_image(str(tmp_path / f"{k}.fits"), arr)
    base = [str(tmp_path / "c.dat"), str(tmp_path / "data.fits"), "--mask", str(tmp_path / "mask.fits"),
            "--psf", str(tmp_path / "psf.fits"), "--chisquare-only"]
    out = io.StringIO()
    cli.run(base, out=out)
    assert out.getvalue().splitlines() == ["  CHI-SQUARE = 235606.146670    (28743 DOF)", "",
                                           "Reduced Chi^2 = 8.196992",
                                           "AIC = 235628.155855, BIC = 235719.078524"]
    # the Cash value, -3.06e8, prints one ulp-level digit past what a different
    # summation order keeps: the numbers within 2e-6 (1e-14 relative)
    out = io.StringIO()
    cli.run(base + ["--cashstat"], out=out)
    got = out.getvalue().splitlines()
    assert len(got) == 2 and got[0].startswith("  CASH STATISTIC = ") and got[1].startswith("AIC = ")
    cash = float(got[0].split("=")[1])
    aic, bic = (float(x.split("=")[1]) for x in got[1].split(","))
    for v, want in ((cash, -305659765.743167), (aic, -305659743.733982), (bic, -305659652.811314)):
        assert abs(v - want) <= 2e-6, (v, want)
