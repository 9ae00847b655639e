"""GPU tests of the command-line front ends and the differential-evolution
driver, against the reference's regression outputs (do_makeimage_tests,
do_imfit_tests) held in tests/golden."""
import io
import os

import numpy as np
import pytest

from helpers import normwise

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

SERSIC_EXP_FLAT = """NCOLS 512
NROWS 512
X0 256.0
Y0 256.0
FUNCTION Sersic   # LABEL bulge
PA 30.0
ell 0.5
n 2.5
I_e 100.0
r_e 50.0
FUNCTION Exponential   # LABEL disk
PA 30.0
ell 0.75
I_0 10.0
h 150.0
FUNCTION FlatSky
I_0 1000.0
"""


def test_makeimage_oversampled_golden(gpu, tmp_path):
    """do_makeimage_tests:68: --psf, --overpsf, --overpsf_scale 3,
    --overpsf_region 100:110,100:110 and --output-functions against
    tests/oversampled_orig.fits (the single Gaussian image too)."""
    from imfit_gb300 import cli, fits
    g = np.load(os.path.join(GOLDEN, "makeimage.npz"))
    names = ["X0", "Y0", "PA", "ell", "I_0", "sigma"]
    lines = [f"{n} {float(v)!r}" for n, v in zip(names[:2], g["ov_params"][:2])] + ["FUNCTION Gaussian"]
    lines += [f"{n} {float(v)!r}" for n, v in zip(names[2:], g["ov_params"][2:])]
    (tmp_path / "c.dat").write_text("\n".join(lines) + "\n")
    fits.write_image(str(tmp_path / "psf.fits"), g["psf_standard"])
    fits.write_image(str(tmp_path / "opsf.fits"), g["psf_oversamp"])
    x1, x2, y1, y2 = (int(v) for v in g["ov_region"])
    out = str(tmp_path / "ov.fits")
    model, _ = cli.makeimage([str(tmp_path / "c.dat"), "-o", out, "--ncols", "200", "--nrows", "200",
                              "--psf", str(tmp_path / "psf.fits"), "--overpsf", str(tmp_path / "opsf.fits"),
                              "--overpsf_scale", str(int(g["ov_scale"])), "--overpsf_region", f"{x1}:{x2},{y1}:{y2}",
                              "--output-functions", str(tmp_path / "single")], out=io.StringIO())
    saved = fits.read_image(out)[0]
    assert normwise(model, g["ov_image"]) < 1e-7
    assert normwise(saved, g["ov_image"]) < 2e-7  # float32 FITS, as the reference writes
    single = fits.read_image(str(tmp_path / "single1_Gaussian.fits"))[0]
    assert normwise(single, g["ov_image"]) < 2e-7


def _within_float32_ulp(model, golden):
    """FP64 model against a float32 reference image: within one float32 ulp,
    plus 1e-12 of the image maximum for the FFT's round-off far from the
    sources (values ~1e-16 there, which the reference's own comparison
    ignores below 1e-7)."""
    g = np.asarray(golden, dtype=np.float32)
    ulp = np.spacing(np.abs(g)).astype(np.float64)
    return np.all(np.abs(model - g.astype(np.float64)) <= ulp + 1e-12 * np.max(np.abs(g)))


def test_makeimage_biggertest_golden(gpu, tmp_path):
    """do_makeimage_tests:48: config_biggertest_4c.dat (three function sets,
    X0/Y0 outside their limits -- makeimage does not check limits) at
    64 x 64 against tests/biggertest_orig.fits, every pixel within one
    float32 ulp."""
    from imfit_gb300 import cli, fits
    g = np.load(os.path.join(GOLDEN, "makeimage.npz"))
    (tmp_path / "c.dat").write_text(str(g["big_config"]))
    out = str(tmp_path / "big.fits")
    model, _ = cli.makeimage([str(tmp_path / "c.dat"), "-o", out, "--ncols", "64", "--nrows", "64"],
                             out=io.StringIO())
    assert _within_float32_ulp(model, g["big_image"])
    assert np.array_equal(fits.read_image(out)[0], g["big_image"].astype(np.float64))


@pytest.mark.parametrize("two_psfs", [False, True])
def test_makeimage_two_oversampled_regions_golden(gpu, tmp_path, two_psfs):
    """do_makeimage_tests:70 and :72: two oversampled regions (100:110,100:110
    and 20:30,20:30) with one PSF image for both, or one each, against
    tests/oversampled2both_orig.fits within one float32 ulp; the
    single-function images sum to the model (do_makeimage_tests:215)."""
    from imfit_gb300 import cli, fits
    g = np.load(os.path.join(GOLDEN, "makeimage.npz"))
    (tmp_path / "c.dat").write_text(str(g["ov2_config"]))
    fits.write_image(str(tmp_path / "psf.fits"), g["psf_standard"])
    fits.write_image(str(tmp_path / "opsf.fits"), g["psf_oversamp"])
    opsf = str(tmp_path / "opsf.fits")
    args = [str(tmp_path / "c.dat"), "-o", str(tmp_path / "ov2.fits"), "--psf", str(tmp_path / "psf.fits")]
    if two_psfs:
        args += ["--overpsf", opsf, "--overpsf_scale", "3", "--overpsf_region", "100:110,100:110",
                 "--overpsf", opsf, "--overpsf_scale", "3", "--overpsf_region", "20:30,20:30"]
    else:
        args += ["--overpsf", opsf, "--overpsf_scale", "3", "--overpsf_region", "100:110,100:110",
                 "--overpsf_region", "20:30,20:30", "--output-functions", str(tmp_path / "double")]
    model, _ = cli.makeimage(args, out=io.StringIO())
    assert _within_float32_ulp(model, g["ov2_image"])
    if not two_psfs:
        parts = [fits.read_image(str(tmp_path / f"double{k}_Gaussian.fits"))[0] for k in (1, 2)]
        assert np.allclose(parts[0] + parts[1], model, rtol=0, atol=1e-6)


def test_makeimage_fluxes_table(gpu, tmp_path):
    """do_makeimage_tests:60 (makeimage_textout5b): --print-fluxes --nosave
    on config_makeimage_sersic+exp512b.dat; the table lines as printed."""
    from imfit_gb300 import cli
    (tmp_path / "c.dat").write_text(SERSIC_EXP_FLAT)
    buf = io.StringIO()
    model, table = cli.makeimage([str(tmp_path / "c.dat"), "--print-fluxes", "--nosave"], out=buf)
    assert model is None
    assert table == ["Component                 Flux        Magnitude   Fraction   Label",
                     "Sersic                    2.2635e+06      ---     0.86495    bulge",
                     "Exponential               3.5343e+05      ---     0.13505    disk",
                     "FlatSky                   0.0000e+00      ---     0.00000",
                     "",
                     "Total                     2.6169e+06      ---     1.00000"]
    assert "\n".join(table) in buf.getvalue()


def test_makeimage_single_function_images_sum_to_model(gpu, tmp_path, oracle_mod):
    """do_makeimage_tests:65 (--output-functions with a PSF; the single images
    sum to the model image), with --save-expanded and the config's own
    NCOLS/NROWS, on a 96 x 80 image; the model against the oracle."""
    from imfit_gb300 import cli, fits
    cfg = SERSIC_EXP_FLAT.replace("NCOLS 512", "NCOLS 96").replace("NROWS 512", "NROWS 80")
    cfg = cfg.replace("X0 256.0", "X0 48.3").replace("Y0 256.0", "Y0 40.6").replace("r_e 50.0", "r_e 9.0")
    (tmp_path / "c.dat").write_text(cfg.replace("h 150.0", "h 15.0"))
    yy, xx = np.mgrid[-7:8, -7:8]
    psf = np.exp(-(xx ** 2 + yy ** 2) / 4.5)
    fits.write_image(str(tmp_path / "psf.fits"), psf, bitpix=-64)
    out = str(tmp_path / "m.fits")
    model, _ = cli.makeimage([str(tmp_path / "c.dat"), "-o", out, "--psf", str(tmp_path / "psf.fits"),
                              "--output-functions", str(tmp_path / "f"), "--save-expanded"], out=io.StringIO())
    assert model.shape == (80, 96)
    parts = [fits.read_image(str(tmp_path / f"f{k}_{n}.fits"))[0]
             for k, n in ((1, "Sersic"), (2, "Exponential"), (3, "FlatSky"))]
    assert normwise(sum(parts), model) < 3e-7
    expanded = fits.read_image(str(tmp_path / "expanded_m.fits"))[0]
    assert expanded.shape == (80 + 2 * 15, 96 + 2 * 15)
    o = oracle_mod.OracleModel()
    for name, new_set in (("Sersic", True), ("Exponential", False), ("FlatSky", False)):
        o.add_function(name, new_set)
    o.finish_functions()
    o.add_psf(psf)
    o.setup_model_image(96, 80)
    o.create_model_image([48.3, 40.6, 30.0, 0.5, 2.5, 100.0, 9.0, 30.0, 0.75, 10.0, 15.0, 1000.0])
    assert normwise(model, o.get_model_image()) < 1e-10


def _ic3478_files(tmp_path):
    from imfit_gb300 import fits
    d = np.load(os.path.join(GOLDEN, "ic3478.npz"))
    names = ["X0", "Y0", "PA", "ell", "n", "I_e", "r_e"]
    lines = [f"GAIN {float(d['gain'])}", f"READNOISE {float(d['read_noise'])}",
             f"ORIGINAL_SKY {float(d['original_sky'])}"]
    for j, (nm, v, lo, hi) in enumerate(zip(names, d["params"], d["lo"], d["hi"])):
        if j == 2:
            lines.append("FUNCTION Sersic")
        lines.append(f"{nm} {float(v)!r} {float(lo)!r},{float(hi)!r}")
    (tmp_path / "c.dat").write_text("\n".join(lines) + "\n")
    fits.write_image(str(tmp_path / "data.fits"), d["data"])
    return d


def test_ic3478_nelder_mead_matches_printed_result(gpu, tmp_path):
    """do_imfit_tests:70 (imfit_textout3b, --nm): the simplex ends at the
    printed minimum (CHI-SQUARE 4555.947706, NLopt's) to 2e-7 and within
    0.1 sigma of its printed parameters."""
    from imfit_gb300 import cli
    d = _ic3478_files(tmp_path)
    p, s = cli.run([str(tmp_path / "c.dat"), str(tmp_path / "data.fits"), "--nm", "--save-params",
                    str(tmp_path / "b.dat")], out=io.StringIO())
    want = np.array([32.9440, 34.0933, 18.2602, 0.235985, 2.40034, 20.0081, 60.7635])
    assert np.all(np.abs(p - want) <= 0.1 * d["lm_errors_printed"]), (p, want)
    assert s <= 4555.947706 * (1 + 2e-7)


@pytest.mark.parametrize("solver", ["lm", "de"])
def test_ic3478_fits_match_printed_results(gpu, tmp_path, solver):
    """do_imfit_tests:68 and :75 (imfit_textout3, imfit_textout3c_tail):
    ic3478rss_64x64.fits with imfit_config_ic3478_64x64b.dat, by LM and by
    differential evolution (--de); the fitted values agree with the printed
    ones to within 0.05 sigma (LM) or 0.1 sigma (DE, whose last digits are
    set by the float32 noise of the statistic it minimises), the reduced
    chi^2 to its six printed decimals."""
    from imfit_gb300 import cli
    d = _ic3478_files(tmp_path)
    args = [str(tmp_path / "c.dat"), str(tmp_path / "data.fits"), "--save-params", str(tmp_path / "b.dat")]
    if solver == "de":
        args += ["--de", "--seed", "7"]
    buf = io.StringIO()
    p, s = cli.run(args, out=buf)
    want = d["lm_params_printed"] if solver == "lm" else d["de_params_printed"]
    tol = (0.05 if solver == "lm" else 0.1) * d["lm_errors_printed"]
    assert np.all(np.abs(p - want) <= tol), (p, want)
    chi2 = float(d["lm_chi2_printed"])
    assert s > chi2 - 1e-6  # the FP64 statistic at the fitted point: never below the minimum
    if solver == "lm":
        assert s - chi2 < 2e-7 * chi2 and abs(s / (64 * 64 - 7) - float(d["lm_reduced_printed"])) < 1e-6
    else:
        assert s - chi2 < 1e-5 * chi2


def test_de_driver_on_the_batched_statistic(gpu):
    """differential_evolution on ModelObject: one batched call per
    generation, and at the LM minimum of the same model."""
    from imfit_gb300 import solvers
    d = np.load(os.path.join(GOLDEN, "ic3478.npz"))
    m = gpu.ModelObject()
    m.add_function("Sersic", True)
    m.finish_functions()
    m.add_image_data(d["data"].astype(np.float64))
    m.add_image_characteristics(float(d["gain"]), float(d["read_noise"]), 1.0, 1, float(d["original_sky"]))
    assert m.final_setup() == 0
    r = solvers.differential_evolution(m, d["params"], d["lo"], d["hi"], seed=1, latin_hypercube=True)
    assert r["population"] == 56
    assert r["batched_calls"] == r["generations"] + (2 if r["converged"] else 1)
    lm = m.fit_lm(d["params"], lower=d["lo"], upper=d["hi"])
    s_lm = m.get_fit_statistic(lm["params"])
    assert r["statistic"] <= s_lm * (1 + 1e-6)
    assert np.all(np.abs(r["params"] - lm["params"]) <= 0.1 * d["lm_errors_printed"])


def _ic3478_model(gpu_or_oracle_cls, d):
    m = gpu_or_oracle_cls()
    m.add_function("Sersic", True)
    m.finish_functions()
    m.add_image_data(d["data"].astype(np.float64))
    m.add_image_characteristics(float(d["gain"]), float(d["read_noise"]), 1.0, 1, float(d["original_sky"]))
    assert m.final_setup() == 0
    return m


def test_batched_bootstrap_matches_sequential_refits_and_oracle_samples(gpu, oracle_mod):
    """imfit_BootstrapFitBatch against the reference's loop
    (core/bootstrap_errors.cpp:171-215: UseBootstrap, then MakeBootstrapSample
    and an LM refit per iteration) run one sample at a time on the same
    handle type, and each sample's statistic against the FP64 oracle's
    bootstrap statistic for the same seed and iteration."""
    from imfit_gb300 import solvers
    d = np.load(os.path.join(GOLDEN, "ic3478.npz"))
    best = d["lm_params_printed"]
    K, seed = 12, 4321
    mb = _ic3478_model(gpu.ModelObject, d)
    samples, status = solvers.bootstrap_errors(mb, best, K, seed, lower=d["lo"], upper=d["hi"], chunk=5)
    assert status.shape == (K,) and np.all(status > 0) and samples.shape == (K, 7)
    ms = _ic3478_model(gpu.ModelObject, d)
    ms.use_bootstrap(seed)
    o = _ic3478_model(oracle_mod.OracleModel, d)
    o.use_bootstrap(seed)
    for k in range(K):
        ms.make_bootstrap_sample()
        o.make_bootstrap_sample()
        r = ms.fit_lm(best, lower=d["lo"], upper=d["hi"])
        err = np.abs(r["params"] - samples[k]) / d["lm_errors_printed"]
        assert np.all(err < 0.05), (k, err)
        s_o = o.get_fit_statistic(samples[k])
        s_g = ms.get_fit_statistic(samples[k])  # plain FP64 path, bootstrap sample k
        assert abs(s_g - s_o) <= 1e-10 * s_o, (k, s_g, s_o)
    # the spread of the refits is the parameters' uncertainty (mpfit's errors, within sampling noise)
    sd = np.array([solvers.standard_deviation(samples[:, j]) for j in range(7)])
    assert np.all(sd > 0.3 * d["lm_errors_printed"]) and np.all(sd < 3.0 * d["lm_errors_printed"]), sd


def test_cli_bootstrap_output(gpu, tmp_path):
    """--bootstrap N --save-bootstrap F: the summary block and the file
    (header of GetParamHeader, one row per successful iteration)."""
    from imfit_gb300 import cli
    _ic3478_files(tmp_path)
    buf = io.StringIO()
    cli.run([str(tmp_path / "c.dat"), str(tmp_path / "data.fits"), "--save-params", str(tmp_path / "b.dat"),
             "--bootstrap", "8", "--seed", "99", "--save-bootstrap", str(tmp_path / "boot.dat")], out=buf)
    text = buf.getvalue()
    assert "Statistics for parameter values from bootstrap resampling (8 successful iterations):" in text
    assert "\nr_e = " in text
    lines = (tmp_path / "boot.dat").read_text().splitlines()
    assert lines[1] == "# Bootstrap resampling output (8 iterations requested):"
    assert lines[2] == "# X0_1\t\tY0_1\t\tPA_1\tell_1\tn_1\tI_e_1\tr_e_1\t"
    assert len(lines) == 3 + 8 and all(len(x.split("\t")) == 7 for x in lines[3:])


def test_mcmc_faintstar_posterior(gpu, tmp_path):
    """do_mcmc_tests:27 (imfit-mcmc on tests/faintstar.fits, --no-subsampling):
    the DREAM chains' post-burn-in posterior against the reference's chain 1
    (tests/imfit-mcmc_reference/mcmc_ref1.1.txt_skip3) -- means within 0.3 of
    its standard deviations, widths within 25 % -- and the chain files'
    layout.  The samplers share the algorithm, not the random stream."""
    from imfit_gb300 import cli, fits
    d = np.load(os.path.join(GOLDEN, "mcmc.npz"))
    names = ["X0", "Y0", "PA", "ell", "I_0", "sigma"]
    lines = [f"GAIN {float(d['gain'])}", f"READNOISE {float(d['read_noise'])}",
             f"ORIGINAL_SKY {float(d['original_sky'])}"]
    for j, (nm, v, lo, hi) in enumerate(zip(names, d["params"], d["lo"], d["hi"])):
        if j == 2:
            lines.append("FUNCTION Gaussian")
        lines.append(f"{nm} {float(v)!r} {float(lo)!r},{float(hi)!r}")
    (tmp_path / "c.dat").write_text("\n".join(lines) + "\n")
    fits.write_image(str(tmp_path / "star.fits"), d["data"])
    root = str(tmp_path / "chain")
    r = cli.mcmc([str(tmp_path / "c.dat"), str(tmp_path / "star.fits"), "--nosubsampling", "--seed", "7",
                  "-o", root], out=io.StringIO())
    # burn-in ends at 5000 unless an outlier chain after it sends the sampler back (dream.cpp:386-397)
    assert r["converged"] and r["n_chains"] == 6 and r["burn_in_end"] >= 5000
    post = r["chains"][r["burn_in"] == 0].reshape(-1, 6)
    mean, std = post.mean(axis=0), post.std(axis=0, ddof=1)
    assert np.all(np.abs(mean - d["ref_mean"]) < 0.3 * d["ref_std"]), (mean, d["ref_mean"])
    assert np.all(np.abs(std / d["ref_std"] - 1.0) < 0.25), (std, d["ref_std"])
    rows = np.loadtxt(root + ".1.txt", comments="#")
    assert rows.shape == (r["generations"], 12) and np.all(rows[:5000, 7] == 1)
    assert np.array_equal(rows[:, 7], r["burn_in"]) and np.all(rows[r["burn_in_end"]:, 7] == 0)
    assert abs(rows[:, 6].max() - float(d["ref_best_loglik"])) < 0.5


def test_image_section_offsets(gpu, tmp_path, oracle_mod):
    """imfit on IMAGE[x1:x2,y1:y2]: X0/Y0 (values and limits) shift by the
    section's offset while fitting and shift back in the output
    (core/imfit_main.cpp:211, 288-309, 350-356).  The statistic through the
    command line equals the oracle's on the cropped image with shifted
    centres; a fit of the section reports full-image coordinates close to
    the whole image's fit."""
    from imfit_gb300 import cli
    d = _ic3478_files(tmp_path)
    sec = str(tmp_path / "data.fits") + "[5:60,3:58]"
    p_full = d["lm_params_printed"]
    cfgp = tmp_path / "c2.dat"
    lines = [f"GAIN {float(d['gain'])}", f"READNOISE {float(d['read_noise'])}",
             f"ORIGINAL_SKY {float(d['original_sky'])}"]
    for j, (nm, v, lo, hi) in enumerate(zip(["X0", "Y0", "PA", "ell", "n", "I_e", "r_e"], p_full, d["lo"], d["hi"])):
        if j == 2:
            lines.append("FUNCTION Sersic")
        lines.append(f"{nm} {float(v)!r} {float(lo)!r},{float(hi)!r}")
    cfgp.write_text("\n".join(lines) + "\n")
    _, s = cli.run([str(cfgp), sec, "--chisquare-only"], out=io.StringIO())
    o = oracle_mod.OracleModel()
    o.add_function("Sersic", True)
    o.finish_functions()
    o.add_image_data(d["data"].astype(np.float64)[2:58, 4:60])
    o.add_image_characteristics(float(d["gain"]), float(d["read_noise"]), 1.0, 1, float(d["original_sky"]))
    assert o.final_setup() == 0
    shifted = p_full.copy()
    shifted[0] -= 4
    shifted[1] -= 2
    assert abs(s - o.get_fit_statistic(shifted)) <= 1e-10 * s
    p, _ = cli.run([str(cfgp), sec, "--save-params", str(tmp_path / "b2.dat")], out=io.StringIO())
    assert abs(p[0] - p_full[0]) < 0.1 and abs(p[1] - p_full[1]) < 0.1
