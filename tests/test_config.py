"""CPU tests of the configuration-file parser (the format of
core/config_file_parser.cpp:494-657) and the FITS round trip."""
import os

import numpy as np
import pytest

import oracle
from imfit_gb300 import config, fits

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_CONFIG = os.path.join(oracle.REFERENCE_DIR, "tests", "imfit_reference", "imfit_config_n3073.dat")

N3073_STYLE = """# comment line
GAIN   4.725
READNOISE   4.3
ORIGINAL_SKY   154.33

X0   101.0    90,110
Y0   97.0     90,110
FUNCTION Sersic
PA    110.0   0,180
ell    0.2    0,1
n      1.5    fixed
I_e    150
r_e    15     0,100

FUNCTION   Exponential   # trailing comment
PA    55.0   0,90      # another
ell    0.2   0,1
I_0   70.0   0,600
h     45.0   0,1000

X0   20.0
Y0   30.0
FUNCTION FlatSky
I_sky  3.0
"""


def test_parse_function_sets_limits_and_fixed():
    c = config.parse_config(N3073_STYLE)
    assert c.gain == 4.725 and c.read_noise == 4.3 and c.original_sky == 154.33
    assert c.functions == [("Sersic", True), ("Exponential", False), ("FlatSky", True)]
    assert c.param_names[:7] == ["X0", "Y0", "PA", "ell", "n", "I_e", "r_e"]
    assert len(c.values) == 2 + 5 + 4 + 2 + 1
    assert c.fixed[4] == 1 and c.fixed.sum() == 1
    assert np.isnan(c.lower[5]) and c.lower[2] == 0 and c.upper[2] == 180
    again = config.parse_config(config.format_params(c, c.values))
    assert np.array_equal(again.values, c.values) and again.functions == c.functions


@pytest.mark.parametrize("bad", ["FUNCTION Sersic\nPA 1\n", "X0 1\nFUNCTION Sersic\n",
                                 "X0 1 0,10\nY0 2\nFUNCTION Exponential\nPA 5 10,20\n",
                                 "X0 1\nY0 2\nPA 3\n", "X0 1\nY0 2\nFUNCTION Sersic\nPA x\n"])
def test_parse_errors(bad):
    with pytest.raises(config.ConfigError):
        config.parse_config(bad)


@pytest.mark.skipif(not os.path.exists(REF_CONFIG), reason="reference checkout not present")
def test_reference_config_matches_the_n3073_fixture():
    c = config.read_config(REF_CONFIG)
    d = np.load(os.path.join(GOLDEN, "n3073.npz"))
    assert np.array_equal(c.values, d["params"])
    assert np.array_equal(c.lower, d["lo"]) and np.array_equal(c.upper, d["hi"])
    assert c.gain == float(d["gain"]) and c.read_noise == float(d["read_noise"])


def test_fits_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    a = rng.normal(size=(7, 5)).astype(np.float32).astype(np.float64)
    p = tmp_path / "x.fits"
    fits.write_image(str(p), a)
    assert np.array_equal(fits.read_image(str(p))[0], a)


def test_labels_optional_params_and_image_size_options():
    """FUNCTION ... # LABEL x (core/config_file_parser.cpp:208-222), an
    OPTIONAL_PARAMS block (config_file_parser.cpp:450-465), NCOLS/NROWS."""
    text = """NCOLS 64
NROWS 48
X0 32
Y0 24
FUNCTION Sersic   # LABEL bulge component
PA 30
ell 0.5
n 2.5
I_e 100
r_e 50
FUNCTION Gaussian
OPTIONAL_PARAMS_START
mode  alpha
OPTIONAL_PARAMS_END
PA 30
ell 0.1
I_0 10
sigma 3
"""
    cfg = config.parse_config(text)
    assert cfg.labels == ["bulge component", ""]
    assert cfg.optional == [{}, {"mode": "alpha"}]
    assert cfg.options["NCOLS"] == "64" and cfg.options["NROWS"] == "48"
    assert len(cfg.values) == 11
    out = config.format_params(cfg, cfg.values)
    assert "FUNCTION Sersic   # LABEL bulge component" in out
    again = config.parse_config(out)
    assert again.labels[0] == "bulge component" and np.allclose(again.values, cfg.values)
    with pytest.raises(config.ConfigError):
        config.parse_config(text.replace("OPTIONAL_PARAMS_END\n", ""))


def test_region_strings():
    from imfit_gb300.cli import parse_region
    assert parse_region("100:110,20:30") == (100, 110, 20, 30)
    with pytest.raises(SystemExit):
        parse_region("100-110,20:30")


def test_fits_image_sections(tmp_path):
    """CFITSIO-style sections file.fits[x1:x2,y1:y2] (1-based, x = column) and
    DetermineImageOffset (core/utilities.cpp:483-489)."""
    a = np.arange(30.0).reshape(5, 6)
    p = str(tmp_path / "a.fits")
    fits.write_image(p, a, bitpix=-64)
    sub = fits.read_image(p + "[2:4,3:5]")[0]
    assert np.array_equal(sub, a[2:5, 1:4])
    assert fits.image_offset(p + "[2:4,3:5]") == (1, 2) and fits.image_offset(p) == (0, 0)
    with pytest.raises(ValueError):
        fits.read_image(p + "[2:9,1:2]")


def test_information_criteria_reproduce_printed_aic_bic():
    """AIC (bias-corrected) and BIC from the printed statistic, the free
    parameters and the valid pixels, as imfit prints them
    (imfit_textout2: 7 free, 4096 pixels; imfit_textout8a: 3 free, 1600;
    imfit_textout7a: 3 free, 8)."""
    import os
    import numpy as np
    from imfit_gb300.cli import information_criteria
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "imfit_regressions.npz"))
    for case, k, n in (("2", 7, 4096), ("3e", 6, 4096), ("8a", 3, 1600), ("7a", 3, 8)):
        aic, bic = information_criteria(float(d[f"{case}__stat"]), k, n)
        # the printed statistic is itself rounded to 1e-6
        assert abs(aic - float(d[f"{case}__aic"])) <= 1.5e-6 and abs(bic - float(d[f"{case}__bic"])) <= 1.5e-6, case


@pytest.mark.skipif(not oracle.reference_checkout(), reason="reference checkout not present")
@pytest.mark.parametrize("name", ["makeimage_reference/config_makeimage_sersictest512_bad1.dat",
                                  "makeimage_reference/config_makeimage_sersictest512_bad2.dat",
                                  "makeimage_reference/config_makeimage_sersictest512_bad3.dat",
                                  "makeimage_reference/config_makeimage_sersictest512_bad4.dat",
                                  "makeimage_reference/config_makeimage_sersictest512_bad5.dat",
                                  "imfit_reference/config_imfit_sersictest512_badlimits1.dat",
                                  "imfit_reference/config_imfit_sersictest512_badlimits2.dat",
                                  "imfit_reference/config_imfit_sersictest512_badlimits3.dat",
                                  "config_imfit_sersictest512_badlimits4.dat",
                                  "imfit_reference/config_imfit_badparamline.dat"])
def test_reference_bad_configurations_are_rejected(name):
    """The configuration files the reference's regression runs reject
    (do_imfit_tests:194-201, do_makeimage_tests:78-82; "Failure reading
    configuration file"): each is rejected here too."""
    from imfit_gb300 import config
    root = os.path.join(oracle.REFERENCE_DIR, "tests")
    with pytest.raises(config.ConfigError):
        config.read_config(os.path.join(root, name))
