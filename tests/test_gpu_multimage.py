"""GPU tests of simultaneous multi-image fitting (multimfit) against the
reference's regression printouts (tests/multimfit_reference)."""
import io
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

SMALLGAUSS = """GAIN 1
ORIGINAL_SKY 100

X0 2 0,5
Y0 2 0,5
FUNCTION Gaussian
PA 0 -50,50
ell 0.1 0,0.6
I_0 900 500,1500
sigma 1.5 0.1,3
"""


def _write(tmp_path, d):
    from imfit_gb300 import fits
    for k in ("g0", "g1", "gsig", "d1a", "d1b"):
        fits.write_image(str(tmp_path / f"{k}.fits"), d[k])
    (tmp_path / "gauss.dat").write_text(SMALLGAUSS)
    (tmp_path / "gauss_info.txt").write_text(f"""IMAGE_START
DATA {tmp_path / 'g0.fits'}
ERROR {tmp_path / 'gsig.fits'}
ORIGINAL_SKY 100.0
IMAGE_START
DATA {tmp_path / 'g1.fits'}
ERROR {tmp_path / 'gsig.fits'}
ORIGINAL_SKY 100.0
PIXEL_SCALE 1.0 fixed
IMAGE_PA 0.0 fixed
FLUX_SCALE 1.0 fixed
X0 2
Y0 2
GAIN 1
ORIGINAL_SKY 100
""")
    (tmp_path / "flat.dat").write_text("X0 1\nY0 1\nFUNCTION FlatSky\nI0 1.0\n")
    (tmp_path / "flat_info.txt").write_text(f"""IMAGE_START
DATA {tmp_path / 'd1a.fits'}
ORIGINAL_SKY 0.0
IMAGE_START
DATA {tmp_path / 'd1b.fits'}
ORIGINAL_SKY 0.0
PIXEL_SCALE 1.0 fixed
IMAGE_PA 0.0 fixed
FLUX_SCALE 1.0 fixed
X0 2 fixed
Y0 2 fixed
""")


def test_multimfit_fitstat_only(gpu, tmp_path):
    """multimfit_textout1a: --fitstat-only on two 2x2 images with a FlatSky
    model: CHI-SQUARE = 6.750000 at the starting parameters."""
    from imfit_gb300 import cli
    d = np.load(os.path.join(GOLDEN, "multimfit.npz"))
    _write(tmp_path, d)
    for flag in ("--fitstat-only", "--chisquare-only"):
        buf = io.StringIO()
        p, s = cli.multimfit([str(tmp_path / "flat.dat"), "--image-info", str(tmp_path / "flat_info.txt"), flag],
                             out=buf)
        assert p.size == 8 and abs(s - float(d["d_chi2_printed"])) < 1e-12
        # the printout's statistic lines (multimfit_textout1a:28-31)
        assert buf.getvalue().strip().splitlines() == ["CHI-SQUARE = 6.750000    (5 DOF)", "",
                                                       "Reduced Chi^2 = 1.350000",
                                                       "AIC = 18.750000, BIC = 12.988325"]


def test_multimfit_smallgauss_fit(gpu, tmp_path):
    """multimfit_textout3a (Nelder-Mead, CHI-SQUARE 36.070608): the summed
    statistic at the printed parameters is the printed minimum (to the
    rounding of the printed digits), the LM fit on the summed normal equations
    reaches it and lands on the printed parameters; the fast path's summed
    statistic and gradient agree with the FP64 statistic and its differences;
    Nelder-Mead through the command line ends at the same minimum."""
    from imfit_gb300 import cli
    from imfit_gb300.config import read_config
    from imfit_gb300.multimage import MultiImageModel, build_handles, global_vector, parse_image_info
    d = np.load(os.path.join(GOLDEN, "multimfit.npz"))
    _write(tmp_path, d)
    cfg = read_config(str(tmp_path / "gauss.dat"))
    images = parse_image_info((tmp_path / "gauss_info.txt").read_text())
    mm = MultiImageModel(cfg.functions, build_handles(cfg.functions, images))
    p0, lo, hi, fx = global_vector(cfg, images)
    assert mm.n_params == 11 and int(np.sum(fx == 0)) == 8
    printed = np.concatenate([[1.0, 0.0, 1.0], d["g_image2_printed"], d["g_model_printed"]])
    s_printed = mm.get_fit_statistic(printed)
    chi2 = float(d["g_chi2_printed"])
    assert abs(s_printed - chi2) < 2e-3, s_printed
    s, g = mm.statistic_and_gradient(printed)
    assert abs(s - s_printed) <= 1e-5 * s_printed
    r = mm.fit_lm(p0, fixed=fx, lower=np.where(np.isnan(lo), 0.0, lo), upper=np.where(np.isnan(hi), 0.0, hi))
    s_fit = mm.get_fit_statistic(r["params"])
    assert r["status"] > 0 and s_fit <= chi2 + 1e-4, s_fit
    assert np.all(np.abs(r["params"] - printed) <= np.array([0, 0, 0, 2e-3, 2e-3, 2e-3, 2e-3, 0.05, 1e-3, 0.1, 1e-3]))
    p_nm, s_nm = cli.multimfit([str(tmp_path / "gauss.dat"), "-i", str(tmp_path / "gauss_info.txt"), "--nm"],
                               out=io.StringIO())
    assert s_nm <= chi2 + 1e-3


GLOBAL_CFG = """X0 31.0 0,4
Y0 31.0 0,4
FUNCTION Exponential
PA 95.0 0,180
ell 0.45 0,1
I_0 90.0 0,1000
h 15.0 0,1000
FUNCTION Sersic
PA 90.0
ell 0.2
n 2.5
I_e 10.0
r_e 10.0
"""
SECOND_SET = """
X0 50.0
Y0 45.0
FUNCTION Gaussian
PA 0
ell 0.5
I_0 100.0
sigma 2.0
"""


def _info(third):
    ps, pa, fs = third
    return f"""IMAGE_START
NCOLS 64
NROWS 64
IMAGE_START
NCOLS 64
NROWS 64
PIXEL_SCALE 1.0 fixed
IMAGE_PA 0.0 fixed
FLUX_SCALE 1.0 fixed
X0 40
Y0 40
IMAGE_START
NCOLS 64
NROWS 64
PIXEL_SCALE {ps} fixed
IMAGE_PA {pa} fixed
FLUX_SCALE {fs} 10,20
X0 10
Y0 20
"""


@pytest.mark.parametrize("case,third,config,goldens", [
    ("plain", (1.0, 0.0, 1.0), GLOBAL_CFG, ["img_0", "img_1", "img_2"]),
    ("flux", (1.0, 0.0, 100.0), GLOBAL_CFG, [None, None, "img_2b"]),
    ("rotation", (1.0, 90.0, 1.0), GLOBAL_CFG, [None, None, "img_2c"]),
    ("scale", (10.0, 0.0, 1.0), GLOBAL_CFG, [None, None, "img_2d"]),
    ("two_sets", (1.0, 0.0, 1.0), GLOBAL_CFG + SECOND_SET, ["blk_0", "blk_1", "blk_2"]),
])
def test_makemultimages_goldens(gpu, tmp_path, case, third, config, goldens):
    """do_makemultimages_tests.sh:59-65: the model of one configuration seen
    through three image descriptions (offset X0/Y0, FLUX_SCALE, IMAGE_PA,
    PIXEL_SCALE, a second function set moved with the image) against the
    reference's float32 output images."""
    from imfit_gb300 import cli
    g = np.load(os.path.join(GOLDEN, "makemultimages.npz"))
    (tmp_path / "c.dat").write_text(config)
    (tmp_path / "info.txt").write_text(_info(third))
    imgs = cli.makemultimages([str(tmp_path / "c.dat"), "-i", str(tmp_path / "info.txt"), "-o",
                               str(tmp_path / "m")], out=io.StringIO())
    for img, key in zip(imgs, goldens):
        if key is None:
            continue
        want = g[key].astype(np.float64)
        assert img.shape == want.shape
        tol = np.spacing(np.abs(g[key])).astype(np.float64) * 2 + 1e-30
        assert np.all(np.abs(img - want) <= tol), (key, np.max(np.abs(img - want) / tol))


_REF_NAMES = {"g0": "smallgauss_5x5_0.fits", "g1": "smallgauss_5x5_1.fits", "gsig": "smallgauss_5x5_sigma.fits",
              "d1a": "smallDataImage1a.fits", "d1b": "smallDataImage1b.fits"}
# per printed parameter (model first, then image 2's description parameters):
# FlatSky cases -- X0, Y0 of the model have no effect (None: not compared)
_TOL_FLAT = [None, None, 2e-4, 0, 0, 1e-3, 0, 0]
# Gaussian cases -- twice the LM bounds of the smallgauss fit above (the
# simplex stops within its own tolerance of the minimum)
_TOL_GAUSS = [4e-3, 4e-3, 0.1, 2e-3, 0.2, 2e-3, 0, 0, 0, 4e-3, 4e-3]


@pytest.mark.parametrize("case", ["1b", "1c", "1d", "1e", "3b", "3c", "3d", "3e", "3f"])
def test_multimfit_regression_runs(gpu, tmp_path, case):
    """do_multimfit_tests.sh:61-92 (multimfit_textout1b-1e, 3b-3f): Nelder-Mead
    and LM fits (chi^2 and Poisson-MLR) with limits on a FlatSky level and on FLUX_SCALE, image
    sections of the reference and of the second image (X0/Y0 offsets), no
    error images, --model-errors: the fitted statistic at the printed one
    (1e-4 relative for the simplex, 1e-7 for LM) and the parameters within
    the tolerances above of the printed values."""
    from imfit_gb300 import cli, fits
    d = np.load(os.path.join(GOLDEN, "multimfit.npz"))
    for k, name in _REF_NAMES.items():
        fits.write_image(str(tmp_path / name), d[k])
    (tmp_path / "c.dat").write_text(str(d[f"{case}__config"]))
    info = str(d[f"{case}__info"]).replace("tests/multimfit_reference/", str(tmp_path) + "/")
    (tmp_path / "info.txt").write_text(info)
    opts = [o for o in (str(x) for x in d[f"{case}__options"]) if o]
    p, s = cli.multimfit([str(tmp_path / "c.dat"), "-i", str(tmp_path / "info.txt")] + opts, out=io.StringIO())
    printed, stat = d[f"{case}__values"], float(d[f"{case}__stat"])
    nm = "--nm" in opts
    assert abs(s - stat) <= (1e-4 if nm else 1e-7) * stat + 1e-6, (s, stat)
    n_model = len(p) - 5
    got = np.concatenate([p[5:], p[:5]])  # printed order: model, then image 2
    assert n_model == len(printed) - 5
    tol = _TOL_FLAT if len(printed) == 8 else _TOL_GAUSS
    for k, t in enumerate(tol):
        if t is not None:
            assert abs(got[k] - printed[k]) <= t + 1e-6 * abs(printed[k]), (k, got, printed)


PER_IMAGE_CFG = """GAIN 1
X0 20.0 10,30
Y0 21.0 10,30
FUNCTION Gaussian
PA 30 0,90
ell 0.3 0,0.8
I_0 200 50,500
sigma 3.0 1,6
"""
PER_IMAGE_LOCAL = """FUNCTIONS_START
X0 1 fixed
Y0 1 fixed
FUNCTION FlatSky
I_sky 5.0 0,20
X0 30.0 25,35
Y0 10.0 5,15
FUNCTION Gaussian
PA 0 fixed
ell 0 fixed
I_0 80 20,200
sigma 1.5 0.5,4
"""
# image 1: the global Gaussian alone; image 2: the Gaussian at its own X0/Y0
# with FLUX_SCALE 1.5, plus its own sky and star
PER_IMAGE_TRUTH = dict(global_=[20.0, 21.0, 30.0, 0.3, 200.0, 3.0], desc2=[1.0, 0.0, 1.5, 17.5, 23.0],
                       local2=[1.0, 1.0, 5.0, 30.0, 10.0, 0.0, 0.0, 80.0, 1.5])


def _per_image_setup(oracle_mod, shape=(40, 44)):
    """Data of both images made by the FP64 oracle from hand-written per-image
    vectors (global functions first, then image 2's own)."""
    g, d2, l2 = PER_IMAGE_TRUTH["global_"], PER_IMAGE_TRUTH["desc2"], PER_IMAGE_TRUTH["local2"]
    v1 = list(g)
    v2 = [d2[3], d2[4], g[2], g[3], g[4] * d2[2], g[5]] + list(l2)
    glob = [("Gaussian", True)]
    local = [("FlatSky", True), ("Gaussian", True)]

    def oracle_model(funcs, data=None):
        m = oracle_mod.OracleModel()
        for name, new_set in funcs:
            m.add_function(name, new_set)
        m.finish_functions()
        if data is None:
            m.setup_model_image(shape[1], shape[0])
        else:
            m.add_image_data(data)
            m.add_image_characteristics(1.0, 0.0, 1.0, 1, 0.0)
            m.add_error_vector(np.full(shape, 2.0), 100)
            assert m.final_setup() == 0
        return m

    m1, m2 = oracle_model(glob), oracle_model(glob + local)
    m1.create_model_image(np.array(v1))
    m2.create_model_image(np.array(v2))
    data = [m1.get_model_image().copy(), m2.get_model_image().copy()]
    return data, (oracle_model(glob, data[0]), oracle_model(glob + local, data[1])), glob, local


def test_multimfit_per_image_functions(gpu, oracle_mod, tmp_path):
    """Per-image functions (a FUNCTIONS_START section in image 2's block):
    the summed statistic at a perturbed vector equals the FP64 oracle's on
    per-image vectors written by hand (global model transformed, image 2's
    own functions appended unchanged, core/param_holder.cpp:215-270); the
    fast gradient matches central differences of the statistic; LM on the
    summed normal equations recovers the truth from noise-free data; the
    command line fits the same files and prints the per-image block."""
    from imfit_gb300 import cli, fits
    from imfit_gb300.config import parse_config
    from imfit_gb300.multimage import MultiImageModel, build_handles, global_vector, parse_image_info
    data, (o1, o2), glob, local = _per_image_setup(oracle_mod)
    for k, img in enumerate(data):
        fits.write_image(str(tmp_path / f"im{k}.fits"), img, bitpix=-64)  # FP64: the oracle's own data
        fits.write_image(str(tmp_path / f"sig{k}.fits"), np.full(img.shape, 2.0), bitpix=-64)
    (tmp_path / "c.dat").write_text(PER_IMAGE_CFG)
    (tmp_path / "info.txt").write_text(f"""IMAGE_START
DATA {tmp_path / 'im0.fits'}
ERROR {tmp_path / 'sig0.fits'}
IMAGE_START
DATA {tmp_path / 'im1.fits'}
ERROR {tmp_path / 'sig1.fits'}
PIXEL_SCALE 1.0 fixed
IMAGE_PA 0.0 fixed
FLUX_SCALE 1.2 0.5,3
X0 17.0 12,22
Y0 22.0 18,28
""" + PER_IMAGE_LOCAL)
    cfg = parse_config(PER_IMAGE_CFG)
    images = parse_image_info((tmp_path / "info.txt").read_text())
    assert images[1].local_functions == local
    mm = MultiImageModel(cfg.functions, build_handles(cfg.functions, images), [im.local_functions for im in images])
    assert mm.n_local == [0, 9] and mm.n_params == 5 + 6 + 9
    p0, lo, hi, fx = global_vector(cfg, images)
    truth = np.array(PER_IMAGE_TRUTH["desc2"] + PER_IMAGE_TRUTH["global_"] + PER_IMAGE_TRUTH["local2"])
    # statistic at a perturbed vector against the oracle on hand-written vectors
    q = truth + np.where(fx == 0, 0.03 * np.abs(truth) + 0.05, 0.0)
    gq = q[5:11]
    v1 = gq
    v2 = np.concatenate([[q[3], q[4], gq[2], gq[3], gq[4] * q[2], gq[5]], q[11:]])
    want = o1.get_fit_statistic(v1) + o2.get_fit_statistic(v2)
    s = mm.get_fit_statistic(q)
    assert abs(s - want) <= 1e-10 * want, (s, want)
    # fast gradient against central differences of the FP64 statistic
    s_f, grad = mm.statistic_and_gradient(q)
    assert abs(s_f - want) <= 1e-5 * want
    fd = np.zeros(len(q))
    for j in range(len(q)):
        h = 1e-5 * max(abs(q[j]), 1.0)
        a, b = q.copy(), q.copy()
        a[j] += h
        b[j] -= h
        fd[j] = (mm.get_fit_statistic(a) - mm.get_fit_statistic(b)) / (2 * h)
    free = fx == 0
    scale = np.abs(fd[free]) + 1e-3 * np.max(np.abs(fd[free]))
    assert np.all(np.abs(grad[free] - fd[free]) <= 2e-3 * scale), list(zip(grad[free], fd[free]))
    # LM from the file's starting values
    r = mm.fit_lm(p0, fixed=fx, lower=np.where(np.isnan(lo), 0.0, lo), upper=np.where(np.isnan(hi), 0.0, hi))
    assert r["status"] > 0
    assert np.all(np.abs(r["params"] - truth) <= 1e-3 * np.maximum(np.abs(truth), 1.0)), (r["params"], truth)
    buf = io.StringIO()
    p_cli, s_cli = cli.multimfit([str(tmp_path / "c.dat"), "-i", str(tmp_path / "info.txt")], out=buf)
    # noise-free data: the minimum is 0 up to the FP32 evaluation's floor (start: ~7e4)
    assert len(p_cli) == mm.n_params and s_cli < 1e-3
    assert "# Per-image function parameters for image 2" in buf.getvalue()
    assert np.all(np.abs(p_cli - truth) <= 1e-3 * np.maximum(np.abs(truth), 1.0))


def test_makemultimages_per_image_functions(gpu, oracle_mod, tmp_path):
    """makemultimages adds an image's own functions after the global ones
    (core/makemultimages_main.cpp:266-300): image 2's output is the oracle's
    model of the global Gaussian moved and scaled plus its sky and star."""
    from imfit_gb300 import cli
    data, _, _, _ = _per_image_setup(oracle_mod)
    g, d2, l2 = PER_IMAGE_TRUTH["global_"], PER_IMAGE_TRUTH["desc2"], PER_IMAGE_TRUTH["local2"]
    cfg = "\n".join(f"{k} {v}" for k, v in zip(["X0", "Y0"], g[:2])) + "\nFUNCTION Gaussian\n" + \
        "\n".join(f"{k} {v}" for k, v in zip(["PA", "ell", "I_0", "sigma"], g[2:])) + "\n"
    local = PER_IMAGE_LOCAL.replace("I_sky 5.0 0,20", f"I_sky {l2[2]}").replace("I_0 80 20,200", f"I_0 {l2[7]}")
    (tmp_path / "c.dat").write_text(cfg)
    (tmp_path / "info.txt").write_text(f"""IMAGE_START
NCOLS 44
NROWS 40
IMAGE_START
NCOLS 44
NROWS 40
PIXEL_SCALE {d2[0]} fixed
IMAGE_PA {d2[1]} fixed
FLUX_SCALE {d2[2]} fixed
X0 {d2[3]}
Y0 {d2[4]}
""" + local)
    imgs = cli.makemultimages([str(tmp_path / "c.dat"), "-i", str(tmp_path / "info.txt"), "-o", str(tmp_path / "m")],
                              out=io.StringIO())
    for img, want in zip(imgs, data):
        assert np.max(np.abs(img - want)) <= 1e-10 * np.max(np.abs(want))
