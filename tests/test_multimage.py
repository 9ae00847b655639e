"""CPU tests of the multi-image parameter transform (core/param_holder.cpp,
core/paramvector_processing.cpp) and the image-info file format
(core/imageparams_file_parser.cpp)."""
import numpy as np
import pytest

from imfit_gb300 import multimage


class FakeHandle:
    def __init__(self, n):
        self.n_params = n


FUNCS = [("Sersic", True), ("Exponential", False), ("Gaussian", True), ("FlatSky", False)]
# X0 Y0 | Sersic PA ell n I_e r_e | Exp PA ell I_0 h | X0 Y0 | Gauss PA ell I_0 sigma | FlatSky I_sky
MODEL = [50.0, 40.0, 30.0, 0.3, 2.0, 10.0, 5.0, 35.0, 0.4, 3.0, 20.0, 60.0, 45.0, 10.0, 0.1, 100.0, 2.0, 7.0]


def _mm(n_images=2):
    return multimage.MultiImageModel(FUNCS, [FakeHandle(len(MODEL))] * n_images)


def test_reference_image_is_the_model_itself():
    mm = _mm()
    p = np.array([0.5, 12.0, 2.0, 20.0, 25.0] + MODEL)
    assert np.array_equal(mm.image_vector(p, 0), np.array(MODEL))


def test_second_image_transform():
    """First set at the image's (X0, Y0); later sets offset by the rotated,
    scaled reference offset (CalculateOffset_X0Y0); PA - IMAGE_PA, intensities
    x FLUX_SCALE, sizes / PIXEL_SCALE (each class's Setup)."""
    mm = _mm()
    ps, rot, fs, x0i, y0i = 0.5, 12.0, 2.0, 20.0, 25.0
    v = mm.image_vector(np.array([ps, rot, fs, x0i, y0i] + MODEL), 1)
    t = np.deg2rad(rot)
    dx, dy = 60.0 - 50.0, 45.0 - 40.0
    assert v[0] == x0i and v[1] == y0i
    assert np.isclose(v[11], x0i + ps * (dx * np.cos(t) + dy * np.sin(t)))
    assert np.isclose(v[12], y0i + ps * (-dx * np.sin(t) + dy * np.cos(t)))
    assert v[2] == 30.0 - rot and v[5] == 10.0 * fs and v[6] == 5.0 * (1.0 / ps)
    assert v[7] == 35.0 - rot and v[9] == 3.0 * fs and v[10] == 20.0 * (1.0 / ps)
    assert v[13] == 10.0 - rot and v[15] == 100.0 * fs and v[16] == 2.0 * (1.0 / ps)
    assert v[17] == 7.0 * fs and v[3] == 0.3 and v[4] == 2.0


def test_transform_jacobian_matches_the_analytic_one():
    mm = _mm()
    p = np.array([0.5, 12.0, 2.0, 20.0, 25.0] + MODEL)
    T = mm.transform_jacobian(p, 1)
    assert T.shape == (len(MODEL), 5 + len(MODEL))
    assert np.isclose(T[6, 0], -5.0 / 0.25) and np.isclose(T[5, 2], 10.0) and np.isclose(T[2, 1], -1.0)
    t = np.deg2rad(12.0)
    assert np.isclose(T[11, 5 + 11], 0.5 * np.cos(t)) and np.isclose(T[11, 5 + 0], -0.5 * np.cos(t))
    assert np.isclose(T[0, 3], 1.0) and T[0, 5] == 0.0


def test_image_info_parser():
    text = """# comment
IMAGE_START
DATA    ref.fits
ERROR   ref_sig.fits
ORIGINAL_SKY   100.0
IMAGE_START
DATA  second.fits
MASK  second_mask.fits
MASK_ZERO_IS_BAD
GAIN  4.5
PIXEL_SCALE   1.0   fixed
IMAGE_PA      5.0   0,10
X0   20
"""
    ims = multimage.parse_image_info(text)
    assert len(ims) == 2 and ims[0].data == "ref.fits" and ims[0].error == "ref_sig.fits"
    assert ims[0].options["ORIGINAL_SKY"] == "100.0"
    assert ims[1].mask == "second_mask.fits" and "MASK_ZERO_IS_BAD" in ims[1].flags
    assert ims[1].params["PIXEL_SCALE"][3] and ims[1].params["IMAGE_PA"][1:3] == (0.0, 10.0)
    assert ims[1].params["X0"][0] == 20.0
    with pytest.raises(ValueError):
        multimage.parse_image_info("DATA x.fits\n")


PER_IMAGE_INFO = """IMAGE_START
DATA  ref.fits
IMAGE_START
DATA  second.fits
PIXEL_SCALE   0.5   fixed
X0   20
Y0   25
FUNCTIONS_START
X0   10   5,15
Y0   12
FUNCTION PointSource   # LABEL star
I_tot   300   fixed
X0   30
Y0   31
FUNCTION FlatSky
I_sky   4.0
IMAGE_START
DATA  third.fits
"""


def test_image_info_per_image_functions():
    """FUNCTIONS_START ends an image's own lines; the rest of its block is a
    function section (core/imageparams_file_parser.cpp:531-547, 626-650)."""
    ims = multimage.parse_image_info(PER_IMAGE_INFO)
    assert len(ims) == 3 and ims[0].local is None and ims[2].local is None and ims[2].data == "third.fits"
    loc = ims[1].local
    assert ims[1].params["X0"][0] == 20.0 and ims[1].data == "second.fits"
    assert loc.functions == [("PointSource", True), ("FlatSky", True)]
    assert loc.labels[0] == "star"
    assert list(loc.values) == [10.0, 12.0, 300.0, 30.0, 31.0, 4.0]
    assert loc.lower[0] == 5.0 and loc.upper[0] == 15.0 and loc.fixed[2] == 1
    with pytest.raises(ValueError):
        multimage.parse_image_info("IMAGE_START\nDATA a.fits\nFUNCTIONS_START\n")


def test_per_image_parameters_follow_the_global_model():
    """[image descriptions][global model][image 1 locals][image 2 locals] ...;
    locals copied unchanged after the transformed global model
    (core/param_holder.cpp:257-268), not scaled by the image description."""
    cfg_values = list(MODEL)
    ims = multimage.parse_image_info(PER_IMAGE_INFO)
    local = [im.local_functions for im in ims]
    handles = [FakeHandle(len(MODEL)), FakeHandle(len(MODEL) + 6), FakeHandle(len(MODEL))]
    mm = multimage.MultiImageModel(FUNCS, handles, local)
    assert mm.n_local == [0, 6, 0] and mm.n_params == 10 + len(MODEL) + 6
    desc = [0.5, 12.0, 2.0, 20.0, 25.0, 1.0, 0.0, 1.0, 50.0, 40.0]
    loc = [10.0, 12.0, 300.0, 30.0, 31.0, 4.0]
    p = np.array(desc + cfg_values + loc)
    v1 = mm.image_vector(p, 1)
    assert len(v1) == len(MODEL) + 6 and list(v1[len(MODEL):]) == loc
    assert v1[5] == 10.0 * 2.0  # global intensity still scaled
    assert np.array_equal(mm.image_vector(p, 2), np.array(MODEL))
    T = mm.transform_jacobian(p, 1)
    assert T.shape == (len(MODEL) + 6, len(p))
    assert np.array_equal(T[len(MODEL):, mm.local_slice(1)], np.eye(6))
    assert np.all(T[:len(MODEL), mm.local_slice(1)] == 0) and np.all(T[len(MODEL):, :mm.local_slice(1).start] == 0)
    with pytest.raises(ValueError):
        multimage.MultiImageModel(FUNCS, [FakeHandle(len(MODEL))] * 3, local)


def test_global_vector_and_names_with_per_image_functions():
    from imfit_gb300.config import parse_config
    cfg = parse_config("X0 50 40,60\nY0 40\nFUNCTION FlatSky\nI_sky 7\n")
    ims = multimage.parse_image_info(PER_IMAGE_INFO)
    vals, lo, hi, fx = multimage.global_vector(cfg, ims)
    assert len(vals) == 10 + 3 + 6
    assert list(vals[13:]) == [10.0, 12.0, 300.0, 30.0, 31.0, 4.0]
    assert lo[13] == 5.0 and hi[13] == 15.0 and fx[15] == 1
    names = multimage.parameter_names(cfg, ims)
    assert names[0] == "PIXEL_SCALE_2" and names[10] == "X0" and names[13] == "X0_2" and names[-1] == "I_sky_2"
