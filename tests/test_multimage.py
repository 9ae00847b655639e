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
