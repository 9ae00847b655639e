"""GPU edge cases of image and PSF geometry against the oracle: non-square
images with even, non-square PSFs (ShiftAndWrapPSF's centre at floor(P/2),
core/convolver.cpp:421-441), single-row and single-column images, a 1 x 1 PSF,
and an oversampled region clipped at the image border
(ModelObject::AddOversampledPsfInfo, core/model_object.cpp:881-952)."""
import numpy as np
import pytest

from helpers import normwise, relerr

pytestmark = pytest.mark.gpu

FUNCS = [("Sersic", True), ("Exponential", False), ("FlatSky", False)]


def _psf(nc, nr, fwhm=2.5, dx=0.3):
    yy, xx = np.mgrid[0:nr, 0:nc].astype(float)
    yy -= (nr - 1) / 2.0
    xx -= (nc - 1) / 2.0 + dx
    a = fwhm / (2.0 * np.sqrt(2.0 ** (1.0 / 3.0) - 1.0))
    return (1.0 + (xx ** 2 + yy ** 2) / a ** 2) ** -3.0


def _params(nc, nr):
    return np.array([nc / 2.0 + 0.3, nr / 2.0 - 0.2, 35.0, 0.3, 1.6, 25.0, 4.0, 110.0, 0.45, 8.0, 6.0, 12.0])


def _data(oracle_mod, nc, nr, psf, region, seed):
    """Poisson data drawn around the oracle's model image."""
    m = oracle_mod.OracleModel()
    for name, new_set in FUNCS:
        m.add_function(name, new_set)
    m.finish_functions()
    if psf is not None:
        m.add_psf(psf)
    m.setup_model_image(nc, nr)
    if region is not None:
        m.add_oversampled_psf(_psf(3 * 7, 3 * 7, fwhm=7.5), 3, region)
    m.create_model_image(_params(nc, nr))
    rng = np.random.default_rng(seed)
    return rng.poisson(np.clip(m.get_model_image(), 0, None) + 15.0).astype(float) - 15.0


def _pair(gpu, oracle_mod, nc, nr, psf=None, region=None, seed=1):
    data = _data(oracle_mod, nc, nr, psf, region, seed)
    hs = []
    for cls in (oracle_mod.OracleModel, gpu.ModelObject):
        m = cls()
        for name, new_set in FUNCS:
            m.add_function(name, new_set)
        m.finish_functions()
        if psf is not None:
            m.add_psf(psf)
        m.add_image_data(data)
        if region is not None:
            m.add_oversampled_psf(_psf(3 * 7, 3 * 7, fwhm=7.5), 3, region)
        m.add_image_characteristics(2.0, 3.0, 1.0, 1, 15.0)
        assert m.final_setup() == 0
        hs.append(m)
    return hs, _params(nc, nr)


@pytest.mark.parametrize("nc,nr,pc,pr", [(41, 27, 6, 9), (30, 44, 8, 4), (50, 1, 1, 1), (1, 40, 1, 1),
                                         (33, 21, 1, 1), (25, 25, 2, 2)])
def test_geometry_parity(gpu, oracle_mod, nc, nr, pc, pr):
    """Plain path within 1e-10 of the oracle (image, statistic); fast path
    statistic within 1e-5 and its gradient against the FP64 differences."""
    psf = _psf(pc, pr) if pc * pr > 1 else np.ones((1, 1))
    (o, g), p = _pair(gpu, oracle_mod, nc, nr, psf)
    so, sg = o.get_fit_statistic(p), g.get_fit_statistic(p)
    assert relerr(sg, so) < 1e-10, (sg, so)
    assert normwise(g.get_model_image(), o.get_model_image()) < 1e-10
    s, grad = g.statistic_and_gradient(p)
    _, gfd = g.statistic_and_gradient_fd(p)
    assert relerr(s, sg) < 1e-5, (s, sg)
    top = np.max(np.abs(gfd))
    assert np.all(np.abs(grad - gfd) <= 3e-3 * np.abs(gfd) + 1e-3 * top), (grad, gfd)


def test_unit_psf_is_the_identity(gpu, oracle_mod):
    """A 1 x 1 PSF: the convolved model equals the unconvolved one."""
    p = _params(31, 23)
    imgs = []
    for psf in (None, np.ones((1, 1))):
        m = gpu.ModelObject()
        for name, new_set in FUNCS:
            m.add_function(name, new_set)
        m.finish_functions()
        if psf is not None:
            m.add_psf(psf)
        m.setup_model_image(31, 23)
        m.create_model_image(p)
        imgs.append(m.get_model_image())
    assert normwise(imgs[1], imgs[0]) < 1e-12


def test_region_clipped_at_the_border(gpu, oracle_mod):
    """An oversampled region reaching past the image's left and top edges is
    clipped as the reference clips it; the plain path matches the oracle and
    the fast path either matches or declines with an error."""
    (o, g), p = _pair(gpu, oracle_mod, 40, 32, _psf(7, 7), region=(-3, 9, 25, 40))
    so, sg = o.get_fit_statistic(p), g.get_fit_statistic(p)
    assert relerr(sg, so) < 1e-10, (sg, so)
    try:
        s, grad = g.statistic_and_gradient(p)
    except gpu.ImfitError:
        return
    assert relerr(s, sg) < 1e-5 and np.all(np.isfinite(grad))
