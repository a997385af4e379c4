"""Host checks of the PSF-patch interpolation oracle."""
import numpy as np
import pytest
from scipy import ndimage

import psf_oracle as PO
from jubik_gb300 import psf as jpsf
from jubik_gb300 import synthetic


def test_radial_weights_known_answers():
    rs = np.array([0.0, 2.0, 6.0])
    np.testing.assert_allclose(PO.interpolation_weights(rs, -1.0), [1, 0, 0])
    np.testing.assert_allclose(PO.interpolation_weights(rs, 1.0), [0.5, 0.5, 0])
    np.testing.assert_allclose(PO.interpolation_weights(rs, 5.0), [0, 0.25, 0.75])
    np.testing.assert_allclose(PO.interpolation_weights(rs, 9.0), [0, 0, 1])
    # at exactly the last radius the clamp and the last interval both count
    np.testing.assert_allclose(PO.interpolation_weights(rs, 6.0), [0, 0, 2])
    for r in (-1.0, 1.0, 5.0, 6.0, 9.0):
        np.testing.assert_array_equal(jpsf.get_interpolation_weights(rs, r),
                                      PO.interpolation_weights(rs, r))


def test_polar_round_trip():
    rng = np.random.default_rng(0)
    cc = rng.normal(size=(100, 2))
    np.testing.assert_allclose(PO.to_ra_dec(PO.to_r_phi(cc)), cc, atol=1e-14)
    np.testing.assert_allclose(jpsf.to_ra_dec(jpsf.to_r_phi(cc)), cc, atol=1e-14)
    # the angle is measured from the second axis
    np.testing.assert_allclose(PO.to_r_phi([0.0, 1.0]), [1.0, 0.0], atol=1e-15)


def test_bilinear_nearest_matches_scipy():
    rng = np.random.default_rng(1)
    img = rng.normal(size=(9, 7))
    q0 = rng.uniform(-3, 12, 500)
    q1 = rng.uniform(-3, 10, 500)
    ref = ndimage.map_coordinates(img, [q0, q1], order=1, mode="nearest")
    np.testing.assert_allclose(PO.bilinear_nearest(img, q0, q1), ref, rtol=1e-12, atol=1e-14)


def test_interpolator_patch_order_and_roll():
    infos = synthetic.erosita_like_psf_infos(n_energies=1, field=(32, 32))
    out = PO.psf_interpolator((1, 32, 32), (1.0, 1.0, 1.0), 4, infos)
    assert out.shape == (16, 1, 32, 32)
    # the PSF peak of every patch sits at the rolled origin
    for k in range(16):
        i = np.unravel_index(np.argmax(out[k, 0]), (32, 32))
        d = [min(v, 32 - v) for v in i]
        assert max(d) <= 2
    # patch k's centre: dec along k % n, ra reversed along k // n
    c_ra, c_dec = PO.patch_centres((32, 32), (1.0, 1.0), 4)
    assert c_dec[1] > c_dec[0] and c_ra[4] < c_ra[0]
    with pytest.raises(ValueError):
        PO.psf_interpolator((1, 30, 30), (1.0, 1.0, 1.0), 4, infos)
