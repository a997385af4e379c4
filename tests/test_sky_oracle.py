"""Host checks of the correlated-field log-sky: the padded-grid size, the
Fourier-mode distributor, and the oracle's Hartley transform and hand-written
vector-Jacobian products."""
import numpy as np
import pytest

import sky_oracle as SO
from jubik_gb300 import sky as jsky


def test_good_fft_size_matches_the_reference_padding():
    # eROSITA/JWST demo configs: s_padding_ratio 1.1075 "leads to a 1134,
    # which is a 'good size' padded space" (demos/configs/eROSITA_demo.yaml:50)
    assert jsky.good_fft_size(int(1024 * 1.1075)) == 1134
    assert jsky.good_fft_size(int(512 * 1.1075)) == 567
    # the reference's own sky-model test grid (test/test_sky_model.py:55-58)
    assert jsky.good_fft_size(int(128 * 1.1)) == 140
    assert jsky.good_fft_size(1025) == 1029  # 3 * 7^3
    assert jsky.good_fft_size(13) == 14
    for n in range(1, 2500):
        assert jsky.good_fft_size(n) == SO.good_size(n)
    with pytest.raises(ValueError):
        jsky.good_fft_size(0)


def test_mode_distributor_known_answer():
    pidx, um, cnt = jsky.fourier_mode_distributor((4,), 1.0)
    np.testing.assert_array_equal(pidx, [0, 1, 2, 1])
    np.testing.assert_allclose(um, [0.0, 0.25, 0.5])
    np.testing.assert_array_equal(cnt, [1, 2, 1])


@pytest.mark.parametrize("shape,dist", [((9,), 0.3), ((6, 10), (1.0, 0.5)), ((16, 16), 1.0),
                                        ((12, 20), 0.25)])
def test_mode_distributor_matches_oracle(shape, dist):
    pidx, um, cnt = jsky.fourier_mode_distributor(shape, dist)
    p2, u2, c2 = SO.mode_distributor(shape, dist)
    np.testing.assert_array_equal(pidx, p2)
    np.testing.assert_allclose(um, u2, rtol=1e-15, atol=0)  # 1/(n d) vs division by n d
    np.testing.assert_array_equal(cnt, c2)
    assert cnt.sum() == np.prod(shape)


def test_mode_distributor_merges_equal_lengths():
    # (3, 4) and (5, 0) have the same length on a square grid
    pidx, um, _ = jsky.fourier_mode_distributor((16, 16), 1.0)
    assert pidx[3, 4] == pidx[5, 0] == pidx[4, 3] == pidx[0, 5]
    assert np.all(np.diff(um) > 0)


def test_hartley_is_symmetric_and_self_inverse():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((6, 10))
    y = rng.standard_normal((6, 10))
    np.testing.assert_allclose(SO.hartley(SO.hartley(x)), x.size * x, rtol=1e-12, atol=1e-10)
    assert abs(np.vdot(SO.hartley(x), y) - np.vdot(x, SO.hartley(y))) < 1e-10


def test_oracle_vjp_by_adjoint_identity_and_finite_differences():
    rng = np.random.default_rng(1)
    shape, nf = (8, 12), 2
    pidx, um, _ = jsky.fourier_mode_distributor(shape, (1.0, 0.5))
    amp = rng.uniform(0.5, 2.0, (nf, um.size))
    xi = rng.standard_normal((nf,) + shape)
    off = rng.standard_normal(nf)
    coef = np.stack([np.ones(3), SO.log_rel_ebin_centers([0.2, 1.0, 2.0], [1.0, 2.0, 4.5], 2.0)], 1)
    crop = (6, 9)

    def f(a, x, o):
        return SO.logsky(SO.fields(a, x, o, pidx), coef, crop)

    g = rng.standard_normal((3,) + crop)
    gf = SO.logsky_cotangent_to_fields(g, coef, shape)
    dxi, damp, doff = SO.fields_vjp(amp, xi, pidx, gf)
    # the map is linear in xi and in the offsets: <J v, g> = <v, J^T g>
    v = rng.standard_normal(xi.shape)
    jv = f(amp, v, np.zeros(nf)) - f(amp, 0 * v, np.zeros(nf))
    assert abs(np.vdot(jv, g) - np.vdot(v, dxi)) < 1e-9 * abs(np.vdot(v, dxi))
    # offsets and amplitudes by central differences
    h = 1e-6
    for b in range(nf):
        e = np.zeros(nf)
        e[b] = h
        fd = np.vdot(f(amp, xi, off + e) - f(amp, xi, off - e), g) / (2 * h)
        assert abs(fd - doff[b]) < 1e-6 * max(1.0, abs(doff[b]))
        for m in (0, 3, um.size - 1):
            da = np.zeros_like(amp)
            da[b, m] = h
            fd = np.vdot(f(amp + da, xi, off) - f(amp - da, xi, off), g) / (2 * h)
            assert abs(fd - damp[b, m]) < 1e-6 * max(1.0, abs(damp[b, m]))


def test_diffuse_coefficients():
    c = jsky.diffuse_coefficients([0.2, 1.0, 2.0], [1.0, 2.0, 4.5], 2.0)
    np.testing.assert_allclose(c[:, 0], 1.0)
    np.testing.assert_allclose(c[:, 1], 0.5 * np.log([0.2, 2.0, 9.0]) - np.log(2.0), rtol=1e-15)
    assert jsky.diffuse_coefficients([1.0], [2.0], 1.0, plaw=False).shape == (1, 1)


def test_pair_packed_hartley_identity():
    """The identity the correlated-field kernels use to take two real fields
    through one complex transform: with Z = fftn(x0 + i x1) and Zm(k) = Z(-k),
    H x0 = (Re Z + Re Zm + Im Z - Im Zm) / 2 and
    H x1 = (Im Z + Im Zm + Re Zm - Re Z) / 2."""
    rng = np.random.default_rng(5)
    for shape in [(6, 10), (9, 7), (1, 12), (1134, 3)]:
        x0, x1 = rng.standard_normal(shape), rng.standard_normal(shape)
        Z = np.fft.fftn(x0 + 1j * x1)
        Zm = np.roll(np.flip(Z), 1, axis=(0, 1))  # Z at (-k0, -k1) mod the grid
        h0 = 0.5 * ((Z.real + Zm.real) + (Z.imag - Zm.imag))
        h1 = 0.5 * ((Z.imag + Zm.imag) + (Zm.real - Z.real))
        np.testing.assert_allclose(h0, SO.hartley(x0), rtol=0, atol=1e-10 * np.abs(Z).max())
        np.testing.assert_allclose(h1, SO.hartley(x1), rtol=0, atol=1e-10 * np.abs(Z).max())
