"""Pin the CPU oracle against the reference's own known-answer tests and
self-consistency properties (no GPU).

Ported assertions: test/test_convolve.py, test/test_slice_patches.py,
test/test_build_exposure_function.py, test/test_build_exposure_readout_function.py,
test/test_utils.py:66-68.
"""
import os
import sys

import numpy as np
import pytest

import jubik_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)


# ---- test/test_convolve.py
def test_bilinear_weights_even_shape_properties():
    w = O.bilinear_weights((4, 4))
    assert w.shape == (4, 4)
    assert np.isfinite(w).all() and np.all(w >= 0)
    np.testing.assert_allclose(w, w[::-1, :])
    np.testing.assert_allclose(w, w[:, ::-1])


def test_bilinear_weights_odd_shape_raises():
    with pytest.raises(ValueError):
        O.bilinear_weights((3, 3))


def test_integrate_constant_field_exact():
    res = O.integrate(np.ones((3, 4)), O.Domain((3, 4), (0.5, 0.25)), axes=(0, 1))
    assert res == pytest.approx(3 * 4 * 0.5 * 0.25)


def test_convolve_identity_kernel_returns_input_for_unit_cell_volume():
    rng = np.random.default_rng(0)
    signal = rng.normal(size=(4, 4))
    kernel = np.zeros((4, 4))
    kernel[0, 0] = 1.0
    res = O.convolve(kernel, signal, O.Domain((4, 4), (1.0, 1.0)), axes=(-2, -1))
    np.testing.assert_allclose(res, signal, rtol=1e-10, atol=1e-10)


def test_convolve_broadcasting_branch_prints_and_preserves_channel_shape(capsys):
    kernel = np.zeros((4, 4))
    kernel[0, 0] = 1.0
    signal = np.stack([np.ones((4, 4)), 2.0 * np.ones((4, 4))])
    res = O.convolve(kernel, signal, O.Domain((4, 4), (1.0, 1.0)), axes=(-2, -1))
    assert "Dimension Inconsistency. Broadcasting PSFs" in capsys.readouterr().out
    assert res.shape == signal.shape
    np.testing.assert_allclose(res, signal, rtol=1e-10, atol=1e-10)


# ---- test/test_slice_patches.py
SHAPE, NP, OVL = (36, 36), 16, 2


def test_slice_patches_shape():
    x = np.arange(36 * 36, dtype=float).reshape(SHAPE)
    s = O.slice_patches(x, SHAPE, NP, OVL)
    dx = int((SHAPE[0] - 2 * OVL) / NP)
    assert s.shape == (NP ** 2, 2 * dx + 2 * OVL, 2 * dx + 2 * OVL)
    assert np.isfinite(s).all()


def test_slice_patches_linearity():
    rng = np.random.default_rng(0)
    a, b = rng.normal(size=SHAPE), rng.normal(size=SHAPE)
    f = lambda v: O.slice_patches(v, SHAPE, NP, OVL)  # noqa: E731
    np.testing.assert_allclose(f(a + b), f(a) + f(b))


def test_slice_patches_adjointness():
    rng = np.random.default_rng(1)
    a = rng.random(SHAPE)
    res = O.slice_patches(a, SHAPE, NP, OVL)
    b = rng.random(res.shape)
    np.testing.assert_allclose(np.vdot(b, res),
                               np.vdot(O.slice_patches_adjoint(b, SHAPE, NP, OVL), a))


def test_slice_patches_order_matches_coord_center():
    # patch k is centred on coord_center's k-th index (jubik/utils.py:185-207)
    N, n = 32, 4
    x = np.arange(N * N, dtype=float).reshape(N, N)
    s = O.slice_patches(x, (N, N), n, 0)
    dx = N // n
    cc = O.coord_center(N, n)
    np.testing.assert_array_equal(s[:, dx, dx], x.reshape(-1)[cc] + 0 * cc)


# ---- test/test_utils.py:66-68
def test_coord_center_small_grid():
    np.testing.assert_array_equal(O.coord_center(4, 2), np.array([5, 13, 7, 15]))


# ---- test/test_build_exposure_function.py
@pytest.fixture
def exposures():
    return np.random.default_rng(0).uniform(0.0, 3e3, size=3 * 100 ** 2).reshape((3, 100, 100))


def test_build_exposure_applies_threshold_and_multiplies_input(exposures):
    x = np.linspace(0.25, 1.75, num=100 * 100).reshape(100, 100)
    result = O.build_exposure_function(exposures.copy(), 500)(x)
    expected = exposures.copy()
    expected[expected < 500] = 0
    np.testing.assert_allclose(result, expected * x)
    assert (result >= 0).all()


def test_build_exposure_negative_cut_raises(exposures):
    with pytest.raises(ValueError):
        O.build_exposure_function(exposures.copy(), -1)


# ---- test/test_build_exposure_readout_function.py
def test_readout_order_and_errors():
    rng = np.random.default_rng(0)
    exp = rng.uniform(0.0, 3e3, size=2 * 24 ** 2 * 3).reshape((2, 3, 24, 24))
    x = np.arange(2 * 3 * 24 * 24, dtype=float).reshape((2, 3, 24, 24)) + 0.5
    flags = exp.copy()
    mask = flags < 20
    res = O.build_readout_function(flags, 20, ("tm_1", "tm_2"))(x)
    assert tuple(res.keys()) == ("tm_1", "tm_2")
    for i, k in enumerate(("tm_1", "tm_2")):
        np.testing.assert_array_equal(res[k], x[i][~mask[i]])
    with pytest.raises(ValueError):
        O.build_readout_function(exp.copy(), 20, ("tm_1", "tm_2"))(x[0])
    with pytest.raises(ValueError):
        O.build_readout_function(exp.copy(), -1, ("tm_1", "tm_2"))
    with pytest.raises(ValueError):
        O.build_readout_function(exp.copy(), 20, ("tm_1",))
    with pytest.raises(ValueError, match="flags should have shape"):
        O.build_readout_function(np.ones((1, 4, 4)), None, ("tm_1",))(np.ones((1, 2, 4, 4)))


# ---- self-consistency of the restated linpatch_convolve
def _case(seed=0, E=2, N=48, n=3, m=8):
    rng = np.random.default_rng(seed)
    dx = N // n
    K = 2 * dx
    return rng, O.Domain((E, N, N), (1.0, 0.5, 0.5)), rng.random((n * n, E, K, K)), n, m, dx


def test_linpatch_adjoint_identity():
    rng, dom, ker, n, m, _ = _case()
    x, g = rng.random(dom.shape), rng.random(dom.shape)
    y = O.linpatch_convolve(x, dom, ker, n, m, precut=True)
    z = O.linpatch_convolve_adjoint(g, dom, ker, n, m, precut=True)
    np.testing.assert_allclose(np.vdot(g, y), np.vdot(z, x), rtol=1e-12)


def test_linpatch_full_kernel_equals_precut():
    rng, dom, ker, n, m, dx = _case()
    N = dom.shape[-1]
    K = 2 * dx
    full = np.zeros(ker.shape[:2] + (N, N))
    a = (np.arange(K) - dx) % N
    full[..., a[:, None], a[None, :]] = ker
    np.testing.assert_array_equal(O.cut_kernel(full, dom.shape, n), ker)
    x = rng.random(dom.shape)
    np.testing.assert_array_equal(O.linpatch_convolve(x, dom, full, n, m),
                                  O.linpatch_convolve(x, dom, ker, n, m, precut=True))


def test_linpatch_delta_psf_is_identity_in_interior():
    rng, dom, ker, n, m, dx = _case()
    d = np.zeros_like(ker)
    d[..., dx, dx] = 1.0
    x = rng.random(dom.shape)
    y = O.linpatch_convolve(x, dom, d, n, m, precut=True)
    h = dx // 2
    np.testing.assert_allclose(y[:, h:-h, h:-h], x[:, h:-h, h:-h], rtol=1e-12, atol=1e-14)


def test_linpatch_kernel_scale_invariance():
    # kernels are renormalised per (patch, energy), convolve.py:126-131
    rng, dom, ker, n, m, _ = _case()
    x = rng.random(dom.shape)
    s = rng.uniform(0.5, 2.0, size=ker.shape[:2])[..., None, None]
    np.testing.assert_allclose(O.linpatch_convolve(x, dom, ker * s, n, m, precut=True),
                               O.linpatch_convolve(x, dom, ker, n, m, precut=True), rtol=1e-12)


def test_response_gradient_central_fd():
    rng, dom, ker, n, m, _ = _case(E=1, N=32, n=2, m=4)
    M = 2
    kernel = np.stack([ker, ker[::-1]])
    exp = rng.uniform(500, 1500, size=(M,) + dom.shape)
    rm = rng.random((M,) + dom.shape) > 0.05
    R = O.Response(dom, kernel, n, m, exp, rm, pixel_area=0.5)
    x = np.exp(rng.normal(size=dom.shape))
    data = [rng.poisson(l) for l in R(x)]
    e0, g = R.energy_and_grad(x, data)
    for _ in range(4):
        v = rng.normal(size=x.shape)
        eps = 1e-4
        ep, _ = R.energy_and_grad(x + eps * v, data)
        em, _ = R.energy_and_grad(x - eps * v, data)
        np.testing.assert_allclose((ep - em) / (2 * eps), np.vdot(g, v), rtol=1e-6)


# ---- committed golden fixtures (generated by tests/golden/make_golden.py)
def test_golden_fixtures_reproduce():
    import make_golden  # noqa: E402

    for name, fn in make_golden.CASES.items():
        ref = np.load(os.path.join(GOLDEN, name + ".npz"))
        got = fn()
        assert set(ref.files) == set(got)
        for k in ref.files:
            np.testing.assert_allclose(got[k], ref[k], rtol=1e-12, atol=1e-300, err_msg=name + k)


# ---- two independent restatements agree (numpy FFT vs direct C convolution)
@pytest.mark.parametrize("E,N,n,m", [(2, 48, 3, 8), (1, 21, 3, 2), (1, 36, 16, 2),
                                     (2, 40, 4, 5), (1, 64, 4, 24)])
def test_fft_oracle_matches_direct_c_restatement(E, N, n, m):
    import subprocess
    subprocess.run(["make", "-s", "-C", os.path.dirname(O.__file__)], check=True)
    rng = np.random.default_rng(E * 1000 + N)
    dx = N // n
    x = rng.random((E, N, N))
    k = rng.random((n * n, E, 2 * dx, 2 * dx))
    a = O.linpatch_convolve(x, O.Domain((E, N, N), (1.0, 1.0, 1.0)), k, n, m, precut=True)
    b = O.linpatch_direct_c(x, k, n, m)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-14 * np.abs(a).max())
