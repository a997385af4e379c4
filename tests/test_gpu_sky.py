"""Correlated-field log-sky on the GPU (jubik_cf_*): fields, the diffuse
log-sky (spatial + spectral index x log energy centres, cropped) and their
vector-Jacobian products against the float64 oracle, and the chain into the
response's Poisson energy."""
import numpy as np
import pytest
import torch

import jubik_oracle as O
import sky_oracle as SO
import jubik_gb300 as ju
from jubik_gb300 import sky as jsky
from jubik_gb300 import synthetic

pytestmark = pytest.mark.gpu

EMIN, EMAX, EREF = [0.2, 1.0, 2.0], [1.0, 2.0, 4.5], 2.0


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_inputs(sky, seed, slope=-2.0):
    rng = np.random.default_rng(seed)
    k = sky.mode_lengths / max(sky.mode_lengths[-1], 1e-300)
    base = (1.0 + (k / 0.05) ** 2) ** (slope / 2)
    amp = np.stack([base * rng.uniform(0.5, 1.5) / np.sqrt(sky.pindex.size)
                    for _ in range(sky.n_fields)])
    xi = rng.standard_normal((sky.n_fields,) + sky.shape)
    off = rng.normal(0.0, 0.5, sky.n_fields)
    return amp, xi, off


def T(a, dtype, dev):
    return torch.as_tensor(np.asarray(a), device=dev).to(dtype)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
# FFT radices: 96 = 8.4.3, 80 = 8.2.5, 70 = 2.5.7, 88 = 8.11, 99 = 9.11,
# 1134 = 2.9.9.7, 200 = 8.5.5; 26 = 2.13 and 34 = 2.17 take the generic radix
@pytest.mark.parametrize("shape,nf", [((96, 80), 1), ((96, 80), 2), ((48, 70), 3),
                                      ((64, 64), 4), ((88, 99), 1), ((26, 34), 2),
                                      ((1134, 1134), 2), ((200,), 2)])
def test_fields_and_vjp_match_oracle(cuda, dtype, shape, nf):
    sky = jsky.CorrelatedFieldSky(shape, 0.5, n_fields=nf, dtype=dtype)
    try:
        amp, xi, off = make_inputs(sky, 3 + nf)
        p = sky.pindex
        ref = SO.fields(amp, xi.reshape((nf,) + sky.shape), off, p)
        got = sky.fields(T(amp, dtype, cuda), T(xi, dtype, cuda), T(off, dtype, cuda))
        tol = 1e-12 if dtype == torch.float64 else 1e-6
        assert rel(got, ref) < tol
        g = np.random.default_rng(9).standard_normal((nf,) + sky.shape)
        dxi, damp, doff = sky.vjp(T(amp, dtype, cuda), T(xi, dtype, cuda),
                                  g_fields=T(g, dtype, cuda))
        rx, ra, ro = SO.fields_vjp(amp, xi.reshape((nf,) + sky.shape), p, g)
        assert rel(dxi, rx) < tol
        assert rel(damp, ra) < (tol if dtype == torch.float64 else 2e-6)
        assert rel(doff, ro) < tol
        # no atomics: a second call is bitwise identical
        dxi2, damp2, doff2 = sky.vjp(T(amp, dtype, cuda), T(xi, dtype, cuda),
                                     g_fields=T(g, dtype, cuda))
        assert torch.equal(dxi, dxi2) and torch.equal(damp, damp2) and torch.equal(doff, doff2)
    finally:
        sky.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_diffuse_logsky_and_vjp_match_oracle(cuda, dtype):
    shape, crop = (140, 126), (128, 120)
    coef = jsky.diffuse_coefficients(EMIN, EMAX, EREF)
    sky = jsky.CorrelatedFieldSky(shape, (1.0, 1.0), n_fields=2, crop=crop, coefficients=coef,
                                  dtype=dtype)
    try:
        amp, xi, off = make_inputs(sky, 5)
        flds = SO.fields(amp, xi, off, sky.pindex)
        ref = SO.logsky(flds, coef, crop)
        fo = torch.empty((2,) + shape, dtype=dtype, device=cuda)
        got = sky.logsky(T(amp, dtype, cuda), T(xi, dtype, cuda), T(off, dtype, cuda),
                         fields_out=fo)
        tol = 1e-12 if dtype == torch.float64 else 1e-6
        assert got.shape == (3,) + crop
        assert rel(got, ref) < tol and rel(fo, flds) < tol
        g = np.random.default_rng(2).standard_normal((3,) + crop)
        dxi, damp, doff = sky.vjp(T(amp, dtype, cuda), T(xi, dtype, cuda), g_logsky=T(g, dtype, cuda))
        rx, ra, ro = SO.fields_vjp(amp, xi, sky.pindex, SO.logsky_cotangent_to_fields(g, coef, shape))
        assert rel(dxi, rx) < tol and rel(damp, ra) < (tol if dtype == torch.float64 else 2e-6)
        assert rel(doff, ro) < tol
    finally:
        sky.close()


def test_autograd_function_matches_vjp(cuda):
    coef = jsky.diffuse_coefficients(EMIN, EMAX, EREF)
    sky = jsky.CorrelatedFieldSky((72, 66), 1.0, n_fields=2, crop=(64, 60), coefficients=coef,
                                  dtype=torch.float64)
    try:
        amp, xi, off = make_inputs(sky, 8)
        a = T(amp, torch.float64, cuda).requires_grad_()
        x = T(xi, torch.float64, cuda).requires_grad_()
        o = T(off, torch.float64, cuda).requires_grad_()
        w = torch.randn(3, 64, 60, dtype=torch.float64, device=cuda)
        (jsky.correlated_field_logsky(sky, a, x, o) * w).sum().backward()
        rx, ra, ro = SO.fields_vjp(amp, xi, sky.pindex,
                                   SO.logsky_cotangent_to_fields(w.cpu().numpy(), coef, sky.shape))
        assert rel(x.grad, rx) < 1e-12 and rel(a.grad, ra) < 1e-12 and rel(o.grad, ro) < 1e-12
    finally:
        sky.close()


@pytest.fixture(scope="module")
def chain_case():
    nx, dx, m, M, E = 128, 32, 16, 2, 3
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
    coef = jsky.diffuse_coefficients(EMIN, EMAX, EREF)
    shape = (jsky.good_fft_size(int(nx * 1.1075)),) * 2
    pidx, um, _ = jsky.fourier_mode_distributor(shape, 1.0)
    rng = np.random.default_rng(17)
    k = um / um[-1]
    amp = np.stack([0.4 * (1 + (k / 0.05) ** 2) ** -1.0, 0.05 * (1 + (k / 0.05) ** 2) ** -1.0])
    amp /= np.sqrt(pidx.size) / 8
    xi = rng.standard_normal((2,) + shape)
    off = np.array([0.3, -0.2])
    ls = SO.logsky(SO.fields(amp, xi, off, pidx), coef, (nx, nx))
    x = np.exp(ls)
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, nx // dx, m, inst.exposure, inst.readmask)
    lam = R(x)
    data = [synthetic.poisson_data(l, 41 + i) for i, l in enumerate(lam)]
    e, gx = R.energy_and_grad(x, data)
    rx, ra, ro = SO.fields_vjp(amp, xi, pidx, SO.logsky_cotangent_to_fields(x * gx, coef, shape))
    # the gradient is x R^T(1 - d / lam): the size of its cancelling term
    # x R^T(d / lam), carried through the same maps, scales FP32 errors
    xc = x * R.adjoint([d / l for d, l in zip(data, lam)])
    cx, _, _ = SO.fields_vjp(amp, xi, pidx, SO.logsky_cotangent_to_fields(xc, coef, shape))
    co = np.abs(coef).T @ xc.sum(axis=(1, 2))
    return dict(inst=inst, coef=coef, shape=shape, amp=amp, xi=xi, off=off,
                data=np.concatenate(data), energy=e, dxi=rx, damp=ra, doff=ro,
                cancel_dxi=np.linalg.norm(cx), cancel_doff=co)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_energy_and_grad_through_the_sky_model(cuda, chain_case, dtype):
    c = chain_case
    inst = c["inst"]
    plan = ju.ResponsePlan(inst.n_modules, inst.n_energies, inst.shape, inst.n_patches,
                           inst.margin, dtype=dtype)
    plan.set_psf(inst.psf).set_exposure(inst.exposure, inst.readmask).set_data(c["data"])
    sky = jsky.CorrelatedFieldSky(c["shape"], 1.0, n_fields=2, crop=inst.shape,
                                  coefficients=c["coef"], dtype=dtype)
    try:
        e, dxi, damp, doff = sky.energy_and_grad(plan, T(c["amp"], dtype, cuda),
                                                 T(c["xi"], dtype, cuda), T(c["off"], dtype, cuda))
        if dtype == torch.float64:
            assert abs(float(e) - c["energy"]) / abs(c["energy"]) < 1e-12
            assert rel(dxi, c["dxi"]) < 1e-10
            assert rel(damp, c["damp"]) < 1e-10
            assert rel(doff, c["doff"]) < 1e-10
        else:
            # the energy gradient cancels (1 - d / lam); FP32 error is judged
            # against the cancelling term, as for the sky gradient
            assert abs(float(e) - c["energy"]) / abs(c["energy"]) < 1e-6
            err_off = np.abs(doff.double().cpu().numpy() - c["doff"]) / c["cancel_doff"]
            assert err_off.max() < 1e-5
            err_xi = np.linalg.norm(dxi.double().cpu().numpy() - c["dxi"]) / c["cancel_dxi"]
            assert err_xi < 1e-5
    finally:
        sky.close()
        plan.close()


def test_energy_gradient_by_finite_differences(cuda, chain_case):
    c = chain_case
    inst = c["inst"]
    plan = ju.ResponsePlan(inst.n_modules, inst.n_energies, inst.shape, inst.n_patches,
                           inst.margin, dtype=torch.float64)
    plan.set_psf(inst.psf).set_exposure(inst.exposure, inst.readmask).set_data(c["data"])
    sky = jsky.CorrelatedFieldSky(c["shape"], 1.0, n_fields=2, crop=inst.shape,
                                  coefficients=c["coef"], dtype=torch.float64)
    try:
        amp = T(c["amp"], torch.float64, cuda)
        xi = T(c["xi"], torch.float64, cuda)
        off = T(c["off"], torch.float64, cuda)
        _, dxi, damp, doff = sky.energy_and_grad(plan, amp, xi, off)

        def energy(a, x, o):
            ee, _ = plan.energy_and_grad_logsky(sky.logsky(a, x, o), need_grad=False)
            return float(ee)

        def deriv(f, h=1e-4):
            # central differences at h and h/2, Richardson-extrapolated (error
            # O(h^4)): |energy| ~ 1e9 here, so the rounding of each energy
            # (~1e-7) limits how small h can be, and a shift of the offsets
            # scales the whole sky, whose third derivative is large
            d1 = (f(h) - f(-h)) / (2 * h)
            d2 = (f(h / 2) - f(-h / 2)) / h
            return (4 * d2 - d1) / 3

        rng = np.random.default_rng(4)
        v = torch.as_tensor(rng.standard_normal(c["xi"].shape), device=cuda)
        fd = deriv(lambda t: energy(amp, xi + t * v, off))
        an = float((dxi * v).sum())
        assert abs(fd - an) < 1e-5 * abs(an)
        do = torch.tensor([1.0, -0.5], dtype=torch.float64, device=cuda)
        fd = deriv(lambda t: energy(amp, xi, off + t * do))
        assert abs(fd - float((doff * do).sum())) < 1e-5 * abs(fd)
        va = torch.as_tensor(rng.uniform(-1, 1, c["amp"].shape), device=cuda) * amp
        fd = deriv(lambda t: energy(amp + t * va, xi, off))
        assert abs(fd - float((damp * va).sum())) < 1e-5 * abs(fd)
    finally:
        sky.close()
        plan.close()


def test_cf_argument_errors(cuda):
    with pytest.raises(ValueError):
        jsky.CorrelatedFieldSky((16, 16), 1.0, n_fields=5)
    with pytest.raises(ValueError):
        jsky.CorrelatedFieldSky((16, 16), 1.0, crop=(17, 4))
    sky = jsky.CorrelatedFieldSky((16, 16), 1.0, dtype=torch.float64)
    try:
        amp, xi, off = make_inputs(sky, 1)
        with pytest.raises(ValueError):  # no coefficients: fields only
            sky.logsky(amp, xi, off)
        with pytest.raises(ValueError):
            sky.vjp(amp, xi)
    finally:
        sky.close()
    with pytest.raises(ju.JubikUnsupported):
        jsky.CorrelatedFieldSky((16, 13 * 67), 1.0)  # prime factor above the FFT's radix limit


def test_sky_of_the_reference_sky_model_test(cuda):
    """The properties test/test_sky_model.py:80-97 checks of J-UBIK's sky for
    its config (sdim 128, s_padding_ratio 1.1, 3 bins 0.2-1 / 1-2 / 2-4 keV,
    e_ref 2, spatial + plaw fields): at positions 0.1 x standard normal the sky
    exp(logsky) has the data shape, is finite, non-negative, not constant, and
    a second evaluation repeats it exactly."""
    shape = (jsky.good_fft_size(int(128 * 1.1)),) * 2
    coef = jsky.diffuse_coefficients([0.2, 1.0, 2.0], [1.0, 2.0, 4.0], 2.0)
    sky = jsky.CorrelatedFieldSky(shape, 1.0, n_fields=2, crop=(128, 128), coefficients=coef,
                                  dtype=torch.float64)
    try:
        rng = np.random.default_rng(81)
        k = sky.mode_lengths / sky.mode_lengths[-1]
        amp = np.stack([(1 + (k / 0.05) ** 2) ** -1.0] * 2) / np.sqrt(sky.pindex.size)
        xi = T(0.1 * rng.standard_normal((2,) + shape), torch.float64, cuda)
        off = T(np.array([-14.0, -2.0]), torch.float64, cuda)
        a = T(amp, torch.float64, cuda)
        s1 = torch.exp(sky.logsky(a, xi, off))
        s2 = torch.exp(sky.logsky(a, xi, off))
        assert s1.shape == (3, 128, 128)
        assert bool(torch.isfinite(s1).all()) and bool((s1 >= 0).all())
        assert float(s1.var()) > 0
        assert torch.equal(s1, s2)
    finally:
        sky.close()
