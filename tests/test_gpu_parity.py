"""GPU parity of the response kernels against the float64 oracle.

Tolerances: the FP64 paths must match the oracle to 1e-12 relative L2
(index/mask work bit-exact); the FP32 paths to 1e-6 for the response and its
transpose.  The FP32 Poisson gradient is bounded by the conditioning of
1 - d/lam at faint pixels (lam error 1e-7 -> gradient error ~1e-4), so it is
checked against 5e-4 and, separately, by its agreement with the FP64 GPU path.
"""
import numpy as np
import pytest
import torch

import jubik_oracle as O
import jubik_gb300 as ju
from jubik_gb300 import synthetic

pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-12, torch.float32: 1e-6}
GRAD_TOL = {torch.float64: 1e-11, torch.float32: 5e-4}


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# (nx, dx, margin, M, E): FFT sides 16 .. 192 and unfused-only sides
CASES = [(48, 4, 4, 1, 1), (64, 8, 8, 1, 1), (64, 16, 8, 2, 2), (64, 16, 16, 1, 2),
         (96, 32, 16, 2, 1), (128, 32, 32, 1, 1), (256, 64, 32, 2, 2),
         (64, 16, 24, 1, 1), (36, 2, 2, 1, 2), (60, 20, 5, 1, 1),
         (32, 32, 8, 1, 1), (64, 32, 16, 2, 2),  # one patch (P = 80), 2 x 2 patches
         (256, 64, 16, 2, 2), (160, 32, 48, 1, 1)]  # P = 160 (FP32 fused)


@pytest.fixture(scope="module")
def oracle_cases():
    out = {}
    rng = np.random.default_rng(0)
    for c in CASES:
        nx, dx, m, M, E = c
        inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
        dom = O.Domain((E, nx, nx), (1.0, 0.5, 0.5))
        R = O.Response(dom, inst.psf, nx // dx, m, inst.exposure, inst.readmask, pixel_area=0.3)
        cot_img = rng.normal(size=(M, E, nx, nx))
        lam = R(inst.sky)
        data = [synthetic.poisson_data(l, 1 + i) for i, l in enumerate(lam)]
        e, g = R.energy_and_grad(inst.sky, data)
        v = rng.normal(size=inst.sky.shape)
        cot = rng.normal(size=sum(l.size for l in lam))
        out[c] = dict(inst=inst, img=R.psf(inst.sky), cot_img=cot_img,
                      adj=R.psf_adjoint(cot_img), lam=np.concatenate(lam),
                      data=np.concatenate(data), energy=e, grad=g, v=v,
                      metric=R.metric(inst.sky, v), cot=cot,
                      vjp=R.adjoint(np.split(cot, np.cumsum([l.size for l in lam])[:-1])))
    return out


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"P{2 * c[1] + 2 * c[2]}_M{c[3]}E{c[4]}")
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("path", ["fused", "fused_unit", "plain"])
def test_response_parity(cuda, oracle_cases, case, dtype, path):
    nx, dx, m, M, E = case
    P = 2 * dx + 2 * m
    if path.startswith("fused") and not ju._lib.load().jubik_fused_supported(P, 0 if dtype ==
                                                                    torch.float32 else 1):
        with pytest.raises(ju.JubikUnsupported):
            ju.ResponsePlan(M, E, (nx, nx), nx // dx, m, dtype=dtype, path=path)
        return
    ref = oracle_cases[case]
    inst = ref["inst"]
    plan = ju.ResponsePlan(M, E, (nx, nx), nx // dx, m, dtype=dtype, path=path, pixel_area=0.3)
    try:
        plan.set_psf(inst.psf).set_exposure(inst.exposure, inst.readmask).set_data(ref["data"])
        tol = TOL[dtype]
        assert rel(plan.psf_forward(inst.sky), ref["img"]) < tol
        assert rel(plan.psf_adjoint(ref["cot_img"]), ref["adj"]) < tol
        assert rel(plan.response(inst.sky), ref["lam"]) < tol
        assert rel(plan.response_vjp(ref["cot"]), ref["vjp"]) < tol
        e, g = plan.energy_and_grad(inst.sky)
        assert abs(float(e) - ref["energy"]) / abs(ref["energy"]) < tol
        assert rel(g, ref["grad"]) < GRAD_TOL[dtype]
        assert rel(plan.metric(inst.sky, ref["v"]), ref["metric"]) < 10 * tol
        # metric with the cached lam of the last energy evaluation
        plan.energy_and_grad(inst.sky, need_grad=False)
        assert rel(plan.metric(None, ref["v"]), ref["metric"]) < 10 * tol
    finally:
        plan.close()


def test_readout_index_is_c_order_per_module(cuda):
    inst = synthetic.config2(nx=64, dx=16, margin=8, n_modules=2, n_energies=2)
    plan = ju.ResponsePlan(2, 2, (64, 64), 4, 8, dtype=torch.float64)
    plan.set_exposure(inst.exposure, inst.readmask)
    idx = plan.readout_index().cpu().numpy()
    np.testing.assert_array_equal(idx, np.flatnonzero(inst.readmask.reshape(-1)))
    assert plan.readout_sizes == [int(inst.readmask[i].sum()) for i in range(2)]
    plan.close()


def test_full_field_kernels_match_precut(cuda):
    nx, dx, m = 96, 16, 8
    n = nx // dx
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=1, n_energies=2)
    K = 2 * dx
    full = np.zeros(inst.psf.shape[:3] + (nx, nx))
    a = (np.arange(K) - dx) % nx
    full[..., a[:, None], a[None, :]] = inst.psf
    for dtype in (torch.float64, torch.float32):
        p1 = ju.ResponsePlan(1, 2, (nx, nx), n, m, dtype=dtype).set_psf(inst.psf, "precut")
        p2 = ju.ResponsePlan(1, 2, (nx, nx), n, m, dtype=dtype).set_psf(full, "full")
        # identical spectra; the fused overlap-add sums in atomic order (ulp-level)
        assert rel(p1.psf_forward(inst.sky), p2.psf_forward(inst.sky).double().cpu().numpy()) \
            < (1e-14 if dtype == torch.float64 else 1e-7)
        p1.close()
        p2.close()


def test_energy_broadcast_kernels(cuda):
    nx, dx, m = 64, 16, 8
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=1, n_energies=3)
    k2 = inst.psf[:, :, 0]  # (M, n^2, K, K): the same PSF for every energy
    plan = ju.ResponsePlan(1, 3, (nx, nx), nx // dx, m, dtype=torch.float64).set_psf(k2)
    dom = O.Domain((3, nx, nx), (1.0, 1.0, 1.0))
    ref = O.linpatch_convolve(inst.sky, dom, k2[0], nx // dx, m, precut=True)
    assert rel(plan.psf_forward(inst.sky)[0], ref) < 1e-12
    plan.close()


# ------------------------------------------------------------ drop-in API
def test_slice_patches_bit_exact(cuda):
    rng = np.random.default_rng(0)
    x = rng.random((3, 36, 36))
    for dr in (0, 2):
        ref = O.slice_patches(x, (3, 36, 36), 16, dr)
        got = ju.slice_patches(x, (3, 36, 36), 16, dr).cpu().numpy()
        np.testing.assert_array_equal(got, ref)
        adj = ju.slice_patches_adjoint(ref, (3, 36, 36), 16, dr).cpu().numpy()
        np.testing.assert_allclose(adj, O.slice_patches_adjoint(ref, (3, 36, 36), 16, dr),
                                   rtol=1e-14)


def test_slice_patches_odd_stride_clamp(cuda):
    # odd stride: jax.lax.dynamic_slice clamps the last start (convolve.py:55-57)
    x = np.arange(3 * 21 * 21, dtype=float).reshape(3, 21, 21)
    ref = O.slice_patches(x, (3, 21, 21), 3, 0)
    np.testing.assert_array_equal(ju.slice_patches(x, (3, 21, 21), 3, 0).cpu().numpy(), ref)


def test_golden_fixtures(cuda):
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "slice36.npz"))
    np.testing.assert_array_equal(
        ju.slice_patches(g["x"], (36, 36), 16, 2).cpu().numpy(), g["patches"])
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "linpatch48.npz"))
    dom = ju.Domain((2, 48, 48), (1.0, 0.5, 0.5))
    y = ju.linpatch_convolve(g["x"], dom, g["kernel"], 3, 8)
    assert rel(y, g["y"]) < 1e-12
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "response32.npz"))
    R = ju.Response(ju.Domain((1, 32, 32), (1.0, 1.0, 1.0)), g["kernel"], 2, 4,
                    exposures=g["exposure"].copy(), flags=g["readmask"].astype(float),
                    pixel_area=0.25, keys=["a", "b"], dtype=torch.float64)
    assert rel(R.flat(g["x"]), g["lam"]) < 1e-12
    sizes = [int(g["readmask"][i].sum()) for i in range(2)]
    lh = ju.Poissonian(ju.Vector({"a": g["data"][:sizes[0]], "b": g["data"][sizes[0]:]}))
    e, grad = lh.amend(R).energy_and_gradient(torch.as_tensor(g["x"]))
    assert abs(float(e) - float(g["energy"])) / abs(float(g["energy"])) < 1e-12
    assert rel(grad, g["grad"]) < 1e-11


def test_linpatch_convolve_full_kernel_drop_in(cuda):
    rng = np.random.default_rng(3)
    E, N, n, m = 2, 48, 3, 8
    dx = N // n
    ker = rng.random((n * n, E, N, N))
    x = rng.random((E, N, N))
    dom = ju.Domain((E, N, N), (1.0, 0.5, 0.5))
    ref = O.linpatch_convolve(x, O.Domain(dom.shape, dom.distances), ker, n, m)
    assert rel(ju.linpatch_convolve(x, dom, ker, n, m), ref) < 1e-12
    # float32 input -> FP32 path
    assert rel(ju.linpatch_convolve(x.astype(np.float32), dom, ker.astype(np.float32), n, m),
               ref) < 1e-6


def test_linpatch_convolve_autograd_matches_adjoint(cuda):
    rng = np.random.default_rng(4)
    E, N, n, m = 1, 64, 4, 8
    dx = N // n
    ker = rng.random((n * n, E, 2 * dx, 2 * dx))
    x = torch.tensor(rng.random((E, N, N)), device="cuda", requires_grad=True)
    dom = ju.Domain((E, N, N), (1.0, 1.0, 1.0))
    y = ju.linpatch_convolve(x, dom, ker, n, m)
    g = torch.tensor(rng.normal(size=(E, N, N)), device="cuda")
    (y * g).sum().backward()
    ref = O.linpatch_convolve_adjoint(g.cpu().numpy(), O.Domain(dom.shape, dom.distances),
                                      ker, n, m, precut=True)
    assert rel(x.grad, ref) < 1e-12


def test_linpatch_broadcast_prints(cuda, capsys):
    rng = np.random.default_rng(5)
    N, n, m = 32, 4, 4
    dx = N // n
    ker = rng.random((n * n, 2 * dx, 2 * dx))
    x = rng.random((2, N, N))
    dom = ju.Domain((2, N, N), (1.0, 1.0, 1.0))
    y = ju.linpatch_convolve(x, dom, ker, n, m)
    assert "Dimension Inconsistency. Broadcasting PSFs" in capsys.readouterr().out
    ref = O.linpatch_convolve(x, O.Domain(dom.shape, dom.distances), ker, n, m, precut=True)
    assert rel(y, ref) < 1e-12


def test_linpatch_rejects_degenerate_cut(cuda):
    # n = 2 makes the reference's kernel cut [0:-0] empty (convolve.py:107-111)
    with pytest.raises(ValueError):
        ju.linpatch_convolve(np.ones((1, 32, 32)), ju.Domain((1, 32, 32), (1.0, 1.0, 1.0)),
                             np.ones((4, 1, 32, 32)), 2, 4)


def test_convolve_identity_and_broadcast(cuda, capsys):
    rng = np.random.default_rng(0)
    signal = rng.normal(size=(4, 4))
    kernel = np.zeros((4, 4))
    kernel[0, 0] = 1.0
    dom = ju.Domain((4, 4), (1.0, 1.0))
    np.testing.assert_allclose(ju.convolve(kernel, signal, dom, (-2, -1)).cpu().numpy(), signal,
                               rtol=1e-10, atol=1e-10)
    sig2 = np.stack([np.ones((4, 4)), 2.0 * np.ones((4, 4))])
    res = ju.convolve(kernel, sig2, dom, (-2, -1))
    assert "Dimension Inconsistency. Broadcasting PSFs" in capsys.readouterr().out
    np.testing.assert_allclose(res.cpu().numpy(), sig2, rtol=1e-10, atol=1e-10)
    # general kernel, odd sizes and dvol
    k = rng.normal(size=(3, 10, 15))
    s = rng.normal(size=(3, 10, 15))
    d = ju.Domain((3, 10, 15), (1.0, 0.5, 0.25))
    ref = O.convolve(k, s, O.Domain(d.shape, d.distances), (-2, -1))
    assert rel(ju.convolve(k, s, d, (-2, -1)), ref) < 1e-13


def test_exposure_drop_in(cuda):
    rng = np.random.default_rng(0)
    exp = rng.uniform(0.0, 3e3, size=(3, 100, 100))
    x = np.linspace(0.25, 1.75, num=100 * 100).reshape(100, 100)
    res = ju.build_exposure_function(exp.copy(), 500)(x).cpu().numpy()
    want = exp.copy()
    want[want < 500] = 0
    np.testing.assert_array_equal(res, want * x)
    np.testing.assert_array_equal(ju.build_exposure_function(exp.copy())(x).cpu().numpy(),
                                  exp * x)


def test_readout_drop_in_bit_exact(cuda):
    rng = np.random.default_rng(0)
    exp = rng.uniform(0.0, 3e3, size=(2, 3, 24, 24))
    x = np.arange(2 * 3 * 24 * 24, dtype=float).reshape((2, 3, 24, 24)) + 0.5
    mask = exp < 20
    res = ju.build_readout_function(exp.copy(), 20, ("tm_1", "tm_2"))(x)
    assert tuple(res.tree.keys()) == ("tm_1", "tm_2")
    for i, k in enumerate(("tm_1", "tm_2")):
        np.testing.assert_array_equal(res.tree[k].cpu().numpy(), x[i][~mask[i]])
    res = ju.build_readout_function(exp.copy(), None, ("tm_1", "tm_2"))(x)
    for i, k in enumerate(("tm_1", "tm_2")):
        np.testing.assert_array_equal(res.tree[k].cpu().numpy(), x[i].ravel())
    single = np.expand_dims(exp[0], 0)
    sky1 = np.arange(3 * 24 * 24, dtype=float).reshape((1, 3, 24, 24)) + 1.0
    res = ju.build_readout_function(single.copy(), 20, None)(sky1)
    assert tuple(res.tree.keys()) == ("masked input",)
    np.testing.assert_array_equal(res.tree["masked input"].cpu().numpy(),
                                  sky1[0][~(single < 20)[0]])


def test_poissonian_drop_in(cuda):
    rng = np.random.default_rng(2)
    lam = rng.uniform(0.5, 20.0, size=1000)
    d = rng.poisson(lam)
    t = rng.normal(size=1000)
    lh = ju.Poissonian(d)
    assert abs(float(lh(lam)) - O.poisson_energy(lam, d)) / abs(O.poisson_energy(lam, d)) < 1e-13
    e, g = lh.energy_and_gradient(lam)
    np.testing.assert_allclose(g.cpu().numpy(), O.poisson_grad(lam, d), rtol=1e-14)
    np.testing.assert_allclose(lh.metric(lam, t).cpu().numpy(), O.poisson_metric(lam, t),
                               rtol=1e-14)
    np.testing.assert_allclose(lh.left_sqrt_metric(lam, t).cpu().numpy(),
                               O.poisson_left_sqrt_metric(lam, t), rtol=1e-14)
    np.testing.assert_allclose(lh.normalized_residual(lam).cpu().numpy(),
                               O.poisson_normalized_residual(lam, d), rtol=1e-13)
    with pytest.raises(ValueError):
        ju.Poissonian(np.array([1, -1]))
    # zero expected counts at a zero count: 0 * log(0) = nan, as in the reference's vdot
    assert np.isnan(float(ju.Poissonian(np.array([0, 1]))(np.array([0.0, 1.0]))))


def test_response_poissonian_autograd_and_fd(cuda):
    nx, dx, m, M, E = 64, 16, 8, 2, 1
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
    R = ju.Response(ju.Domain((E, nx, nx), (1.0, 1.0, 1.0)), inst.psf, nx // dx, m,
                    exposures=inst.exposure.copy(), flags=inst.readmask.astype(float),
                    keys=["a", "b"], pixel_area=0.3, dtype=torch.float64)
    lam = R.flat(inst.sky).cpu().numpy()
    data = synthetic.poisson_data(lam, 1)
    s0 = R.plan.readout_sizes[0]
    lh = ju.Poissonian(ju.Vector({"a": data[:s0], "b": data[s0:]})).amend(R)
    x = torch.tensor(inst.sky, device="cuda", requires_grad=True)
    e = lh.energy_autograd(x)
    e.backward()
    _, g = lh.energy_and_gradient(x.detach())
    assert rel(x.grad, g.cpu().numpy()) < 1e-13
    rng = np.random.default_rng(9)
    for _ in range(8):
        v = torch.tensor(rng.normal(size=inst.sky.shape), device="cuda")
        eps = 1e-4
        ep = float(lh.energy(x.detach() + eps * v))
        em = float(lh.energy(x.detach() - eps * v))
        fd = (ep - em) / (2 * eps)
        an = float((g * v).sum())
        assert abs(fd - an) <= 1e-6 * abs(an) + 1e-8 * abs(float(lh.energy(x.detach())))


def test_response_vector_interface(cuda):
    nx, dx, m, M, E = 64, 16, 8, 2, 2
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
    rd = ju.build_response(ju.Domain((E, nx, nx), (1.0, 1.0, 1.0)), inst.psf, nx // dx, m,
                           exposures=inst.exposure.copy(), flags=inst.readmask.astype(float),
                           keys=["tm1", "tm2"], pixel_area=0.5, dtype=torch.float64)
    out = rd["R"](inst.sky)
    assert list(out.tree.keys()) == ["tm1", "tm2"]
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    ref = O.Response(dom, inst.psf, nx // dx, m, inst.exposure, inst.readmask, pixel_area=0.5)
    for i, k in enumerate(["tm1", "tm2"]):
        assert rel(out.tree[k], ref(inst.sky)[i]) < 1e-12
    # the reference's keys, plus the readout transpose its diagnostics expect
    assert set(rd) == {"pix_area", "psf", "exposure", "mask", "kernel", "R", "mask_adj"}


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_dependent_launch_switch_keeps_results(cuda, dtype):
    """The module-shared step runs as one chain of dependent launches; with the
    chain switched off the same kernels run fully serialised."""
    nx, dx, m, M, E = 128, 32, 16, 3, 2
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
    plan = ju.ResponsePlan(M, E, (nx, nx), nx // dx, m, dtype=dtype).set_psf(inst.psf)
    plan.set_exposure(inst.exposure, inst.readmask)
    lam = plan.response(inst.sky).double().cpu().numpy()
    plan.set_data(synthetic.poisson_data(lam, 2))
    e1, g1 = plan.energy_and_grad(inst.sky)
    g1 = g1.clone()
    plan.set_dependent_launch(False)
    for _ in range(2):  # twice, serialised launches: the same bits as the chained call
        e2, g2 = plan.energy_and_grad(inst.sky)
        assert float(e2) == float(e1)
        assert torch.equal(g2, g1)
    plan.close()


def test_fully_masked_module_and_empty_readout(cuda):
    """A module whose every pixel is masked reads out nothing: its readout is
    empty, it adds nothing to the energy and nothing to the gradient."""
    nx, dx, m, M, E = 128, 32, 16, 3, 2
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
    readmask = inst.readmask.copy()
    readmask[1] = False
    exposure = inst.exposure * readmask
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, nx // dx, m, exposure, readmask)
    lam = R(inst.sky)
    assert lam[1].size == 0
    data = [synthetic.poisson_data(l, 9 + i) if l.size else np.zeros(0, np.int32)
            for i, l in enumerate(lam)]
    e_ref, g_ref = R.energy_and_grad(inst.sky, data)
    for dtype in (torch.float64, torch.float32):
        plan = ju.ResponsePlan(M, E, (nx, nx), nx // dx, m, dtype=dtype).set_psf(inst.psf)
        plan.set_exposure(exposure, readmask).set_data(np.concatenate(data))
        assert plan.readout_sizes[1] == 0
        e, g = plan.energy_and_grad(inst.sky)
        tol = 1e-12 if dtype == torch.float64 else 1e-6
        assert abs(float(e) - e_ref) / abs(e_ref) < tol
        assert rel(plan.response(inst.sky), np.concatenate(lam)) < tol
        plan.close()


def test_large_field_adjoint_identity(cuda):
    """4096^2 field, 64 x 64 patches (4096 units, P = 192): the adjoint
    identity and FP32 against FP64 at a size far beyond the oracle's reach."""
    nx, dx, m = 4096, 64, 32
    rng = np.random.default_rng(12)
    K = 2 * dx
    u = np.arange(K) - dx
    g = np.exp(-0.5 * (u[:, None] ** 2 + u[None, :] ** 2) / 9.0)
    psf = np.broadcast_to((g / g.sum())[None, None], (1, (nx // dx) ** 2, K, K)).copy()
    x = torch.as_tensor(rng.random((1, nx, nx)), device=cuda)
    y = torch.as_tensor(rng.normal(size=(1, 1, nx, nx)), device=cuda)
    p64 = ju.ResponsePlan(1, 1, (nx, nx), nx // dx, m, dtype=torch.float64).set_psf(psf)
    p32 = ju.ResponsePlan(1, 1, (nx, nx), nx // dx, m, dtype=torch.float32).set_psf(psf)
    a64 = p64.psf_forward(x)
    b64 = p64.psf_adjoint(y)
    lhs, rhs = float((a64 * y).sum()), float((x * b64).sum())
    assert abs(lhs - rhs) <= 1e-12 * float(torch.linalg.norm(a64) * torch.linalg.norm(y))
    assert rel(p32.psf_forward(x.float()), a64.cpu().numpy()) < 1e-6
    assert rel(p32.psf_adjoint(y.float()), b64.cpu().numpy()) < 1e-6
    p64.close()
    p32.close()


def test_non_finite_sky_propagates_without_fault(cuda):
    """NaN or Inf in the sky gives a non-finite energy and gradient, raises no
    CUDA error, and leaves the plan usable for the next finite call."""
    nx, dx, m, M, E = 64, 16, 8, 2, 1
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
    plan = ju.ResponsePlan(M, E, (nx, nx), nx // dx, m, dtype=torch.float32).set_psf(inst.psf)
    plan.set_exposure(inst.exposure, inst.readmask)
    lam = plan.response(inst.sky).double().cpu().numpy()
    plan.set_data(synthetic.poisson_data(lam, 3))
    e0, g0 = plan.energy_and_grad(inst.sky)
    e0, g0 = float(e0), g0.clone()
    for bad in (np.nan, np.inf):
        x = inst.sky.copy()
        x[0, 10, 10] = bad
        e, g = plan.energy_and_grad(x)
        torch.cuda.synchronize()
        assert not np.isfinite(float(e))
        assert not bool(torch.isfinite(g).all())
    e1, g1 = plan.energy_and_grad(inst.sky)
    # the fused sums are exact in any order: the finite call returns the same bits
    assert float(e1) == e0 and torch.equal(g1, g0)
    plan.close()


def test_path_override_from_environment(cuda, monkeypatch):
    monkeypatch.setenv("JUBIK_PATH", "plain")
    plan = ju.ResponsePlan(1, 1, (64, 64), 4, 8, dtype=torch.float32)
    assert plan.path == "plain"
    plan.close()
    monkeypatch.setenv("JUBIK_PATH", "bogus")
    with pytest.raises(ValueError):
        ju.ResponsePlan(1, 1, (64, 64), 4, 8, dtype=torch.float32)


def test_linpatch_convolve_picks_up_a_new_kernel(cuda):
    """Two calls with different numpy kernels of the same shape: the cached PSF
    spectra must follow the second kernel (its device copy may reuse the
    first one's memory)."""
    nx, dx, m, E = 64, 16, 8, 1
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=1, n_energies=E)
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    ka = np.ascontiguousarray(inst.psf[0])
    for scale in (1.0, 3.0):
        k = ka ** scale  # a new array each time, same shape
        got = ju.linpatch_convolve(inst.sky, ju.Domain(dom.shape, dom.distances), k, nx // dx, m)
        ref = O.linpatch_convolve(inst.sky, dom, k, nx // dx, m, precut=True)
        assert rel(got, ref) < 1e-12
