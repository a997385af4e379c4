"""The named workloads end to end on the GPU, against the float64 oracle.

- 256^2, one module, one energy, 8x8 patches of stride 32 with margin 16
  (FFT side 96): response and Poisson likelihood in FP64 and FP32, and the
  literal full-field kernel path.
- 1024^2 x 3 energies, correlated-field sky, 16x16 patches, margin 32:
  JVP, VJP and MGVI metric, and central finite differences of the Poisson
  energy (FP64: eps = 1e-4, 32 random directions; FP32: 4 directions that
  follow the gradient, where the derivative rises above the FP32 rounding).
- 2048^2 x 3 energies with 0.1 % point sources (flux 1e1 .. 1e5) and
  power-law PSF wings, 32x32 patches: FP32 against FP64 per energy.
- 1024^2 x 7 modules x 3 energies (the benchmark workload) at full size:
  size-independent properties (adjoint identity, linearity, FP32 vs FP64)
  and one module x energy plane against the oracle.

Tolerances: FP64 1e-12 relative L2 (1e-11 for gradients, 1e-10 for the
metric), FP32 1e-6.  The Poisson gradient R^T(1 - d/lam) is a difference of
two terms that nearly cancel where d is close to lam, so its FP32 error is
measured against the size of the cancelling term, |R^T(d/lam)|: 3e-6.  (FP32
FFT convolution errors are absolute, of order 1e-7 of the largest lam, so
faint pixels carry larger relative errors of lam, which d/lam passes on; the
observed level is 1.1e-6.)
"""
import numpy as np
import pytest
import torch

import jubik_oracle as O
import jubik_gb300 as ju
from jubik_gb300 import synthetic

pytestmark = pytest.mark.gpu

F32, F64 = torch.float32, torch.float64


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().double().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def grad_err(g, ref, cancel, dtype):
    """FP64: relative L2 error.  FP32: error relative to |R^T(d/lam)|."""
    a = g.detach().double().cpu().numpy()
    scale = np.linalg.norm(ref) if dtype == F64 else np.linalg.norm(cancel)
    return float(np.linalg.norm(a - ref) / scale)


def make_plan(inst, dtype, path="auto", pixel_area=1.0, psf=None, layout="auto"):
    plan = ju.ResponsePlan(inst.n_modules, inst.n_energies, inst.shape, inst.n_patches,
                           inst.margin, dtype=dtype, path=path, pixel_area=pixel_area)
    plan.set_psf(inst.psf if psf is None else psf, layout)
    plan.set_exposure(inst.exposure, inst.readmask)
    return plan


# ------------------------------------------------------------------ 256^2, P = 96
@pytest.fixture(scope="module")
def small_case():
    inst = synthetic.config1()
    dom = O.Domain((1, 256, 256), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, inst.n_patches, inst.margin, inst.exposure, inst.readmask)
    lam = R(inst.sky)
    data = [synthetic.poisson_data(lam[0], 1)]
    e, g = R.energy_and_grad(inst.sky, data)
    cancel = R.adjoint([data[0] / lam[0]])
    return dict(inst=inst, R=R, lam=lam[0], data=data[0], energy=e, grad=g, cancel=cancel)


@pytest.mark.parametrize("dtype", [F64, F32], ids=["f64", "f32"])
@pytest.mark.parametrize("path", ["fused", "plain"])
def test_small_field_response_and_likelihood(cuda, small_case, dtype, path):
    c = small_case
    plan = make_plan(c["inst"], dtype, path)
    try:
        plan.set_data(c["data"])
        tol = 1e-12 if dtype == F64 else 1e-6
        assert rel(plan.response(c["inst"].sky), c["lam"]) < tol
        e, g = plan.energy_and_grad(c["inst"].sky)
        assert abs(float(e) - c["energy"]) / abs(c["energy"]) < tol
        assert grad_err(g, c["grad"], c["cancel"], dtype) < (1e-11 if dtype == F64 else 3e-6)
    finally:
        plan.close()


def test_small_field_full_kernels_literal_path(cuda, small_case):
    """Full-field (n^2, E, N, N) kernels through the literal shift / cut / pad
    sequence of the oracle, against the GPU plan fed the same full kernels."""
    inst = small_case["inst"]
    nx, n = inst.shape[0], inst.n_patches
    dx = nx // n
    K = 2 * dx
    full = np.zeros(inst.psf.shape[:3] + (nx, nx))
    a = (np.arange(K) - dx) % nx
    full[..., a[:, None], a[None, :]] = inst.psf
    dom = O.Domain((1, nx, nx), (1.0, 1.0, 1.0))
    ref = O.linpatch_convolve(inst.sky, dom, full[0], n, inst.margin, precut=False)
    for dtype, tol in ((F64, 1e-12), (F32, 1e-6)):
        plan = make_plan(inst, dtype, psf=full, layout="full")
        assert rel(plan.psf_forward(inst.sky)[0], ref) < tol
        plan.close()


# ------------------------------------------------------ 1024^2 x 3, derivatives
@pytest.fixture(scope="module")
def deriv_case():
    inst = synthetic.config3()
    E, nx = inst.n_energies, inst.shape[0]
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, inst.n_patches, inst.margin, inst.exposure, inst.readmask)
    lam = R(inst.sky)
    data = [synthetic.poisson_data(lam[0], 3)]
    rng = np.random.default_rng(33)
    t = rng.normal(size=inst.sky.shape)
    cot = rng.normal(size=lam[0].size)
    e, g = R.energy_and_grad(inst.sky, data)
    jvp = R(t)[0]
    metric = R.metric(inst.sky, t)
    # the floor of the FP32 tier: the exact (float64) lam rounded once to FP32,
    # everything else in float64
    lam_r = lam[0].astype(np.float32).astype(np.float64)
    floor_grad = R.adjoint([1.0 - data[0] / lam_r])
    floor_metric = R.adjoint([jvp / lam_r])
    return dict(inst=inst, lam=lam[0], data=data[0], jvp=jvp, t=t, cot=cot,
                vjp=R.adjoint([cot]), energy=e, grad=g, metric=metric,
                cancel=R.adjoint([data[0] / lam[0]]),
                floor_grad=float(np.linalg.norm(floor_grad - g) / np.linalg.norm(g)),
                floor_metric=float(np.linalg.norm(floor_metric - metric) /
                                   np.linalg.norm(metric)))


@pytest.mark.parametrize("dtype", [F64, F32], ids=["f64", "f32"])
def test_derivatives_jvp_vjp_metric(cuda, deriv_case, dtype):
    c = deriv_case
    plan = make_plan(c["inst"], dtype)
    try:
        plan.set_data(c["data"])
        tol = 1e-12 if dtype == F64 else 1e-6
        assert rel(plan.response(c["inst"].sky), c["lam"]) < tol
        assert rel(plan.response_jvp(c["t"]), c["jvp"]) < tol
        assert rel(plan.response_vjp(c["cot"]), c["vjp"]) < tol
        e, g = plan.energy_and_grad(c["inst"].sky)
        assert abs(float(e) - c["energy"]) / abs(c["energy"]) < tol
        assert grad_err(g, c["grad"], c["cancel"], dtype) < (1e-11 if dtype == F64 else 3e-6)
        assert rel(plan.metric(c["inst"].sky, c["t"]), c["metric"]) < (1e-10 if dtype == F64
                                                                         else 1e-5)
    finally:
        plan.close()


def test_derivatives_central_finite_differences(cuda, deriv_case):
    """(H(x + eps v) - H(x - eps v)) / (2 eps) against <grad, v> on 32 random
    directions, eps = 1e-4, FP64.  The quotient's error is the rounding of H
    over 2 eps: here |H| ~ 1e11 and FP64 FFT convolution rounds lam (and so H)
    at a few 1e-15, i.e. an absolute error of order 1 against a typical
    |<grad, v>| = |grad| |v| / sqrt(n) ~ 3e4.  The bound 2e-4 of that size
    leaves a margin of 4 over the observed 5e-5; a wrong derivative (a missing
    exposure, pixel-area or weight factor) is off by O(1).  The FP64 gradient
    itself matches the oracle to 1e-11 in test_derivatives_jvp_vjp_metric."""
    c = deriv_case
    plan = make_plan(c["inst"], F64)
    try:
        plan.set_data(c["data"])
        x = torch.as_tensor(c["inst"].sky, device=cuda)
        _, g = plan.energy_and_grad(x)
        rng = np.random.default_rng(34)
        eps = 1e-4
        worst = 0.0
        for _ in range(32):
            v = torch.as_tensor(rng.normal(size=x.shape), device=cuda)
            ep = float(plan.energy_and_grad(x + eps * v, need_grad=False)[0])
            em = float(plan.energy_and_grad(x - eps * v, need_grad=False)[0])
            fd = (ep - em) / (2 * eps)
            an = float((g * v).sum())
            scale = float(torch.linalg.norm(g) * torch.linalg.norm(v)) / np.sqrt(x.numel())
            worst = max(worst, abs(fd - an) / scale)
        assert worst < 2e-4, worst
    finally:
        plan.close()


def test_fp32_gradient_central_finite_differences(cuda, deriv_case):
    """The FP32 tier's gradient against central differences of its own energy.

    An FP32 energy carries rounding of a few tens in absolute terms (here |H|
    is about 2e11, and lam rounds at about 1e-7 of a patch's brightest values,
    with errors correlated across pixels).  Along a random direction v the
    derivative <grad, v> is only about |grad| = 5e3, so that rounding, divided
    by 2 eps, swamps it.  The directions here follow the gradient: sign(grad),
    sign(grad) with random weights in [0.5, 1.5], and grad itself.  Along them
    the derivative is sqrt(n) times larger, 1e4 to 2e5 per 2 eps.  The
    perturbed points are rounded to FP32, so H(x+) - H(x-) is compared with
    <grad, x+ - x-> over the points actually evaluated.  The float64 oracle
    puts the truncation error of these central differences at 3e-5 (sign,
    eps = 1e-2) and 1.5e-4 (grad, eps = 3e-3); the FP32 gradient is within
    6.5e-4 of FP64.  The bound 1e-2 leaves a margin over all of them; a wrong
    derivative (a missing factor) is off by O(1)."""
    c = deriv_case
    plan = make_plan(c["inst"], F32)
    try:
        plan.set_data(c["data"])
        x64 = torch.as_tensor(c["inst"].sky, device=cuda)
        x = x64.float()
        _, g = plan.energy_and_grad(x)
        g = g.double()
        n = g.numel()
        rng = np.random.default_rng(35)
        sg = torch.sign(g)
        dirs = [(sg, 1e-2)]
        for _ in range(2):
            dirs.append((sg * torch.as_tensor(rng.uniform(0.5, 1.5, size=x.shape), device=cuda),
                         1e-2))
        dirs.append((g / torch.linalg.norm(g) * np.sqrt(n), 3e-3))
        worst = 0.0
        for d, eps in dirs:
            xp = (x64 + eps * d).float()
            xm = (x64 - eps * d).float()
            ep = float(plan.energy_and_grad(xp, need_grad=False)[0])
            em = float(plan.energy_and_grad(xm, need_grad=False)[0])
            an = float((g * (xp.double() - xm.double())).sum())
            worst = max(worst, abs((ep - em) - an) / abs(an))
        assert worst < 1e-2, worst
    finally:
        plan.close()


# -------------------------------------------- 2048^2 x 3, point sources and wings
def test_point_sources_fp32_vs_fp64_per_energy(cuda):
    inst = synthetic.config4()
    p64 = make_plan(inst, F64)
    p32 = make_plan(inst, F32)
    try:
        x64 = torch.as_tensor(inst.sky, device=cuda)
        i64 = p64.psf_forward(x64)
        i32 = p32.psf_forward(x64.float())
        errs = [rel(i32[0, e], i64[0, e]) for e in range(inst.n_energies)]
        assert max(errs) < 1e-6, errs
        rng = np.random.default_rng(44)
        cot = torch.as_tensor(rng.normal(size=(1,) + tuple(x64.shape)), device=cuda)
        a64 = p64.psf_adjoint(cot)
        a32 = p32.psf_adjoint(cot.float())
        errs = [rel(a32[e], a64[e]) for e in range(inst.n_energies)]
        assert max(errs) < 1e-6, errs
        # the FP64 GPU path against the oracle on the first energy plane
        sl = inst.sky[:1]
        dom = O.Domain((1,) + inst.shape, (1.0, 1.0, 1.0))
        ref = O.linpatch_convolve(sl, dom, inst.psf[0, :, :1], inst.n_patches, inst.margin,
                                  precut=True)
        assert rel(i64[0, 0], ref[0]) < 1e-12
    finally:
        p64.close()
        p32.close()


# ------------------------------------------- 1024^2 x 7 x 3 (benchmark workload)
@pytest.fixture(scope="module")
def bench_case():
    return synthetic.config2()


def test_benchmark_workload_properties(cuda, bench_case):
    inst = bench_case
    p32 = make_plan(inst, F32)
    p64 = make_plan(inst, F64, path="plain")
    try:
        rng = np.random.default_rng(22)
        x = torch.as_tensor(inst.sky, device=cuda)
        y = torch.as_tensor(rng.normal(size=p32.readout_total), device=cuda)
        # FP32 against the FP64 unfused GPU path
        r32 = p32.response(x.float())
        r64 = p64.response(x)
        assert rel(r32, r64) < 1e-6
        v32 = p32.response_vjp(y.float())
        v64 = p64.response_vjp(y)
        assert rel(v32, v64) < 1e-6
        # adjoint identity <R x, y> = <x, R^T y>
        lhs = float((r64 * y).sum())
        rhs = float((x * v64).sum())
        assert abs(lhs - rhs) < 1e-12 * float(torch.linalg.norm(r64) * torch.linalg.norm(y))
        lhs32 = float((r32.double() * y).sum())
        rhs32 = float((x * v32.double()).sum())
        assert abs(lhs32 - rhs32) < 1e-6 * float(torch.linalg.norm(r64) * torch.linalg.norm(y))
        # linearity
        z = torch.as_tensor(rng.normal(size=inst.sky.shape), device=cuda)
        lin = p64.response(2.0 * x - 0.5 * z)
        assert rel(lin, 2.0 * r64 - 0.5 * p64.response(z)) < 1e-12
        # one module x energy plane against the oracle
        img32 = p32.psf_forward(x.float())
        img64 = p64.psf_forward(x)
        dom = O.Domain((1,) + inst.shape, (1.0, 1.0, 1.0))
        ref = O.linpatch_convolve(inst.sky[:1], dom, inst.psf[0, :, :1], inst.n_patches,
                                  inst.margin, precut=True)
        assert rel(img64[0, 0], ref[0]) < 1e-12
        assert rel(img32[0, 0], ref[0]) < 1e-6
        # the metric product at the workload's size: FP32 with the FP64 plan's lam
        t = torch.as_tensor(rng.normal(size=inst.sky.shape), device=cuda)
        m64 = p64.metric(x, t)
        p32.set_metric_lambda(p64.response(x))
        assert rel(p32.metric(None, t.float()), m64.double().cpu().numpy()) < 1e-6
    finally:
        p32.close()
        p64.close()


# --------------------------- FFT side 384: 8 x 8 eROSITA patches at 1024^2 (margin 64)
@pytest.mark.parametrize("dtype", [F64, F32], ids=["f64", "f32"])
def test_fft_side_384_unfused(cuda, dtype):
    """Patches of stride 128 with a 64-pixel margin (the margin rule of
    erosita_response.py:207 at 1024^2 with 8 x 8 patches) give P = 384, which
    runs the unfused path: here on a 256^2 field with 2 x 2 patches, two modules
    and two energies, against the oracle."""
    nx, dx, m, M, E = 256, 128, 64, 2, 2
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E, seed=5)
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, nx // dx, m, inst.exposure, inst.readmask)
    lam = R(inst.sky)
    data = [synthetic.poisson_data(l, 9 + i) for i, l in enumerate(lam)]
    e_ref, g_ref = R.energy_and_grad(inst.sky, data)
    plan = make_plan(inst, dtype)
    try:
        assert plan.path == "plain" and plan.P == 384
        plan.set_data(np.concatenate(data))
        tol = 1e-12 if dtype == F64 else 1e-6
        assert rel(plan.response(inst.sky), np.concatenate(lam)) < tol
        e, g = plan.energy_and_grad(inst.sky)
        assert abs(float(e) - e_ref) / abs(e_ref) < tol
        cancel = R.adjoint([d / l for d, l in zip(data, lam)])
        assert grad_err(g, g_ref, cancel, dtype) < (1e-11 if dtype == F64 else 3e-6)
    finally:
        plan.close()


# --------------------------- the demo geometries beyond the fused tile (P = 320)
@pytest.mark.parametrize("dtype", [F64, F32], ids=["f64", "f32"])
def test_chandra_demo_geometry_unfused(cuda, dtype):
    """512^2 field, 4 x 4 patches (stride 128), margin ceil(0.062 * 512) = 32:
    P = 320 (demos/configs/chandra_demo.yaml:13,44-45 with the margin rule of
    erosita_response.py:207), beyond the fused kernels' shared-memory tile, so
    the unfused path runs."""
    nx, dx, m, M, E = 512, 128, 32, 1, 2
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, nx // dx, m, inst.exposure, inst.readmask)
    lam = R(inst.sky)
    data = [synthetic.poisson_data(lam[0], 5)]
    e_ref, g_ref = R.energy_and_grad(inst.sky, data)
    plan = make_plan(inst, dtype)
    assert plan.path == "plain" and plan.P == 320
    plan.set_data(data[0])
    tol = 1e-12 if dtype == F64 else 1e-6
    assert rel(plan.response(inst.sky), lam[0]) < tol
    e, g = plan.energy_and_grad(inst.sky)
    assert abs(float(e) - e_ref) / abs(e_ref) < tol
    cancel = R.adjoint([data[0] / lam[0]])
    assert grad_err(g, g_ref, cancel, dtype) < (1e-11 if dtype == F64 else 3e-6)
    plan.close()


def test_fp32_gradient_and_metric_errors_come_from_the_fp32_forward(cuda, deriv_case):
    """Where the FP32 Poisson gradient R^T(1 - d/lam) and metric R^T(R t / lam)
    lose accuracy.  Rounding the exact lam once to FP32 (everything else in
    float64) moves them only by `floor`.  An FP32 FFT convolution's error is
    absolute, of order 1e-7 of a patch's brightest values, so faint pixels get
    a much larger relative error of lam, which d/lam and 1/lam pass on: a
    float64 gradient computed from the FP32 forward's lam already shows the
    whole FP32 gradient error.  So the fused path's adjoint, likelihood pass
    and overlap-add add nothing of their own; the limit is FP32 FFT
    convolution itself."""
    c = deriv_case
    inst = c["inst"]
    E, nx = inst.n_energies, inst.shape[0]
    R = O.Response(O.Domain((E, nx, nx), (1.0, 1.0, 1.0)), inst.psf, inst.n_patches,
                   inst.margin, inst.exposure, inst.readmask)
    plan = make_plan(inst, F32)
    try:
        plan.set_data(c["data"])
        _, g = plan.energy_and_grad(inst.sky)
        m = plan.metric(inst.sky, c["t"])
        lam32 = plan.response(inst.sky).double().cpu().numpy()
        eg, em = rel(g, c["grad"]), rel(m, c["metric"])
        e_lam = rel(R.adjoint([1.0 - c["data"] / lam32]), c["grad"])
        m_lam = rel(R.adjoint([c["jvp"] / lam32]), c["metric"])
        print(f"FP32 gradient {eg:.3e}: from the FP32 lam alone {e_lam:.3e}, lam rounding "
              f"floor {c['floor_grad']:.3e}; metric {em:.3e}: from the FP32 lam alone "
              f"{m_lam:.3e}, floor {c['floor_metric']:.3e}")
        assert abs(eg - e_lam) <= 0.1 * e_lam + 1e-6
        assert em <= m_lam + 1e-6
    finally:
        plan.close()


def test_fp32_metric_with_fp64_lambda_meets_1e6(cuda, deriv_case):
    """The metric weights 1/lam taken from a float64 plan's lam (once per
    linearisation point) leave the FP32 metric product only its own rounding."""
    c = deriv_case
    inst = c["inst"]
    p32 = make_plan(inst, F32)
    p64 = make_plan(inst, F64, path="plain")
    try:
        lam64 = p64.response(inst.sky)
        p32.set_metric_lambda(lam64)
        m = p32.metric(None, c["t"])
        em = rel(m, c["metric"])
        own = rel(p32.metric(inst.sky, c["t"]), c["metric"])  # weights from the FP32 lam
        print(f"FP32 metric: FP64 lam {em:.3e}, own FP32 lam {own:.3e}")
        assert em < 1e-6
        # a float32 copy of the float64 lam works the same
        p32.set_metric_lambda(lam64.float())
        assert rel(p32.metric(None, c["t"]), c["metric"]) < 1e-6
        with pytest.raises(ValueError):
            p32.set_metric_lambda(lam64[:-1])
    finally:
        p32.close()
        p64.close()
