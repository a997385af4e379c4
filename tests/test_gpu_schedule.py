"""Run length of the module-shared forward (FP32, FFT side 192).

A CTA of the run-ordered forward takes runs of 2 or 4 vertically adjacent
patches of one module and sums the block rows they share in tensor memory;
run length 1 takes one unit at a time.  Every run length must give the
response, energy and gradient of the float64 oracle at the FP32 tier, the same
bits on every call, and results that agree with each other to FP32 rounding.
The library's own choice follows the busiest CTA's work on the GPU's SMs, and
``ResponsePlan.autotune`` keeps the measured fastest.
"""
import math

import numpy as np
import pytest
import torch

import jubik_oracle as O
import jubik_gb300 as ju
from jubik_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _bits(t):
    return t.detach().reshape(-1).contiguous().view(torch.uint8).cpu().numpy().tobytes()


@pytest.fixture(scope="module")
def demo():
    """256² x 2 modules x 2 energies, 4 x 4 patches of stride 64, margin 32 (P = 192)."""
    inst = synthetic.config2(nx=256, n_modules=2, n_energies=2, seed=4)
    dom = O.Domain((2, 256, 256), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, inst.n_patches, inst.margin, inst.exposure, inst.readmask,
                   pixel_area=0.5)
    lam = R(inst.sky)
    data = np.concatenate([synthetic.poisson_data(l, seed=5 + i) for i, l in enumerate(lam)])
    plan = ju.ResponsePlan(2, 2, inst.shape, inst.n_patches, inst.margin, dtype=torch.float32,
                           pixel_area=0.5)
    plan.set_psf(inst.psf.astype(np.float32))
    plan.set_exposure(inst.exposure, inst.readmask)
    plan.set_data(data)
    parts = np.split(data, np.cumsum([l.size for l in lam])[:-1])
    e_ref, g_ref = R.energy_and_grad(inst.sky, parts)
    # R^T(d / lam): the term that cancels in R^T(1 - d/lam), the scale of the
    # FP32 gradient's error
    cancel = R.adjoint([d / l for d, l in zip(parts, lam)])
    yield inst, plan, np.concatenate(lam), e_ref, (g_ref, cancel)
    plan.close()


@pytest.mark.parametrize("run_len", [1, 2, 4])
def test_every_run_length_matches_the_oracle(cuda, demo, run_len):
    inst, plan, lam_ref, e_ref, (g_ref, cancel) = demo
    plan.set_forward_run(run_len)
    assert plan.forward_run == run_len
    x = torch.as_tensor(inst.sky, dtype=torch.float32, device=cuda)
    lam = plan.response(x)
    assert _rel(lam.cpu().numpy(), lam_ref) < 1e-6
    e, g = plan.energy_and_grad(x)
    assert abs(float(e) - e_ref) <= 1e-6 * abs(e_ref)
    # the gradient's FP32 error is that of the FP32 forward's lam, relative to the
    # cancelling term R^T(d / lam)
    gd = g.double().cpu().numpy()
    assert np.linalg.norm(gd - g_ref) < 3e-6 * np.linalg.norm(cancel)
    bits = (_bits(lam), _bits(e), _bits(g))
    for _ in range(2):
        lam2 = plan.response(x)
        e2, g2 = plan.energy_and_grad(x)
        assert (_bits(lam2), _bits(e2), _bits(g2)) == bits
    plan.set_forward_run(0)


def test_run_lengths_agree_to_fp32_rounding(cuda, demo):
    inst, plan, *_ = demo
    x = torch.as_tensor(inst.sky, dtype=torch.float32, device=cuda)
    out = {}
    for r in (1, 2, 4):
        plan.set_forward_run(r)
        out[r] = plan.response(x).double().cpu().numpy()
    plan.set_forward_run(0)
    assert _rel(out[2], out[1]) < 2e-7 and _rel(out[4], out[1]) < 2e-7


def _auto_choice(M, E, n, sms):
    """The library's rule: the run length whose busiest CTA does the least work."""
    U = M * E * n * n
    best, cost = 1, math.ceil(U / sms)
    for r, f in ((2, 0.93), (4, 0.87)):
        if n % r == 0 and M >= 2:
            c = math.ceil(U // r / sms) * r * f
            if c < cost:
                best, cost = r, c
    return best


@pytest.mark.parametrize("geom", [(256, 2, 2), (512, 2, 3), (1024, 7, 3), (1024, 2, 3)],
                         ids=["256x2x2", "erosita-demo-512x2x3", "1024x7x3", "1024x2x3"])
def test_library_choice_follows_the_sm_count(cuda, geom):
    nx, M, E = geom
    plan = ju.ResponsePlan(M, E, (nx, nx), nx // 64, 32, dtype=torch.float32)
    try:
        sms = torch.cuda.get_device_properties(cuda).multi_processor_count
        assert plan.forward_run == _auto_choice(M, E, nx // 64, sms)
    finally:
        plan.close()


def test_run_length_errors(cuda, demo):
    _, plan, *_ = demo
    with pytest.raises(ValueError):
        plan.set_forward_run(3)
    # n = 6 patches per axis: runs of 4 do not tile the column
    p6 = ju.ResponsePlan(2, 1, (384, 384), 6, 32, dtype=torch.float32)
    try:
        p6.set_forward_run(2)
        assert p6.forward_run == 2
        with pytest.raises(_lib.JubikUnsupported):
            p6.set_forward_run(4)
        assert p6.forward_run == 2
    finally:
        p6.close()
    # FP64 and one-module plans have no runs
    p64 = ju.ResponsePlan(2, 1, (256, 256), 4, 32, dtype=torch.float64)
    try:
        with pytest.raises(_lib.JubikUnsupported):
            p64.set_forward_run(2)
        assert p64.forward_run == 1
    finally:
        p64.close()


def test_autotune_keeps_the_fastest(cuda, demo):
    inst, plan, *_ = demo
    x = torch.as_tensor(inst.sky, dtype=torch.float32, device=cuda)
    times = plan.autotune(x, reps=3)
    assert set(times) == {1, 2, 4}
    assert all(t > 0 for t in times.values())
    assert plan.forward_run == min(times, key=times.get)
    plan.set_forward_run(0)
