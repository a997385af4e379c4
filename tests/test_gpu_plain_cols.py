"""The unfused path's fused column stage at every FFT side it covers.

For FFT sides P = 16 L1 with L1 in {10, 12, 16, 20, 24, 32}, the unfused path
runs the column passes of its 2-D transforms and the PSF product in one
kernel per set of columns closed under the mirror c -> P - c.  The forward
(`k_plain_cols_fwd`) transforms the sky pair's columns once and writes every
module's product with its columns transformed back.  The adjoint
(`k_plain_cols_adj`) sums the conjugate-PSF products over modules in module
order.

Each case has 3 x 3 patches, an odd count, so the last pair's second patch is
empty; two modules, one energy.  Tolerances against the float64 oracle: FP64
1e-12 (gradient 1e-11), FP32 1e-6 (gradient 3e-6 of the cancelling term
R^T(d / lam)).

With JUBIK_PLAIN_CHUNK_MODULES=1 every module is its own chunk.  The adjoint
then carries its module sum from chunk to chunk in spectral order, and the
results must be the same bits as with one chunk.
"""
import numpy as np
import pytest
import torch

import jubik_oracle as O
import jubik_gb300 as ju
from jubik_gb300 import synthetic

pytestmark = pytest.mark.gpu

F32, F64 = torch.float32, torch.float64

# (FFT side, patch stride, margin): P = 2 stride + 2 margin, field 3 strides
SIDES = [(160, 48, 32), (192, 64, 32), (256, 64, 64), (320, 128, 32), (384, 128, 64),
         (512, 128, 128)]


def _rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _bits(t):
    return t.detach().reshape(-1).contiguous().view(torch.uint8).cpu().numpy().tobytes()


def _plan(inst, dtype, data):
    plan = ju.ResponsePlan(inst.n_modules, inst.n_energies, inst.shape, inst.n_patches,
                           inst.margin, dtype=dtype, path="plain")
    plan.set_psf(inst.psf)
    plan.set_exposure(inst.exposure, inst.readmask)
    plan.set_data(data)
    return plan


@pytest.mark.parametrize("dtype", [F64, F32], ids=["f64", "f32"])
@pytest.mark.parametrize("side", SIDES, ids=[f"P{s[0]}" for s in SIDES])
def test_column_stage_matches_the_oracle(cuda, side, dtype, monkeypatch):
    P, dx, m = side
    nx, M, E = 3 * dx, 2, 1
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E, seed=P)
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, inst.n_patches, m, inst.exposure, inst.readmask)
    lam = R(inst.sky)
    parts = [synthetic.poisson_data(l, 3 + i) for i, l in enumerate(lam)]
    data = np.concatenate(parts)
    e_ref, g_ref = R.energy_and_grad(inst.sky, parts)
    cancel = R.adjoint([d / l for d, l in zip(parts, lam)])
    x = torch.as_tensor(inst.sky, dtype=dtype, device=cuda)

    plan = _plan(inst, dtype, data)
    try:
        assert plan.path == "plain" and plan.P == P
        tol = 1e-12 if dtype == F64 else 1e-6
        lam_gpu = plan.response(x)
        assert _rel(lam_gpu.cpu().numpy(), np.concatenate(lam)) < tol
        e, g = plan.energy_and_grad(x)
        assert abs(float(e) - e_ref) <= tol * abs(e_ref)
        gd = g.double().cpu().numpy()
        if dtype == F64:
            assert _rel(gd, g_ref) < 1e-11
        else:
            assert np.linalg.norm(gd - g_ref) < 3e-6 * np.linalg.norm(cancel)
        one_chunk = (_bits(lam_gpu), _bits(e), _bits(g))
    finally:
        plan.close()

    monkeypatch.setenv("JUBIK_PLAIN_CHUNK_MODULES", "1")
    plan = _plan(inst, dtype, data)
    try:
        lam1 = plan.response(x)
        e1, g1 = plan.energy_and_grad(x)
        assert (_bits(lam1), _bits(e1), _bits(g1)) == one_chunk
    finally:
        plan.close()
