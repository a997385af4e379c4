"""Repeated calls give the same bits on the fused paths.

The fused overlap-add and the gradient scatter accumulate in two words whose
sums are exact (any order of the atomic reductions gives the same bits), and
the module-shared adjoint sums each patch over modules in module order in
tensor memory.  So every output of a one-problem call -- the image, the
readout, the energy, the gradient, the VJP, the metric product -- is bitwise
reproducible.  Values are checked against the float64 oracle as well.
"""
import numpy as np
import pytest
import torch

import jubik_oracle as O
import jubik_gb300 as ju
from jubik_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _bits(t):
    return t.detach().reshape(-1).contiguous().view(torch.uint8).cpu().numpy().tobytes()


def _plan(inst, dtype, path, data):
    plan = ju.ResponsePlan(inst.n_modules, inst.n_energies, inst.shape, inst.n_patches,
                           inst.margin, dtype=dtype, path=path, pixel_area=0.5)
    plan.set_psf(inst.psf.astype(np.float64 if dtype == torch.float64 else np.float32))
    plan.set_exposure(inst.exposure, inst.readmask)
    plan.set_data(data)
    return plan


CASES = [  # (nx, dx, margin, modules, energies, dtype, path)
    (256, 64, 32, 7, 3, torch.float32, "auto"),      # the config-2 geometry, module-shared
    (256, 64, 32, 2, 2, torch.float32, "fused_unit"),  # one CTA per unit
    (128, 32, 32, 3, 2, torch.float64, "auto"),       # FP64 module-shared (P = 128)
    (96, 16, 16, 1, 2, torch.float64, "auto"),        # FP64 per-unit (one module, P = 64)
]


@pytest.mark.parametrize("case", CASES, ids=["f32-shared-192", "f32-unit-192",
                                                 "f64-shared-128", "f64-unit-64"])
def test_repeated_calls_are_bitwise_identical(cuda, case):
    nx, dx, m, M, E, dtype, path = case
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, inst.n_patches, inst.margin, inst.exposure, inst.readmask,
                   pixel_area=0.5)
    lam = R(inst.sky)
    data = np.concatenate([synthetic.poisson_data(l, seed=3 + i) for i, l in enumerate(lam)])
    plan = _plan(inst, dtype, path, data)
    try:
        assert plan.path == "fused"
        x = torch.as_tensor(inst.sky, dtype=dtype, device=cuda)
        rng = np.random.default_rng(9)
        v = torch.as_tensor(rng.standard_normal(x.shape), dtype=dtype, device=cuda)
        cot = torch.as_tensor(rng.standard_normal(plan.readout_total), dtype=dtype, device=cuda)
        runs = []
        for _ in range(3):
            e, g = plan.energy_and_grad(x)
            out = {"energy": e.clone(), "grad": g.clone(), "lam": plan.response(x),
                   "psf": plan.psf_forward(x), "vjp": plan.response_vjp(cot),
                   "metric": plan.metric(x, v)}
            torch.cuda.synchronize()
            runs.append(out)
        for k in runs[0]:
            for r in runs[1:]:
                assert _bits(r[k]) == _bits(runs[0][k]), k
        # and the values are the oracle's (tolerances of the parity tests)
        tol = 1e-12 if dtype == torch.float64 else 1e-6
        ref = np.concatenate(lam)
        got = runs[0]["lam"].double().cpu().numpy()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < tol
        e_ref, _ = R.energy_and_grad(inst.sky, np.split(data, np.cumsum(plan.readout_sizes)[:-1]))
        assert abs(float(runs[0]["energy"]) - e_ref) / abs(e_ref) < (1e-12 if dtype ==
                                                                      torch.float64 else 1e-6)
    finally:
        plan.close()
