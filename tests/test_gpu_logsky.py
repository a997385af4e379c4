"""Log-sky input: the sky exp(s[:E, :nx, :ny]) of a padded log-sky array
(J-UBIK's exp_padding, jubik/sky_models.py:340-341) with exp and crop fused
into the response's first kernel, against the oracle on the materialised sky."""
import numpy as np
import pytest
import torch

import jubik_oracle as O
import jubik_gb300 as ju
from jubik_gb300 import synthetic

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def case():
    nx, dx, m, M, E = 128, 32, 16, 2, 2
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
    rng = np.random.default_rng(21)
    s = rng.normal(0.5, 0.8, size=(E + 1, nx + 10, nx + 6))   # padded log-sky
    x = np.exp(s[:E, :nx, :nx])
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, nx // dx, m, inst.exposure, inst.readmask, pixel_area=0.4)
    lam = R(x)
    data = [synthetic.poisson_data(l, 31 + i) for i, l in enumerate(lam)]
    e, gx = R.energy_and_grad(x, data)
    gs = np.zeros_like(s)
    gs[:E, :nx, :nx] = x * gx
    return dict(inst=inst, s=s, data=np.concatenate(data), energy=e, grad_s=gs,
                cancel=np.linalg.norm(x * R.adjoint([d / l for d, l in zip(data, lam)])))


@pytest.mark.parametrize("dtype,path", [(torch.float64, "fused"), (torch.float64, "plain"),
                                        (torch.float32, "fused"), (torch.float32, "plain")])
def test_logsky_energy_and_gradient(cuda, case, dtype, path):
    inst = case["inst"]
    nx = inst.shape[0]
    plan = ju.ResponsePlan(inst.n_modules, inst.n_energies, inst.shape, inst.n_patches,
                           inst.margin, dtype=dtype, path=path, pixel_area=0.4)
    plan.set_psf(inst.psf).set_exposure(inst.exposure, inst.readmask).set_data(case["data"])
    e, gs = plan.energy_and_grad_logsky(case["s"])
    tol = 1e-12 if dtype == torch.float64 else 1e-6
    assert abs(float(e) - case["energy"]) / abs(case["energy"]) < tol
    g = gs.double().cpu().numpy()
    assert (g[inst.n_energies:] == 0).all() and (g[:, nx:] == 0).all() and (g[:, :, nx:] == 0).all()
    if dtype == torch.float64:
        assert rel(g, case["grad_s"]) < 1e-11
    else:  # against the cancelling term, as for the sky gradient
        assert np.linalg.norm(g - case["grad_s"]) / case["cancel"] < 3e-6
    # the same as the energy of the materialised sky
    x = torch.as_tensor(np.exp(case["s"][:inst.n_energies, :nx, :nx]), device=cuda)
    e2, _ = plan.energy_and_grad(x)
    assert abs(float(e2) - float(e)) <= (1e-13 if dtype == torch.float64 else 1e-6) * abs(float(e))
    plan.close()


def test_logsky_autograd(cuda, case):
    inst = case["inst"]
    R = ju.Response(ju.Domain((inst.n_energies,) + inst.shape, (1.0, 1.0, 1.0)), inst.psf,
                    inst.n_patches, inst.margin, exposures=inst.exposure.copy(),
                    flags=inst.readmask.astype(float), pixel_area=0.4, dtype=torch.float64,
                    keys=["a", "b"])
    s0 = R.plan.readout_sizes[0]
    lh = ju.Poissonian(ju.Vector({"a": case["data"][:s0], "b": case["data"][s0:]})).amend(R)
    s = torch.tensor(case["s"], device=cuda, requires_grad=True)
    e = lh.energy_autograd_logsky(s)
    e.backward()
    assert rel(s.grad, case["grad_s"]) < 1e-11
    assert abs(float(e.detach()) - case["energy"]) / abs(case["energy"]) < 1e-12
