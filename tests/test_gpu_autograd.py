"""Autograd drop-ins that share one plan between kernels.

``linpatch_convolve`` keeps one plan per geometry and ``build_psf_op`` one plan
per closure; a plan holds one set of PSF spectra at a time.  These tests put
two kernels on one geometry into one graph, and evict a plan from the cache
before the backward pass, and check the gradients against the float64 oracle's
adjoint (``jubik/convolve.py:66-145``, transposed).
"""
import numpy as np
import pytest
import torch

import importlib

import jubik_oracle as O
import jubik_gb300 as ju

jc = importlib.import_module("jubik_gb300.convolve")  # the module (the package exports the function)

pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-12, torch.float32: 1e-6}


def rel(a, b):
    a = a.detach().double().cpu().numpy()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _kernels(rng, n2, E, K, count):
    ks = []
    for _ in range(count):
        k = rng.random((n2, E, K, K)) ** 4
        ks.append(k / k.sum(axis=(-2, -1), keepdims=True))
    return ks


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_two_kernels_one_geometry_one_graph(cuda, dtype):
    rng = np.random.default_rng(11)
    nx, n, m, E = 64, 4, 8, 2
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    x0 = rng.random((E, nx, nx)) + 0.5
    kA, kB = _kernels(rng, n * n, E, 2 * nx // n, 2)
    wA, wB = rng.standard_normal((2, E, nx, nx))
    x = torch.tensor(x0, dtype=dtype, device=cuda, requires_grad=True)
    dd = ju.Domain(dom.shape, dom.distances)
    yA = ju.linpatch_convolve(x, dd, torch.tensor(kA, dtype=dtype, device=cuda), n, m)
    yB = ju.linpatch_convolve(x, dd, torch.tensor(kB, dtype=dtype, device=cuda), n, m)
    loss = (torch.tensor(wA, dtype=dtype, device=cuda) * yA).sum() + \
        (torch.tensor(wB, dtype=dtype, device=cuda) * yB).sum()
    loss.backward()
    ref = (O.linpatch_convolve_adjoint(wA, dom, kA, n, m, precut=True) +
           O.linpatch_convolve_adjoint(wB, dom, kB, n, m, precut=True))
    assert rel(x.grad, ref) < TOL[dtype]
    # and the forward values of both terms
    assert rel(yA, O.linpatch_convolve(x0, dom, kA, n, m, precut=True)) < TOL[dtype]
    assert rel(yB, O.linpatch_convolve(x0, dom, kB, n, m, precut=True)) < TOL[dtype]


def test_evicted_plan_keeps_its_graph(cuda):
    rng = np.random.default_rng(12)
    nx, n, m = 32, 4, 4
    dom = O.Domain((nx, nx), (1.0, 1.0))
    x0 = rng.random((nx, nx)) + 0.5
    (k,) = _kernels(rng, n * n, 1, 2 * nx // n, 1)
    k = k[:, 0]
    w = rng.standard_normal((nx, nx))
    x = torch.tensor(x0, dtype=torch.float64, device=cuda, requires_grad=True)
    y = ju.linpatch_convolve(x, ju.Domain(dom.shape, dom.distances), k, n, m)
    # fill the cache with other geometries so that this plan is evicted
    for j in range(jc._CACHE.capacity + 2):
        sz = 16 * (j + 3)
        ju.linpatch_convolve(np.ones((sz, sz)), ju.Domain((sz, sz), (1.0, 1.0)),
                             np.full((16, 2 * sz // 4, 2 * sz // 4), 1.0), 4, 4)
    (torch.tensor(w, device=cuda) * y).sum().backward()
    ref = O.linpatch_convolve_adjoint(w, dom, k, n, m, precut=True)
    assert rel(x.grad, ref) < 1e-12


def test_psf_op_two_kernels_one_graph(cuda):
    rng = np.random.default_rng(13)
    nx, n, m, E, M = 64, 4, 8, 1, 2
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    op = ju.build_psf_op(ju.Domain(dom.shape, dom.distances), n, m, dtype=torch.float64)
    x0 = rng.random((E, nx, nx)) + 0.5
    kA = np.stack(_kernels(rng, n * n, E, 2 * nx // n, M))
    kB = np.stack(_kernels(rng, n * n, E, 2 * nx // n, M))
    wA, wB = rng.standard_normal((2, M, E, nx, nx))
    x = torch.tensor(x0, device=cuda, requires_grad=True)
    loss = (torch.tensor(wA, device=cuda) * op(x, kA)).sum() + \
        (torch.tensor(wB, device=cuda) * op(x, kB)).sum()
    loss.backward()
    ref = sum(O.linpatch_convolve_adjoint(wA[i], dom, kA[i], n, m, precut=True) +
              O.linpatch_convolve_adjoint(wB[i], dom, kB[i], n, m, precut=True)
              for i in range(M))
    assert rel(x.grad, ref) < 1e-12


def test_inplace_kernel_edit_after_forward_raises(cuda):
    rng = np.random.default_rng(14)
    nx, n, m = 32, 4, 4
    (k,) = _kernels(rng, n * n, 1, 2 * nx // n, 1)
    kt = torch.tensor(k[:, 0], device=cuda)
    x = torch.ones((nx, nx), dtype=torch.float64, device=cuda, requires_grad=True)
    dd = ju.Domain((nx, nx), (1.0, 1.0))
    y = ju.linpatch_convolve(x, dd, kt, n, m)
    kt.mul_(2.0)  # the first kernel changes in place ...
    ju.linpatch_convolve(x, dd, kt, n, m)  # ... and the plan takes the new values
    with pytest.raises(RuntimeError, match="modified in place"):
        y.sum().backward()
