"""The CUDA path against outputs of J-UBIK's own code.

``tests/golden/ref_*.npz`` hold outputs of the reference's unmodified
``jubik/convolve.py`` (``slice_patches``, ``linpatch_convolve`` with full-field
and energy-broadcast kernels, odd strides, its VJP, ``convolve``) and
``jubik/response.py`` (exposure and readout), evaluated through the numpy
JAX stand-in of ``tests/golden/make_ref_fixtures.py``.  Tiers: slicing and
readout bit-exact; FP64 1e-12 relative L2; FP32 1e-6.
"""
import os

import numpy as np
import pytest
import torch

import jubik_gb300 as ju

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = {torch.float64: 1e-12, torch.float32: 1e-6}


def cases(name):
    d = np.load(os.path.join(HERE, name + ".npz"))
    out = {}
    for k in d.files:
        if "/" in k:
            c, f = k.split("/", 1)
            out.setdefault(c, {})[f] = d[k]
    return out


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("case", sorted(cases("ref_slice")))
def test_slice_patches_bit_exact_vs_reference(cuda, case):
    c = cases("ref_slice")[case]
    n, dr = int(c["n"]), int(c["dr"])
    p = ju.slice_patches(c["x"], c["x"].shape, n, dr)
    assert tuple(p.shape) == c["patches"].shape
    assert np.array_equal(p.cpu().numpy(), c["patches"])
    a = ju.slice_patches_adjoint(c["patches"], c["x"].shape, n, dr)
    assert np.array_equal(a.cpu().numpy(), c["adjoint"])


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("case", sorted(cases("ref_linpatch")))
def test_linpatch_convolve_vs_reference(cuda, case, dtype, capsys):
    c = cases("ref_linpatch")[case]
    dom = ju.Domain(c["x"].shape, tuple(float(v) for v in c["distances"]))
    n, m = int(c["n"]), int(c["margin"])
    x = torch.tensor(c["x"], dtype=dtype, device=cuda, requires_grad=True)
    k = torch.tensor(c["kernel"], dtype=dtype, device=cuda)
    y = ju.linpatch_convolve(x, dom, k, n, m)
    assert tuple(y.shape) == c["y"].shape
    assert rel(y, c["y"]) < TOL[dtype]
    assert capsys.readouterr().out == str(c["printed"])  # the broadcast message, or none
    if "xt" in c:
        (torch.tensor(c["cot"], dtype=dtype, device=cuda) * y).sum().backward()
        assert rel(x.grad, c["xt"]) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("case", sorted(cases("ref_convolve")))
def test_convolve_vs_reference(cuda, case, dtype, capsys):
    c = cases("ref_convolve")[case]
    dom = ju.Domain(c["y"].shape, tuple(float(v) for v in c["distances"]))
    out = ju.convolve(torch.tensor(c["x"], dtype=dtype), torch.tensor(c["y"], dtype=dtype), dom,
                      tuple(int(a) for a in c["axes"]))
    assert tuple(out.shape) == c["out"].shape
    err = np.max(np.abs(out.double().cpu().numpy() - c["out"]))
    assert err <= TOL[dtype] * max(1.0, np.max(np.abs(c["out"])))
    assert capsys.readouterr().out == str(c["printed"])


def test_exposure_and_readout_bit_exact_vs_reference(cuda):
    cs = cases("ref_response")
    for name in ("e0", "e20"):
        c = cs[name]
        ex = c["exposures"].copy()
        cut = None if np.isnan(c["cut"]) else float(c["cut"])
        out = ju.build_exposure_function(ex, cut)(c["x"])
        assert np.array_equal(out.cpu().numpy(), c["out"])
        assert np.array_equal(ex, c["thresholded"])  # the in-place cut of response.py:40
    for name in ("r0", "r500"):
        c = cs[name]
        flags = c["flags"].copy()
        thr = None if np.isnan(c["threshold"]) else float(c["threshold"])
        keys = None if name == "r0" else tuple(str(k) for k in c["keys"])
        vec = ju.build_readout_function(flags, thr, keys)(c["x"])
        assert [str(k) for k in vec.tree] == [str(k) for k in c["keys"]]
        vals = torch.cat([v.reshape(-1) for v in vec.tree.values()]).cpu().numpy()
        assert np.array_equal(vals, c["values"])
        assert np.array_equal(flags, c["thresholded"])  # the in-place cut of response.py:86
