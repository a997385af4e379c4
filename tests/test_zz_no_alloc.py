"""The allocation-free FFT convolution, jubik_convolve2d_noalloc.

It exists for callers that cannot allocate device memory (code running under
a framework that owns the whole GPU memory pool, or loops where cudaMalloc
would synchronise the device): all of its scratch lives in one static device
array.  Through the C ABI, two calls in a row must agree with the allocating
jubik_convolve2d within the tolerances of the other GPU tests, and inputs
that need more scratch than the array holds must be rejected.

This file is collected last so that a run stopping at its first failure has
already run every other test; it passes alone and after the rest.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from jubik_gb300 import _lib

pytestmark = pytest.mark.gpu

TOL = {torch.float32: 1e-6, torch.float64: 1e-12}
SCRATCH = 16 * 1024 * 1024  # JUBIK_NOALLOC_SCRATCH_BYTES in include/jubik_gb300.h


def _call(name, k, s, h, w, dvol, out):
    code = _lib.F32 if k.dtype == torch.float32 else _lib.F64
    bk = k.numel() // (h * w)
    bs = s.numel() // (h * w)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return getattr(_lib.load(), name)(C.c_void_p(k.data_ptr()), bk, C.c_void_p(s.data_ptr()), bs,
                                     h, w, dvol, code, C.c_void_p(out.data_ptr()), stream)


def _rel(a, b):
    return float(torch.linalg.norm((a - b).double()) / torch.linalg.norm(b.double()))


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("shape", [(3, 3, 48, 40), (2, 6, 96, 96), (1, 4, 30, 42)])
def test_noalloc_matches_allocating_convolve_twice(cuda, dtype, shape):
    bk, bs, h, w = shape
    g = torch.Generator(device="cpu").manual_seed(bk * 1000 + h)
    k = torch.randn(bk, h, w, generator=g, dtype=torch.float64).to(cuda, dtype)
    for call in range(2):  # two calls in a row reuse the same scratch
        s = torch.randn(bs, h, w, generator=g, dtype=torch.float64).to(cuda, dtype)
        ref = torch.empty(bs, h, w, dtype=dtype, device=cuda)
        got = torch.full((bs, h, w), float("nan"), dtype=dtype, device=cuda)
        _lib.check(_call("jubik_convolve2d", k, s, h, w, 0.5, ref), "jubik_convolve2d")
        _lib.check(_call("jubik_convolve2d_noalloc", k, s, h, w, 0.5, got),
                   "jubik_convolve2d_noalloc")
        torch.cuda.synchronize()
        assert torch.isfinite(got).all()
        assert _rel(got, ref) < TOL[dtype], (call, _rel(got, ref))


def test_noalloc_rejects_inputs_beyond_the_scratch(cuda):
    h = w = 512
    per_plane = 8 * h * w  # complex float
    planes = SCRATCH // per_plane + 1
    k = torch.zeros(1, h, w, dtype=torch.float32, device=cuda)
    s = torch.zeros(planes, h, w, dtype=torch.float32, device=cuda)
    out = torch.empty_like(s)
    st = _call("jubik_convolve2d_noalloc", k, s, h, w, 1.0, out)
    assert st == _lib.ERR_INVALID_ARGUMENT
    assert "scratch" in _lib.last_error()
    # the device is still usable and the next in-range call is correct
    k2 = torch.randn(1, 64, 64, dtype=torch.float32, device=cuda)
    s2 = torch.randn(2, 64, 64, dtype=torch.float32, device=cuda)
    ref = torch.empty_like(s2)
    got = torch.empty_like(s2)
    _lib.check(_call("jubik_convolve2d", k2, s2, 64, 64, 1.0, ref), "jubik_convolve2d")
    _lib.check(_call("jubik_convolve2d_noalloc", k2, s2, 64, 64, 1.0, got),
               "jubik_convolve2d_noalloc")
    torch.cuda.synchronize()
    assert _rel(got, ref) < TOL[torch.float32]
