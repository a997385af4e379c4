"""Random draws and FP64 reductions on the GPU for the callers of the response.

* :func:`random_normal` -- standard normal deviates (the xi ~ N(0, 1) of an
  MGVI linear sample);
* :func:`random_poisson` -- Poisson deviates of expected counts (the mock
  data of ``jubik/data.py:143-146``, which draws ``jax.random.poisson`` per
  module);
* :func:`dot` -- sum(a * b) accumulated in FP64 in a fixed order (the global
  dot products of the conjugate-gradient step sizes).

Draws come from the counter-based Philox4x32-10 generator keyed by ``seed``:
element i of a call has its own counter, so a draw depends only on (seed,
offset, i), never on the launch shape; different ``offset`` values give
independent streams.  The generator differs from JAX's (threefry), so draws
match the reference in distribution, not value by value.
"""
from __future__ import annotations

from typing import Optional, Sequence, Union

import torch

from . import _lib
from .plan import as_device, dtype_code, ptr, require_cuda, stream_handle


def _dev(device: Optional[torch.device]) -> torch.device:
    return device if device is not None else require_cuda()


def random_normal(shape: Union[int, Sequence[int]], dtype: torch.dtype = torch.float32,
                  seed: int = 0, offset: int = 0,
                  device: Optional[torch.device] = None) -> torch.Tensor:
    """Standard normal deviates of ``shape`` on the GPU."""
    dev = _dev(device)
    out = torch.empty(shape, dtype=dtype, device=dev)
    _lib.call("jubik_random_normal", ptr(out), out.numel(), dtype_code(dtype),
              int(seed) & 0xFFFFFFFFFFFFFFFF, int(offset) & 0xFFFFFFFFFFFFFFFF,
              stream_handle(dev))
    return out


def random_poisson(lam, seed: int = 0, offset: int = 0,
                   device: Optional[torch.device] = None) -> torch.Tensor:
    """Poisson deviates (int32) of the expected counts ``lam`` (same shape).
    Raises ValueError for negative or NaN expected counts."""
    dev = _dev(device)
    t = as_device(lam, None, dev)
    if not t.is_floating_point():
        t = t.to(torch.float64)
    out = torch.empty(t.shape, dtype=torch.int32, device=dev)
    _lib.call("jubik_random_poisson", ptr(t), t.numel(), dtype_code(t.dtype),
              int(seed) & 0xFFFFFFFFFFFFFFFF, int(offset) & 0xFFFFFFFF, ptr(out),
              stream_handle(dev))
    if t.numel() and bool((out < 0).any()):
        raise ValueError("expected counts must be finite, >= 0 and below 2e9")
    return out


def dot(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """sum(a * b) as a float64 0-d device tensor, summed in a fixed order
    (float32 operands: compensated FP32 partial sums flushed into FP64)."""
    if a.shape != b.shape or a.dtype != b.dtype:
        raise ValueError("dot needs two tensors of the same shape and dtype")
    dev = a.device
    a = a.contiguous()
    b = b.contiguous()
    out = torch.empty((), dtype=torch.float64, device=dev)
    _lib.call("jubik_dot", ptr(a), ptr(b), a.numel(), dtype_code(a.dtype), ptr(out),
              stream_handle(dev))
    return out
