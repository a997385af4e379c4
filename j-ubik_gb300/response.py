"""GB300 drop-ins for ``jubik/response.py`` (exposure and readout).

``build_readout_function`` returns a :class:`Vector`, a minimal stand-in for
``nifty.re.Vector`` with the same ``.tree`` dict interface.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .plan import as_device, dtype_code, ptr, require_cuda, stream_handle


class Vector:
    """Dict-of-arrays container with the ``.tree`` interface of ``jft.Vector``."""

    def __init__(self, tree):
        self.tree = dict(tree)

    def __getitem__(self, k):
        return self.tree[k]

    def keys(self):
        return self.tree.keys()

    def items(self):
        return self.tree.items()

    def values(self):
        return self.tree.values()

    def __len__(self):
        return len(self.tree)

    def _map2(self, other, op):
        if isinstance(other, Vector):
            return Vector({k: op(v, other.tree[k]) for k, v in self.tree.items()})
        return Vector({k: op(v, other) for k, v in self.tree.items()})

    def __add__(self, o):
        return self._map2(o, lambda a, b: a + b)

    def __sub__(self, o):
        return self._map2(o, lambda a, b: a - b)

    def __mul__(self, o):
        return self._map2(o, lambda a, b: a * b)

    def __truediv__(self, o):
        return self._map2(o, lambda a, b: a / b)

    __radd__ = __add__
    __rmul__ = __mul__

    def __repr__(self):
        return "Vector(" + ", ".join(f"{k}: {tuple(v.shape)}" for k, v in self.tree.items()) + ")"


def _float_dtype(a) -> torch.dtype:
    dt = a.dtype if isinstance(a, torch.Tensor) else np.asarray(a).dtype
    return torch.float32 if dt in (torch.float32, np.float32) else torch.float64


def build_exposure_function(exposures, exposure_cut=None):
    """Returns ``exposure(x) = exposures * x`` (``jubik/response.py:12-45``).

    As in the reference, the threshold is applied to ``exposures`` in place and
    a negative ``exposure_cut`` raises ValueError.  The product runs on the GPU."""
    if exposure_cut is not None:
        if exposure_cut < 0:
            raise ValueError("exposure_cut should be non-negative or None!")
        exposures[exposures < exposure_cut] = 0
    dev = require_cuda()
    ex = as_device(exposures, _float_dtype(exposures), dev)

    def exposure(x):
        xt = as_device(x, ex.dtype, dev)
        a, b = torch.broadcast_tensors(ex, xt)
        a, b = a.contiguous(), b.contiguous()
        out = torch.empty_like(a)
        _lib.call("jubik_elementwise", 3, ptr(a), ptr(b), None, a.numel(), dtype_code(a.dtype),
                  ptr(out), stream_handle(dev))
        return out

    return exposure


def build_readout_function(flags, threshold=None, keys=None):
    """Readout of the pixels where ``flags != 0`` (``jubik/response.py:48-112``).

    Returns a callable ``x -> Vector({key_i: x[i][~mask[i]]})`` in C order, with
    the reference's in-place threshold and its ValueError branches."""
    if threshold is not None and threshold < 0:
        raise ValueError("threshold should be positive!")
    if threshold is not None:
        flags[flags < threshold] = 0
    mask = np.asarray(flags.cpu() if isinstance(flags, torch.Tensor) else flags) == 0
    if keys is None:
        keys = ['masked input']
    elif len(keys) != flags.shape[0]:
        raise ValueError("length of keys should match the number of flag maps.")
    state = {}

    def _index(dev):
        if "idx" not in state:
            per = int(np.prod(mask.shape[1:]))
            flat = [np.flatnonzero(~mask[i].reshape(-1)) + i * per for i in range(len(keys))]
            state["sizes"] = [len(f) for f in flat]
            state["idx"] = torch.as_tensor(np.concatenate(flat).astype(np.int64), device=dev)
        return state["idx"], state["sizes"]

    def _apply_readout(x):
        if len(mask.shape) != 4:
            raise ValueError("flags should have shape (n, m, q, l)!")
        if len(x.shape) != 4:
            raise ValueError("input should have shape (n, m, q, l)!")
        dev = require_cuda()
        xt = as_device(x, _float_dtype(x), dev)
        idx, sizes = _index(dev)
        out = torch.empty(idx.numel(), dtype=xt.dtype, device=dev)
        _lib.call("jubik_readout_gather", ptr(xt), None, ptr(idx), idx.numel(),
                  dtype_code(xt.dtype), ptr(out), stream_handle(dev))
        parts = torch.split(out, sizes)
        return Vector({key: parts[i] for i, key in enumerate(keys)})

    def _adjoint(vec):
        """Transpose of the readout (``jax.linear_transpose`` of it, as the
        reference's callers build at ``data.py:156``, ``diagnostics.py:101``):
        the readout vectors scattered back into zero (n, m, q, l) images."""
        dev = require_cuda()
        if isinstance(vec, Vector):
            parts = [vec.tree[k] for k in keys]
        elif isinstance(vec, dict):
            parts = [vec[k] for k in keys]
        else:
            parts = list(vec)
        flat = torch.cat([as_device(v, None, dev).reshape(-1) for v in parts])
        if not flat.is_floating_point():
            flat = flat.to(torch.float64)
        idx, sizes = _index(dev)
        if flat.numel() != idx.numel():
            raise ValueError("readout vectors do not match the mask")
        img = torch.zeros(mask.shape, dtype=flat.dtype, device=dev)
        _lib.call("jubik_readout_scatter", ptr(flat), None, ptr(idx), idx.numel(),
                  dtype_code(flat.dtype), ptr(img), stream_handle(dev))
        return img

    _apply_readout.mask = mask
    _apply_readout.keys = list(keys)
    _apply_readout.adjoint = _adjoint
    return _apply_readout
