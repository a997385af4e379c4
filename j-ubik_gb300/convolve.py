"""GB300 drop-ins for ``jubik/convolve.py`` (same names, arguments, errors).

Every function runs hand-written sm_103a kernels through the C ABI; there is
no CPU path.  Inputs may be numpy arrays or tensors; results are CUDA tensors.
"""
from __future__ import annotations

from functools import reduce
from typing import NamedTuple

import numpy as np
import torch

from . import _lib
from .plan import ResponsePlan, as_device, dtype_code, ptr, require_cuda, stream_handle


class Domain(NamedTuple):
    """Mimicking NIFTy Domain (``jubik/data.py:19-29``)."""

    shape: tuple
    distances: tuple


def _is_domain(d) -> bool:
    return isinstance(d, Domain) or (hasattr(d, "shape") and hasattr(d, "distances")
                                     and isinstance(d, tuple))


def _float_dtype(*arrays) -> torch.dtype:
    for a in arrays:
        dt = a.dtype if isinstance(a, torch.Tensor) else np.asarray(a).dtype
        if dt in (torch.float64, np.float64, torch.int64, np.int64, torch.int32, np.int32):
            return torch.float64
    return torch.float32


def _bilinear_weights(shape):
    """Build bilinear interpolation kernel (``jubik/convolve.py:18-25``).

    Host-side constant, as in the reference; raises ValueError for odd windows."""
    if shape[0] / 2 != int(shape[0] / 2):
        raise ValueError("this should happen")
    a = np.linspace(0, 1, int(shape[0] / 2), dtype="float64")
    b = np.concatenate([a, np.flip(a)])
    return np.outer(b, b)


def slice_patches(x, shape, n_patches_per_axis, additional_margin):
    """Slice into n^2 overlapping windows (``jubik/convolve.py:28-63``).

    Returns (n^2, *x.shape[:-2], 2dx+2dr, 2dy+2dr); patch k starts at padded
    row ``(k % n) * dx`` and column ``(k // n) * dy``."""
    dev = require_cuda()
    t = as_device(x, _float_dtype(x), dev)
    if tuple(shape[-2:]) != tuple(t.shape[-2:]):
        raise ValueError("shape must match the trailing axes of x")
    n, dr = int(n_patches_per_axis), int(additional_margin)
    nx, ny = int(t.shape[-2]), int(t.shape[-1])
    dx, dy = int((nx - 2 * dr) / n), int((ny - 2 * dr) / n)
    lead = tuple(t.shape[:-2])
    batch = int(np.prod(lead)) if lead else 1
    out = torch.empty((n * n,) + lead + (2 * dx + 2 * dr, 2 * dy + 2 * dr), dtype=t.dtype,
                      device=dev)
    _lib.call("jubik_slice_patches", ptr(t), batch, nx, ny, n, dr, dtype_code(t.dtype), ptr(out),
              stream_handle(dev))
    return out


def slice_patches_adjoint(patches, shape, n_patches_per_axis, additional_margin):
    """Transpose of :func:`slice_patches` (the ``jax.linear_transpose`` used as
    overlap-add at ``jubik/convolve.py:138-143``); returns ``shape``."""
    dev = require_cuda()
    t = as_device(patches, _float_dtype(patches), dev)
    n, dr = int(n_patches_per_axis), int(additional_margin)
    nx, ny = int(shape[-2]), int(shape[-1])
    lead = tuple(shape[:-2])
    batch = int(np.prod(lead)) if lead else 1
    out = torch.empty(tuple(shape), dtype=t.dtype, device=dev)
    _lib.call("jubik_slice_patches_adjoint", ptr(t), batch, nx, ny, n, dr, dtype_code(t.dtype),
              ptr(out), stream_handle(dev))
    return out


# ---------------------------------------------------------------- linpatch
class _PlanCache:
    """Plans keyed by geometry (the PSF spectra a plan holds carry their own key).

    An evicted plan is only dropped from the cache, never closed: an autograd
    graph that still holds it runs its backward pass on it, and the plan frees
    its device memory when the last reference goes."""

    def __init__(self, capacity: int = 8):
        self.capacity = capacity
        self.plans = {}

    def get(self, key, make):
        ent = self.plans.pop(key, None)
        if ent is None:
            ent = {"plan": make()}
            while len(self.plans) >= self.capacity:
                self.plans.pop(next(iter(self.plans)))
        self.plans[key] = ent
        return ent

    def clear(self):
        self.plans.clear()


_CACHE = _PlanCache()


def _kernel_key(src):
    """Cache key of a PSF kernel as the caller passed it, and the object to keep
    alive with the cached spectra.  A torch tensor is keyed by its storage and
    version counter (in-place edits change the version); any other array by
    its identity plus a sample of its values.  Keeping the source alive stops
    its storage or identity from being reused by a different kernel while
    the spectra are cached."""
    if isinstance(src, torch.Tensor):
        return ("tensor", src.data_ptr(), src._version, tuple(src.shape), src.dtype,
                str(src.device)), src
    a = np.asarray(src)
    flat = a.reshape(-1)
    sample = flat[:: max(1, flat.size // 4096)][:4096]
    return ("array", id(src), a.shape, a.dtype.str, hash(sample.tobytes())), src


def linpatch_plan(x_shape, kernel_shape, n_patches_per_axis, margin, dtype, n_modules=1):
    """(plan, layout, e_broadcast) for a linpatch call of these shapes."""
    dev = require_cuda()
    shape = tuple(int(s) for s in x_shape)
    lead = shape[:-2]
    E = int(np.prod(lead)) if lead else 1
    key = (shape, int(n_patches_per_axis), int(margin), dtype, dev.index, int(n_modules))
    ent = _CACHE.get(key, lambda: ResponsePlan(n_modules, E, shape[-2:], n_patches_per_axis,
                                               margin, dtype=dtype, device=dev))
    return ent


def _prepare_kernel(ent, src, kernel: torch.Tensor, E: int, field):
    """Kernels shaped like the field are full-field kernels (the reference's
    input, cut by convolve.py:107-111); any other window is taken as pre-cut.
    The plan's spectra are recomputed only when the kernel changed."""
    plan: ResponsePlan = ent["plan"]
    key, keep = _kernel_key(src)
    if plan.psf_key == key:
        return
    n2 = plan.n_patches ** 2
    layout = "full" if tuple(kernel.shape[-2:]) == tuple(field) else "precut"
    kshape = tuple(kernel.shape)

    def shaped(k):
        if len(kshape) == 3:  # (n^2, k, k): one kernel for every energy
            return k.unsqueeze(0)
        return k.reshape(1, n2, E, kshape[-2], kshape[-1])

    def again():  # the kernel as the caller passed it, on the device again
        return shaped(as_device(keep, plan.dtype, plan.device))

    plan.set_psf(shaped(kernel), layout, key=key, source=again,
                 watch=keep if isinstance(keep, torch.Tensor) else None)


class _LinpatchFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, plan):
        # the plan may hold another kernel when the backward pass runs
        ctx.plan, ctx.psf = plan, plan.psf_snapshot()
        return plan.psf_forward(x)[0] if plan.n_modules == 1 else plan.psf_forward(x)

    @staticmethod
    def backward(ctx, g):
        plan = ctx.plan
        plan.restore_psf(ctx.psf)
        gg = g.unsqueeze(0) if plan.n_modules == 1 else g
        return plan.psf_adjoint(gg.contiguous()), None


def linpatch_convolve(x, domain, kernel, n_patches_per_axis, margin):
    """Functional version of linear patching convolution
    (``jubik/convolve.py:66-145``), differentiable in ``x``.

    ``kernel`` is (n^2, *lead, N, N) full-field (as in the reference),
    (n^2, *lead, 2dx, 2dx) pre-cut, or without the ``lead`` axes (broadcast,
    with the reference's message)."""
    if not _is_domain(domain):
        raise ValueError("domain has to be an instance of jubik.Domain")
    dev = require_cuda()
    shape = tuple(int(s) for s in domain.shape)
    dtype = _float_dtype(x, kernel)
    xt = x if isinstance(x, torch.Tensor) and x.requires_grad else as_device(x, dtype, dev)
    if xt.dtype != dtype or xt.device != dev:
        xt = xt.to(device=dev, dtype=dtype)
    if tuple(xt.shape) != shape:
        raise ValueError(f"x has shape {tuple(xt.shape)}, the domain {shape}")
    kt = as_device(kernel, dtype, dev)
    lead = shape[:-2]
    E = int(np.prod(lead)) if lead else 1
    if kt.dim() not in (3, len(shape) + 1):
        raise ValueError(f"kernel of shape {tuple(kt.shape)} does not match x of shape {shape}")
    if kt.dim() < len(shape) + 1:  # the broadcast branch of convolve.py:167-171
        print("kernel_shape:", tuple(kt.shape))
        print("signal_shape:", (kt.shape[0],) + shape)
        print("Dimension Inconsistency. Broadcasting PSFs")
    ent = linpatch_plan(shape, tuple(kt.shape), n_patches_per_axis, margin, dtype)
    _prepare_kernel(ent, kernel, kt, E, shape[-2:])
    plan = ent["plan"]
    xin = xt.reshape((E,) + shape[-2:])
    out = _LinpatchFn.apply(xin, plan)
    return out.reshape(shape)


def convolve(x, y, domain, axes):
    """FFT convolution (``jubik/convolve.py:148-176``): ``x`` is the kernel,
    ``y`` the signal; ``dvol * Re(ifftn(fftn(x) * fftn(y)))`` over ``axes``."""
    dev = require_cuda()
    dtype = _float_dtype(x, y)
    xt = as_device(x, dtype, dev)
    yt = as_device(y, dtype, dev)
    dlist = [domain.distances[i] for i in axes]  # as convolve.py:161 (negative axes allowed)
    axes = tuple(a % yt.dim() for a in axes)
    dvol = float(reduce(lambda a, b: a * b, dlist))
    if len(axes) not in (1, 2):
        raise NotImplementedError("convolve covers one or two axes")
    broadcast = yt.dim() > xt.dim()
    if broadcast:
        print("kernel_shape:", tuple(xt.shape))
        print("signal_shape:", tuple(yt.shape))
        print("Dimension Inconsistency. Broadcasting PSFs")
    # move the transform axes last
    nd = yt.dim()
    perm = [a for a in range(nd) if a not in axes] + list(axes)
    ys = yt.permute(perm).contiguous()
    if broadcast:
        xs = xt.permute([a for a in range(xt.dim()) if a not in tuple(a - 1 for a in axes)] +
                        [a - 1 for a in axes]).contiguous()
    else:
        xs, ys = torch.broadcast_tensors(xt, yt)
        xs = xs.permute(perm).contiguous()
        ys = ys.permute(perm).contiguous()
    if len(axes) == 1:
        xs, ys = xs.unsqueeze(-2), ys.unsqueeze(-2)
    h, w = int(ys.shape[-2]), int(ys.shape[-1])
    bs = int(ys.numel() // (h * w))
    bk = int(xs.numel() // (h * w))
    out = torch.empty_like(ys)
    _lib.call("jubik_convolve2d", ptr(xs), bk, ptr(ys), bs, h, w, dvol, dtype_code(dtype),
              ptr(out), stream_handle(dev))
    if len(axes) == 1:
        out = out.squeeze(-2)
    inv = [0] * nd
    for i, p in enumerate(perm):
        inv[p] = i
    return out.permute(inv).contiguous()


def integrate(x, domain, axes):
    """Integrate on a domain (``jubik/convolve.py:179-184``)."""
    dev = require_cuda()
    t = as_device(x, _float_dtype(x), dev)
    s = t.sum(dim=tuple(axes))
    dlist = [domain.distances[i] for i in axes]
    return float(reduce(lambda a, b: a * b, dlist)) * s
