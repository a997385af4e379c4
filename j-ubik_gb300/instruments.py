"""Instrument response builders with the call shapes of J-UBIK's instruments.

* :func:`build_psf_op` mirrors the ``psf_op(x, kernel)`` closure of
  ``build_erosita_psf`` (``erosita_response.py:168-214``): ``linpatch_convolve``
  vmapped over the module axis of ``kernel``.
* :func:`build_response` mirrors the composition of
  ``build_erosita_response`` (``erosita_response.py:217-358``) and
  ``build_chandra_response_from_config`` (``chandra_response.py:127-149``)
  without their file I/O: ``R(x[, k]) = mask(exposure(psf(x * pixel_area, k)))``
  returning a :class:`~.response.Vector` keyed by module.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np
import torch

from .autograd import PsfOpFn, ResponseFn
from .convolve import _is_domain, _kernel_key
from .plan import ResponsePlan, as_device, require_cuda
from .response import Vector, build_exposure_function, build_readout_function


def _np(a):
    return a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)


def build_psf_op(domain, npatch: int, margin: int, dtype: torch.dtype = torch.float64,
                 path: str = "auto"):
    """``psf_op(x, kernel) -> (M, E, N, N)``, differentiable in ``x``."""
    if not _is_domain(domain):
        raise ValueError("domain has to be an instance of jubik.Domain")
    shape = tuple(int(s) for s in domain.shape)
    E = int(np.prod(shape[:-2])) if len(shape) > 2 else 1
    state = {}

    def psf_op(x, kernel):
        dev = require_cuda()
        k = as_device(kernel, dtype, dev)
        M = int(k.shape[0])
        plan = state.get("plan")
        if plan is None or plan.n_modules != M:
            plan = ResponsePlan(M, E, shape[-2:], npatch, margin, dtype=dtype, path=path,
                                device=dev)
            state["plan"] = plan
        key, keep = _kernel_key(kernel)
        if plan.psf_key != key:
            kshape = tuple(k.shape)

            def shaped(t):
                return t if len(kshape) == 4 else t.reshape(M, npatch ** 2, E, kshape[-2],
                                                             kshape[-1])

            plan.set_psf(shaped(k), key=key, source=lambda: shaped(as_device(keep, dtype, dev)),
                         watch=keep if isinstance(keep, torch.Tensor) else None)
        xt = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x))
        xt = xt.to(device=dev, dtype=dtype).reshape((E,) + shape[-2:])
        out = PsfOpFn.apply(xt, plan)
        return out.reshape((M,) + shape)

    psf_op.state = state
    return psf_op


class Response:
    """``R(x[, k]) = mask(exposure(psf(x * pixel_area, k)))`` on one GPU plan.

    ``kernel`` (M, n^2, E, K, K) pre-cut or (M, n^2, E, N, N) full-field;
    ``exposures`` (M, E, N, N) (thresholded in place by ``exposure_cut`` as in
    ``response.py:40``; multiplied by ``effective_area`` (M, E) when given, as
    ``erosita_response.py:327-328``); ``flags`` (M, E, N, N) readout flags
    (default: the exposures), thresholded by ``threshold``; ``keys`` name the
    modules (``response.py:90``)."""

    def __init__(self, domain, kernel, n_patch: int, margin: int, exposures=None, flags=None,
                 exposure_cut: Optional[float] = None, threshold: Optional[float] = None,
                 keys: Optional[Sequence[str]] = None, pixel_area: float = 1.0,
                 effective_area=None, dtype: torch.dtype = torch.float32, path: str = "auto"):
        if not _is_domain(domain):
            raise ValueError("domain has to be an instance of jubik.Domain")
        dev = require_cuda()
        self.domain = domain
        shape = tuple(int(s) for s in domain.shape)
        self.shape = shape
        self.E = int(np.prod(shape[:-2])) if len(shape) > 2 else 1
        k = as_device(kernel, dtype, dev)
        self.M = int(k.shape[0])
        self.pixel_area = float(pixel_area)
        self.plan = ResponsePlan(self.M, self.E, shape[-2:], n_patch, margin, dtype=dtype,
                                 path=path, pixel_area=self.pixel_area, device=dev)
        self._use_kernel(kernel, k)
        self.kernel = k
        full = (self.M, self.E) + shape[-2:]
        exp = None
        if exposures is not None:
            # the in-place threshold of response.py:40 on the caller's array
            self.exposure = build_exposure_function(exposures, exposure_cut)
            exp = _np(exposures).astype(np.float64).reshape(full)
            if effective_area is not None:
                exp = exp * _np(effective_area).reshape(self.M, self.E, 1, 1)
        else:
            self.exposure = None
        if flags is None and exposures is not None:
            flags = _np(exposures).copy()
        if flags is not None:
            self.mask_func = build_readout_function(flags, threshold, keys)
            readmask = ~self.mask_func.mask.reshape(full)
            self.keys = list(self.mask_func.keys)
        else:
            self.mask_func = None
            readmask = None
            self.keys = list(keys) if keys is not None else ['masked input']
        if len(self.keys) != self.M:
            raise ValueError("length of keys should match the number of flag maps.")
        self.plan.set_exposure(exp, readmask)

    def _use_kernel(self, src, kt=None) -> None:
        """Give the plan the kernels ``src`` unless it holds them already."""
        key, keep = _kernel_key(src)
        if self.plan.psf_key == key:
            return
        plan, M, E = self.plan, self.M, self.E

        def shaped(t):
            return t if t.dim() == 4 else t.reshape(M, plan.n_patches ** 2, E, t.shape[-2],
                                                    t.shape[-1])

        if kt is None:
            kt = as_device(src, plan.dtype, plan.device)
        plan.set_psf(shaped(kt), key=key,
                     source=lambda: shaped(as_device(keep, plan.dtype, plan.device)),
                     watch=keep if isinstance(keep, torch.Tensor) else None)

    def _sky(self, x):
        dev = self.plan.device
        xt = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x))
        return xt.to(device=dev, dtype=self.plan.dtype).reshape((self.E,) + self.shape[-2:])

    def flat(self, x) -> torch.Tensor:
        """R(x) as one flat readout vector (modules concatenated)."""
        return ResponseFn.apply(self._sky(x), self.plan)

    def __call__(self, x, k=None) -> Vector:
        if k is not None:
            self._use_kernel(k)
        parts = torch.split(self.flat(x), self.plan.readout_sizes)
        return Vector(dict(zip(self.keys, parts)))

    def vjp(self, cot) -> torch.Tensor:
        """R^T applied to a readout Vector (or flat vector)."""
        if isinstance(cot, Vector):
            cot = torch.cat([cot.tree[k].reshape(-1) for k in self.keys])
        return self.plan.response_vjp(cot).reshape(self.shape)

    def psf(self, x, k=None):
        """(M, E, N, N) PSF images without pixel area (the vmapped linpatch)."""
        if k is not None:
            self._use_kernel(k)
        out = PsfOpFn.apply(self._sky(x), self.plan)
        return out.reshape((self.M,) + self.shape)


def build_response(domain, kernel, n_patch: int, margin: int, exposures=None, flags=None,
                   exposure_cut=None, threshold=None, keys=None, pixel_area: float = 1.0,
                   effective_area=None, dtype: torch.dtype = torch.float32, path: str = "auto"):
    """Response dictionary with the keys of ``build_erosita_response``
    (``erosita_response.py:352-358``): 'pix_area', 'psf', 'exposure', 'mask',
    'kernel', 'R', plus 'mask_adj', the readout transpose that the reference's
    diagnostics expect the caller to add (``diagnostics.py:101``)."""
    R = Response(domain, kernel, n_patch, margin, exposures=exposures, flags=flags,
                 exposure_cut=exposure_cut, threshold=threshold, keys=keys,
                 pixel_area=pixel_area, effective_area=effective_area, dtype=dtype, path=path)

    def psf_func(x, k=None):
        return R.psf(x, k)

    def mask_adj(vec):
        """Readout transpose in the form ``jax.linear_transpose`` returns it: a
        1-tuple holding the (M, E, N, N) image (``diagnostics.py:101``)."""
        if R.mask_func is None:
            raise ValueError("the response has no readout mask")
        return (R.mask_func.adjoint(vec),)

    return {"pix_area": R.pixel_area, "psf": psf_func, "exposure": R.exposure,
            "mask": R.mask_func, "mask_adj": mask_adj, "kernel": R.kernel, "R": R}
