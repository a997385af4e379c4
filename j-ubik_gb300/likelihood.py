"""Poisson likelihood on the GB300 (stand-in for NIFTy.re ``jft.Poissonian``).

J-UBIK builds its likelihood as ``jft.Poissonian(masked_data).amend(model)``
(``jubik/instruments/erosita/erosita_likelihood.py:89``,
``jubik/instruments/chandra/chandra_likelihood.py:37``).  The energy is the
negative log-likelihood up to the constant ``log(d!)``:
``H(lam) = sum(lam) - sum(d * log(lam))`` (``demos/x-ray-imaging.py:312-315``);
its gradient is ``1 - d/lam``, the Fisher metric ``t / lam`` and the left
square-root metric ``t / sqrt(lam)``.  Totals are accumulated in FP64 on the
GPU.  When the model is a :class:`~.instruments.Response`, ``amend`` returns a
likelihood whose energy, gradient and metric run as fused response kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .plan import as_device, dtype_code, ptr, require_cuda, stream_handle
from .response import Vector


def _leaves(v):
    if isinstance(v, Vector):
        return list(v.tree.keys()), list(v.tree.values())
    if isinstance(v, dict):
        return list(v.keys()), list(v.values())
    if hasattr(v, "tree") and isinstance(v.tree, dict):
        return list(v.tree.keys()), list(v.tree.values())
    return None, [v]


def _is_integer(a) -> bool:
    if isinstance(a, torch.Tensor):
        return not a.is_floating_point() and not a.is_complex() and a.dtype != torch.bool
    return np.issubdtype(np.asarray(a).dtype, np.integer)


class Poissonian:
    """``jft.Poissonian(data)``: data must be integer and non-negative."""

    def __init__(self, data):
        keys, leaves = _leaves(data)
        if not all(_is_integer(d) for d in leaves):
            raise TypeError("`data` of invalid type; expected integer")
        dev = require_cuda()
        flat = [as_device(d, torch.int32, dev).reshape(-1) for d in leaves]
        if any(bool(torch.any(f < 0)) for f in flat):
            raise ValueError("`data` may not be negative")
        self.keys = keys
        self.sizes = [f.numel() for f in flat]
        self.data = torch.cat(flat) if flat else torch.empty(0, dtype=torch.int32, device=dev)
        self.device = dev

    # -------------------------------------------------------------- helpers
    def _flat(self, primals, dtype=None):
        _, leaves = _leaves(primals)
        t = [as_device(p, dtype, self.device).reshape(-1) for p in leaves]
        dt = dtype or (torch.float64 if any(x.dtype == torch.float64 for x in t)
                       else torch.float32)
        f = torch.cat([x.to(dt) for x in t])
        if f.numel() != self.data.numel():
            raise ValueError("primals do not match the data layout")
        return f

    def _unflat(self, flat):
        parts = torch.split(flat, self.sizes)
        if self.keys is None:
            return parts[0]
        return Vector(dict(zip(self.keys, parts)))

    # -------------------------------------------------------------- API
    def energy(self, primals) -> torch.Tensor:
        lam = self._flat(primals)
        e = torch.empty((), dtype=torch.float64, device=self.device)
        _lib.call("jubik_poisson_energy", ptr(lam), ptr(self.data), lam.numel(),
                  dtype_code(lam.dtype), ptr(e), None, stream_handle(self.device))
        return e

    __call__ = energy

    def energy_and_gradient(self, primals):
        """(H, dH/dlam) with dH/dlam = 1 - d/lam."""
        lam = self._flat(primals)
        e = torch.empty((), dtype=torch.float64, device=self.device)
        g = torch.empty_like(lam)
        _lib.call("jubik_poisson_energy", ptr(lam), ptr(self.data), lam.numel(),
                  dtype_code(lam.dtype), ptr(e), ptr(g), stream_handle(self.device))
        return e, self._unflat(g)

    def _elementwise(self, op, a, b=None):
        out = torch.empty_like(a)
        _lib.call("jubik_elementwise", op, ptr(a), ptr(b), ptr(self.data) if op == 2 else None,
                  a.numel(), dtype_code(a.dtype), ptr(out), stream_handle(self.device))
        return out

    def metric(self, primals, tangents):
        """Fisher metric applied to ``tangents``: t / lam."""
        lam = self._flat(primals)
        return self._unflat(self._elementwise(0, lam, self._flat(tangents, lam.dtype)))

    def left_sqrt_metric(self, primals, tangents):
        """t / sqrt(lam)."""
        lam = self._flat(primals)
        return self._unflat(self._elementwise(1, lam, self._flat(tangents, lam.dtype)))

    def normalized_residual(self, primals):
        """(d - lam) / sqrt(lam)."""
        lam = self._flat(primals)
        return self._unflat(self._elementwise(2, lam))

    def transformation(self, primals):
        """geoVI coordinate transformation 2 sqrt(lam) (its Jacobian squared is 1/lam)."""
        lam = self._flat(primals)
        return self._unflat(2.0 * torch.sqrt(lam))

    def amend(self, model):
        """Likelihood of ``model(x)``: fused GPU response when ``model`` is a
        :class:`~.instruments.Response`, torch autograd through it otherwise."""
        from .instruments import Response  # local import: module cycle
        if isinstance(model, Response):
            return ResponsePoissonian(model, self)
        return ModelPoissonian(model, self)


class ResponsePoissonian:
    """``Poissonian(d).amend(R)`` for the GB300 response: energy, gradient and
    MGVI metric run as fused response kernels."""

    def __init__(self, response, lh: Poissonian):
        self.response = response
        self.likelihood = lh
        plan = response.plan
        if lh.data.numel() != plan.readout_total:
            raise ValueError("data size does not match the response readout")
        if lh.keys is not None and response.keys is not None and list(lh.keys) != list(
                response.keys):
            raise ValueError("data keys do not match the response keys")
        plan.set_data(lh.data)

    def energy(self, x) -> torch.Tensor:
        e, _ = self.response.plan.energy_and_grad(x, need_grad=False)
        return e

    __call__ = energy

    def energy_and_gradient(self, x):
        return self.response.plan.energy_and_grad(x, need_grad=True)

    def metric(self, x, v):
        """R^T diag(1/lam) R v at lam = R(x) (x=None reuses the last lam)."""
        return self.response.plan.metric(x, v)

    def energy_autograd(self, x: torch.Tensor) -> torch.Tensor:
        """Energy as a differentiable torch scalar (gradient from the same fused pass)."""
        from .autograd import PoissonEnergyFn
        return PoissonEnergyFn.apply(x, self.response.plan)

    def energy_and_gradient_logsky(self, s):
        """Energy and dE/ds for the sky exp(s[:E, :nx, :ny]) of a padded log-sky
        (the exp_padding of ``jubik/sky_models.py:340-341``), exp and crop fused
        into the response's first kernel."""
        return self.response.plan.energy_and_grad_logsky(s)

    def energy_autograd_logsky(self, s: torch.Tensor) -> torch.Tensor:
        """Differentiable energy of a padded log-sky s (for a torch sky model)."""
        from .autograd import LogSkyPoissonEnergyFn
        return LogSkyPoissonEnergyFn.apply(s, self.response.plan)


class ModelPoissonian:
    """``Poissonian(d).amend(f)`` for an arbitrary differentiable torch model."""

    def __init__(self, model, lh: Poissonian):
        self.model = model
        self.likelihood = lh

    def energy(self, x):
        return self.likelihood.energy(self.model(x))

    __call__ = energy

    def energy_and_gradient(self, x):
        xt = x.detach().clone().requires_grad_(True)
        lam = self.model(xt)
        flat = self.likelihood._flat(lam)
        e, g = self.likelihood.energy_and_gradient(flat.detach())
        gflat = self.likelihood._flat(g, flat.dtype)
        (grad,) = torch.autograd.grad(flat, xt, gflat)
        return e, grad
