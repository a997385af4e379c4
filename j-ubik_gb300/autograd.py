"""torch.autograd wrappers of the GB300 response kernels.

The response is linear in the sky, so its JVP is the forward kernel on the
tangent and its VJP is the hand-written adjoint kernel (correlation with the
PSF, transposed overlap-add, transposed exposure and readout).  The Poisson
energy returns its gradient from the same fused forward+adjoint pass.

A plan holds one set of PSF spectra at a time, and callers may give it other
kernels between a forward pass and its backward pass (two kernels on one
geometry in one graph).  Every node therefore keeps a snapshot of the PSF its
forward used and restores it before it runs the adjoint.
"""
from __future__ import annotations

import torch


class PsfOpFn(torch.autograd.Function):
    """x (E,nx,ny) -> (M,E,nx,ny): linpatch_convolve for every module."""

    @staticmethod
    def forward(ctx, x, plan):
        ctx.plan, ctx.psf = plan, plan.psf_snapshot()
        return plan.psf_forward(x)

    @staticmethod
    def backward(ctx, g):
        ctx.plan.restore_psf(ctx.psf)
        return ctx.plan.psf_adjoint(g.contiguous()), None

    @staticmethod
    def jvp(ctx, t, _):
        ctx.plan.restore_psf(ctx.psf)
        return ctx.plan.psf_forward(t)


class ResponseFn(torch.autograd.Function):
    """x (E,nx,ny) -> flat readout of R(x)."""

    @staticmethod
    def forward(ctx, x, plan):
        ctx.plan, ctx.psf = plan, plan.psf_snapshot()
        return plan.response(x)

    @staticmethod
    def backward(ctx, g):
        ctx.plan.restore_psf(ctx.psf)
        return ctx.plan.response_vjp(g.contiguous()), None

    @staticmethod
    def jvp(ctx, t, _):
        ctx.plan.restore_psf(ctx.psf)
        return ctx.plan.response(t)


class PoissonEnergyFn(torch.autograd.Function):
    """x -> H(R(x)) (float64 scalar); dH/dx from the fused pass."""

    @staticmethod
    def forward(ctx, x, plan):
        e, g = plan.energy_and_grad(x, need_grad=True)
        ctx.save_for_backward(g)
        return e

    @staticmethod
    def backward(ctx, ge):
        (g,) = ctx.saved_tensors
        return (ge.to(g.dtype) * g), None


class LogSkyPoissonEnergyFn(torch.autograd.Function):
    """s -> H(R(exp(s[:E, :nx, :ny]))) (float64 scalar) for a padded log-sky s,
    the exp_padding of ``jubik/sky_models.py:340-341``; dH/ds from the fused pass."""

    @staticmethod
    def forward(ctx, s, plan):
        e, g = plan.energy_and_grad_logsky(s, need_grad=True)
        ctx.save_for_backward(g)
        return e

    @staticmethod
    def backward(ctx, ge):
        (g,) = ctx.saved_tensors
        return (ge.to(g.dtype) * g), None
