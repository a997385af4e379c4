"""The MGVI linear-sample solve around the metric product, on the GPU.

:func:`conjugate_gradient` solves ``mat(x) = j`` for a symmetric positive
definite ``mat`` by conjugate gradients with every global dot product
accumulated in FP64 on the device (:func:`jubik_gb300.sampling.dot`), the
stopping rules that ``jubik/minimization_parser.py:337-420`` configures for
NIFTy.re's ``conjugate_gradient`` (``absdelta``, ``tol``, ``atol``,
``miniter``, ``maxiter``).

:func:`draw_linear_sample` draws one MGVI linear residual sample of the
response likelihood in the sky coordinates of a standard-normal prior:
``z = R^T(xi_d / sqrt(lam)) + xi_x`` has covariance ``M + 1`` with the Poisson
metric ``M = R^T diag(1/lam) R`` (its left square root applied to normal
data-space noise, plus prior noise), and ``s = (M + 1)^{-1} z`` has the
covariance ``(M + 1)^{-1}`` of the MGVI approximation.  Priors other than
the standard normal enter through the caller's model Jacobian and are not
part of this path.
"""
from __future__ import annotations

from typing import Callable, Optional, Tuple

import torch

from .sampling import dot, random_normal


def conjugate_gradient(mat: Callable[[torch.Tensor], torch.Tensor], j: torch.Tensor,
                       x0: Optional[torch.Tensor] = None, *, absdelta: Optional[float] = None,
                       tol: float = 1e-5, atol: float = 0.0, miniter: Optional[int] = None,
                       maxiter: Optional[int] = None) -> Tuple[torch.Tensor, dict]:
    """Solve ``mat(x) = j``, minimising ``E(x) = 0.5 <x, mat x> - <j, x>``.

    Stops after at least ``miniter`` iterations once the residual norm is at
    most ``max(tol * |j|, atol)`` or an iteration lowered E by less than
    ``absdelta``; at most ``maxiter`` iterations (default 10 n).  Returns
    ``(x, info)`` with the iteration count, final residual norm and energy.
    Raises ValueError when ``mat`` is not positive definite along a search
    direction."""
    x = torch.zeros_like(j) if x0 is None else x0.clone()
    r = j.clone() if x0 is None else j - mat(x)
    d = r.clone()
    gamma = float(dot(r, r))
    energy = -0.5 * float(dot(x, r + j))
    miniter = miniter or 0
    maxiter = maxiter if maxiter is not None else 10 * j.numel()
    bound = max(tol * float(dot(j, j)) ** 0.5, atol)
    it = 0
    while it < maxiter:
        if gamma ** 0.5 <= bound and it >= miniter:
            break
        q = mat(d)
        curv = float(dot(d, q))
        if not curv > 0.0:
            raise ValueError("conjugate_gradient: the matrix is not positive definite")
        alpha = gamma / curv
        x.add_(d, alpha=alpha)
        r.sub_(q, alpha=alpha)
        new_gamma = float(dot(r, r))
        new_energy = -0.5 * float(dot(x, r + j))
        it += 1
        delta = energy - new_energy
        energy = new_energy
        if absdelta is not None and it >= miniter and delta < absdelta:
            break
        d.mul_(new_gamma / gamma).add_(r)
        gamma = new_gamma
    return x, {"iterations": it, "residual_norm": gamma ** 0.5, "energy": energy}


def draw_linear_sample(likelihood, x: torch.Tensor, seed: int = 0,
                       **cg_kwargs) -> Tuple[torch.Tensor, dict]:
    """One MGVI linear residual sample around ``x`` for a likelihood built by
    ``Poissonian(data).amend(response)`` (fused GPU response).  Returns the
    sample (shape of x) and the CG info."""
    plan = likelihood.plan if hasattr(likelihood, "plan") else likelihood.response.plan
    xs = plan._sky(x)
    plan.energy_and_grad(xs, need_grad=False)          # lam = R(x) kept in the plan
    lam = plan.response(xs)
    xi_d = random_normal(lam.shape, lam.dtype, seed=seed, offset=0, device=lam.device)
    xi_x = random_normal(xs.shape, xs.dtype, seed=seed, offset=1, device=xs.device)
    z = plan.response_vjp(xi_d / torch.sqrt(lam)) + xi_x

    def mat(v):
        return plan.metric(None, v) + v

    return conjugate_gradient(mat, z, **cg_kwargs)
