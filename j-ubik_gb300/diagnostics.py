"""Mock data and noise-weighted residuals on the GPU.

* :func:`generate_mock_data` -- the data step of ``jubik/data.py:138-159``:
  expected counts R(sky) of every module, one Poisson draw each, as integer
  counts in a readout Vector (the sky itself comes from the caller's model);
* :func:`calculate_nwr` -- ``jubik/diagnostics.py:62-124``: the residuals
  ``(R(op(x)) - d) / sqrt(R(op(x)))`` of every sample, back-projected by the
  readout transpose, with the minimum-count and zero-exposure masks.
"""
from __future__ import annotations

from typing import Optional, Sequence

import torch

from .response import Vector
from .sampling import random_poisson


def _leaves(v, keys):
    if isinstance(v, Vector):
        return [v.tree[k] for k in keys]
    if isinstance(v, dict):
        return [v[k] for k in keys]
    return list(v)


def generate_mock_data(response_dict: dict, sky, seed: int = 0, kernel=None) -> Vector:
    """Poisson mock data of ``response_dict['R'](sky[, kernel])`` per module
    (``jubik/data.py:138-146``), one independent stream per module."""
    R = response_dict["R"]
    lam = R(sky) if kernel is None else R(sky, kernel)
    out = {}
    for i, (key, val) in enumerate(lam.tree.items()):
        out[key] = random_poisson(val.detach(), seed=seed, offset=i).to(torch.int64)
    return Vector(out)


def calculate_nwr(pos: Sequence, op, data, response_dict: dict, abs: bool = False,
                  min_counts: Optional[int] = None, exposure_mask: bool = True,
                  response: bool = True):
    """Noise-weighted residuals ``(R(op(x)) - d) / sqrt(R(op(x)))`` for every
    sample x in ``pos``, back-projected by ``response_dict['mask_adj']``.

    Returns ``(res, mask)``: res (M, S, E, N, N); mask (M, S, E, N, N) bool,
    True where a pixel is excluded (data below ``min_counts``, or zero
    exposure when ``exposure_mask``), or None when neither applies --
    the outputs of ``jubik/diagnostics.py:62-124``."""
    R = response_dict["R"] if response else (lambda x: x)
    adj = response_dict["mask_adj"]
    keys = list(response_dict["R"].keys) if hasattr(response_dict["R"], "keys") else None
    per_sample = []
    for x in pos:
        lam = R(op(x))
        lam_l = _leaves(lam, keys)
        d_l = _leaves(data, keys)
        res = []
        for l_, d_ in zip(lam_l, d_l):
            l_ = l_.detach().to(torch.float64)
            d_t = torch.as_tensor(d_, device=l_.device).to(torch.float64)
            r = (l_ - d_t) / torch.sqrt(l_)
            res.append(r.abs() if abs else r)
        per_sample.append(adj(Vector(dict(zip(keys, res))))[0])
    res = torch.stack(per_sample, dim=1)
    S = res.shape[1]

    mask = None
    if min_counts is not None:
        dl = [(torch.as_tensor(d_).to(res.device) < min_counts).to(torch.float64)
              for d_ in _leaves(data, keys)]
        mask = adj(Vector(dict(zip(keys, dl))))[0] > 0
    if exposure_mask:
        exp = response_dict["exposure"]
        if exp is None:
            raise ValueError("exposure_mask needs the response's exposure")
        em = exp(torch.ones(res.shape[:1] + res.shape[2:], dtype=torch.float64,
                            device=res.device)) == 0.0
        mask = em if mask is None else torch.logical_or(mask, em)
    if mask is not None:
        mask = mask.unsqueeze(1).expand(-1, S, *mask.shape[1:])
    return res, mask
