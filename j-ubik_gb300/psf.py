"""eROSITA PSF patches on the GPU (``jubik/instruments/erosita/erosita_psf_utils.py``).

:func:`psf_interpolator` builds the per-patch PSFs of one module from the
gridded PSFs measured at a few off-axis radii (one ``psf_infos`` dict per
energy, as ``eROSITA_PSF._get_psf_infos`` makes them at
``erosita_psf.py:211-219``): the radius of each patch centre from the
pointing centre weights the gridded PSFs linearly, and each is sampled by
clamped bilinear interpolation at the pixel offsets rotated by the patch's
angle.  ``layout='full'`` returns the reference's (n^2, E, N, N) array;
``layout='precut'`` returns only the (2dx, 2dy) windows that the response
keeps (``jubik/convolve.py:107-111``), which ``ResponsePlan.set_psf`` takes
directly, without forming the full-field array.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from . import _lib
from .convolve import _is_domain
from .plan import as_device, dtype_code, ptr, require_cuda, stream_handle


def to_r_phi(cc):
    """(..., 2) offsets -> (..., 2) (radius, angle from the second axis)
    (``erosita_psf_utils.py:18-28``)."""
    cc = np.asarray(cc, np.float64)
    r = np.sqrt(cc[..., 0] ** 2 + cc[..., 1] ** 2)
    phi = np.angle(cc[..., 0] + 1.0j * cc[..., 1]) - np.pi / 2.0
    return np.stack((r, phi), axis=-1)


def to_ra_dec(rp):
    """Inverse of :func:`to_r_phi` (``erosita_psf_utils.py:31-37``)."""
    rp = np.asarray(rp, np.float64)
    return np.stack((rp[..., 0] * np.cos(rp[..., 1] + np.pi / 2.0),
                     rp[..., 0] * np.sin(rp[..., 1] + np.pi / 2.0)), axis=-1)


def get_interpolation_weights(rs, r):
    """Linear weights of radius r over the radii rs (``erosita_psf_utils.py:40-71``):
    the first PSF below rs[0], the last from rs[-1] on."""
    rs = np.asarray(rs, np.float64)
    w = np.zeros(rs.shape)
    if r <= rs[0]:
        w[0] += 1.0
    if r >= rs[-1]:
        w[-1] += 1.0
    for i in range(rs.size - 1):
        if rs[i] < r <= rs[i + 1]:
            t = (r - rs[i]) / (rs[i + 1] - rs[i])
            w[i] += 1.0 - t
            w[i + 1] += t
    return w


def _check_info(info):
    psfs = np.asarray(info["psfs"], np.float64)
    rs = np.asarray(info["rs"], np.float64).reshape(-1)
    cids = np.asarray(info["patch_center_ids"], np.float64)
    if psfs.shape[0] != rs.size or psfs.ndim != 3:
        raise ValueError("psfs must have shape rs.shape + psf.shape")
    if cids.shape != (rs.size, 2):
        raise ValueError("patch_center_ids must have shape rs.shape + (2,)")
    if np.any(cids > np.array(psfs.shape[1:])) or np.any(cids < 0):
        raise ValueError("a patch centre index lies outside its PSF grid")
    order = np.argsort(rs, kind="stable")
    return (psfs[order], rs[order], cids[order],
            np.asarray(list(info["patch_deltas"]), np.float64),
            np.asarray(list(info["pointing_center"]), np.float64))


def psf_interpolator(domain, npatch: int, psf_infos: Sequence[dict], layout: str = "full",
                     dtype: torch.dtype = torch.float64) -> torch.Tensor:
    """Per-patch PSFs of one module on the GPU.

    ``domain``: Domain whose last two axes are the field; ``psf_infos``: one
    dict per energy with 'psfs' (R, h, w), 'rs' (R,), 'patch_center_ids'
    (R, 2), 'patch_deltas' (2,), 'pointing_center' (2,).  Returns
    (n^2, E, N0, N1) for ``layout='full'`` or (n^2, E, 2 N0/n, 2 N1/n) for
    ``layout='precut'``."""
    if not _is_domain(domain):
        raise ValueError("domain has to be an instance of jubik.Domain")
    if layout not in ("full", "precut"):
        raise ValueError("layout must be 'full' or 'precut'")
    shp = tuple(int(s) for s in domain.shape[-2:])
    dist = tuple(float(d) for d in domain.distances[-2:])
    for ss in shp:
        if ss % npatch != 0 or ss % 2 != 0:
            raise ValueError("the field must be even and divisible by npatch")
    infos = [_check_info(i) for i in psf_infos]
    if len({(p.shape, r.size) for p, r, _, _, _ in infos}) != 1:
        raise ValueError("all energies need PSF grids of the same shape and count")
    dev = require_cuda()
    stack = lambda j: torch.as_tensor(np.stack([i[j] for i in infos]), device=dev).contiguous()
    psfs, rs, cids, deltas, pointing = (stack(j) for j in range(5))
    E, R, h, w = psfs.shape
    if layout == "full":
        out_shape = (npatch * npatch, E) + shp
    else:
        out_shape = (npatch * npatch, E, 2 * (shp[0] // npatch), 2 * (shp[1] // npatch))
    out = torch.empty(out_shape, dtype=dtype, device=dev)
    _lib.call("jubik_psf_interpolate", ptr(psfs), ptr(rs), ptr(cids), ptr(deltas), ptr(pointing),
              E, R, h, w, shp[0], shp[1], dist[0], dist[1], npatch,
              _lib.PSF_FULL if layout == "full" else _lib.PSF_PRECUT, dtype_code(dtype),
              ptr(out), stream_handle(dev))
    return out
