"""CPU oracle for the eROSITA PSF-patch interpolation (TEST INFRASTRUCTURE).

This module is the oracle (test infrastructure), never the product: only ``tests/`` may import it.
It restates in float64 numpy the behaviour of
``jubik/instruments/erosita/erosita_psf_utils.py``:

* ``to_r_phi`` / ``to_ra_dec`` (:18-37): polar coordinates with the angle
  measured from the second axis (``angle(x + i y) - pi/2``);
* ``get_interpolation_weights`` (:40-71): linear weights over the sorted PSF
  radii; the first PSF below ``rs[0]``, the last one from ``rs[-1]`` on (at
  exactly ``r == rs[-1]`` both the last interval and the clamp contribute, so
  the last PSF gets weight 2 there, as in the reference);
* ``get_psf`` (:90-172): the PSF at a patch centre is the radius-weighted sum
  of the gridded PSFs, each sampled by bilinear interpolation with clamped
  ("nearest") indices -- ``jax.scipy.ndimage.map_coordinates(order=1,
  mode='nearest')`` -- at the pixel offsets rotated by the patch's angle about
  the pointing centre;
* ``psf_interpolator`` (:198-264): patch centres, the (dec, -ra) pixel offset
  grid, the patch order (dec along k % n, ra reversed along k // n), the roll
  by half the field, output (n^2, E, N, N).

The reference module has no tests; parity rests on this restatement.
"""
from __future__ import annotations

import numpy as np


def to_r_phi(cc):
    cc = np.asarray(cc, np.float64)
    r = np.sqrt(cc[..., 0] ** 2 + cc[..., 1] ** 2)
    phi = np.angle(cc[..., 0] + 1j * cc[..., 1]) - np.pi / 2.0
    return np.stack((r, phi), axis=-1)


def to_ra_dec(rp):
    rp = np.asarray(rp, np.float64)
    x = rp[..., 0] * np.cos(rp[..., 1] + np.pi / 2.0)
    y = rp[..., 0] * np.sin(rp[..., 1] + np.pi / 2.0)
    return np.stack((x, y), axis=-1)


def interpolation_weights(rs, r):
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


def bilinear_nearest(img, q0, q1):
    """Order-1 interpolation of img at (q0, q1) with indices clamped to the grid."""
    h, w = img.shape
    f0, f1 = np.floor(q0), np.floor(q1)
    t0, t1 = q0 - f0, q1 - f1
    i0 = f0.astype(np.int64)
    i1 = f1.astype(np.int64)
    a0, b0 = np.clip(i0, 0, h - 1), np.clip(i0 + 1, 0, h - 1)
    a1, b1 = np.clip(i1, 0, w - 1), np.clip(i1 + 1, 0, w - 1)
    return ((1 - t0) * (1 - t1) * img[a0, a1] + (1 - t0) * t1 * img[a0, b1]
            + t0 * (1 - t1) * img[b0, a1] + t0 * t1 * img[b0, b1])


def psf_at(info, ra, dec, dra, ddec):
    """``get_psf(...)(ra, dec, dra, ddec)`` for one patch centre (scalars)."""
    order = np.argsort(np.asarray(info["rs"], np.float64))
    rs = np.asarray(info["rs"], np.float64)[order]
    psfs = np.asarray(info["psfs"], np.float64)[order]
    cids = np.asarray(info["patch_center_ids"], np.float64)[order]
    deltas = np.asarray(info["patch_deltas"], np.float64)
    pc = np.asarray(info["pointing_center"], np.float64)
    rp = to_r_phi(np.array([ra, dec]) - pc)
    w = interpolation_weights(rs, rp[0])
    ic = to_r_phi(np.stack((dra, ddec), axis=-1))
    ic[..., 1] = ic[..., 1] - rp[1]
    ic = to_ra_dec(ic)
    res = np.zeros(np.shape(dra))
    for cid, pp, ww in zip(cids, psfs, w):
        q0 = (ic[..., 0] + cid[0] * deltas[0]) / deltas[0]
        q1 = (ic[..., 1] + cid[1] * deltas[1]) / deltas[1]
        res += ww * bilinear_nearest(pp, q0, q1)
    return res


def patch_centres(shape, distances, npatch):
    """(c_ra, c_dec) of the n^2 patches in the reference's order."""
    ps = [s // npatch for s in shape]
    c0 = np.array([(i * ps[0] + ps[0] / 2) * distances[0] for i in range(npatch)])
    c1 = np.array([(i * ps[1] + ps[1] / 2) * distances[1] for i in range(npatch)])
    g0, g1 = np.meshgrid(c0, c1, indexing="xy")
    return np.flip(g1.flatten()), g0.flatten()


def psf_interpolator(shape, distances, npatch, psf_infos):
    """(n^2, E, N, N) interpolated, rolled PSFs (``erosita_psf_utils.py:198-264``)."""
    shape = tuple(int(s) for s in shape[-2:])
    distances = tuple(float(d) for d in distances[-2:])
    for s in shape:
        if s % npatch != 0 or s % 2 != 0:
            raise ValueError("field shape must be even and divisible by npatch")
    cp = [(np.arange(s) - s / 2) * d for s, d in zip(shape, distances)]
    g = np.meshgrid(*cp, indexing="ij")
    d_dec, d_ra = g[0], -1.0 * g[1]
    c_ra, c_dec = patch_centres(shape, distances, npatch)
    out = []
    for info in psf_infos:
        pats = [np.roll(np.roll(psf_at(info, ra, dec, d_ra, d_dec), -shape[0] // 2, axis=0),
                        -shape[1] // 2, axis=1) for ra, dec in zip(c_ra, c_dec)]
        out.append(np.array(pats))
    return np.moveaxis(np.stack(out), 0, -3)


def precut_windows(full, npatch):
    """The (2dx, 2dy) windows ``convolve.py:107-111`` cuts from full-field
    kernels (n^2, E, N0, N1): window pixel a is full pixel (a - dx) mod N0."""
    N0, N1 = full.shape[-2:]
    dx, dy = N0 // npatch, N1 // npatch
    a = (np.arange(2 * dx) - dx) % N0
    b = (np.arange(2 * dy) - dy) % N1
    return full[..., a[:, None], b[None, :]]
