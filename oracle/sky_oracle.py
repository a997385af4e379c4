"""CPU oracle for the correlated-field log-sky (TEST INFRASTRUCTURE).

This module is the oracle (test infrastructure), never the product: only ``tests/`` may import it.
It restates in float64 numpy, independently of the product code:

* the padded grid size of ``jubik/sky_models.py:306-307``
  (``ducc0.fft.good_size``: the smallest size >= n with prime factors
  2, 3, 5, 7, 11), by trial division of every candidate;
* NIFTy.re's Fourier-mode power distributor (``get_fourier_mode_distributor``
  of ``nifty.re.correlated_field``, a dependency of J-UBIK, ``pyproject.toml``
  ``nifty >= 9.0.0``; not vendored, absent here): per-pixel mode lengths from
  explicit index loops, grouped over the sorted list with relative tolerance
  1e-12 of the largest length, each pixel assigned to the nearest kept length;
* the field ``offset + hartley(amp[pindex] * xi)`` with
  ``hartley(p) = fftn(p).real + fftn(p).imag`` (NIFTy.re's harmonic transform);
* the diffuse log-sky of ``sky_models.py:333-341``: spatial field plus the
  outer product of the log energy-bin centres (``:455-466``) with the
  spectral-index field (``_apply_slope``, ``:593-602``), cropped to the data
  grid;
* the vector-Jacobian products of all of the above, written out by hand.

Parity of the distributor and of the Hartley convention with NIFTy.re itself
is unpinned: neither NIFTy.re nor JAX is installed, and the reference's own
tests do not cover its sky models.
"""
from __future__ import annotations

import itertools

import numpy as np


def good_size(n):
    m = int(n)
    while True:
        r = m
        for p in (2, 3, 5, 7, 11):
            while r % p == 0:
                r //= p
        if r == 1:
            return m
        m += 1


def mode_distributor(shape, distances):
    shape = tuple(int(s) for s in np.atleast_1d(shape))
    dist = [float(d) for d in np.broadcast_to(np.asarray(distances, float), (len(shape),))]
    lengths = np.empty(shape)
    for idx in itertools.product(*[range(s) for s in shape]):
        acc = 0.0
        for i, s, d in zip(idx, shape, dist):
            k = min(i, s - i) / (s * d)
            acc += k * k
        lengths[idx] = np.sqrt(acc)
    flat = sorted(set(lengths.ravel().tolist()))
    tol = 1e-12 * flat[-1]
    kept = [v for v, nxt in zip(flat, flat[1:] + [2 * flat[-1]]) if nxt - v > tol]
    kept = np.array(kept)
    pindex = np.empty(shape, dtype=np.int64)
    for idx in itertools.product(*[range(s) for s in shape]):
        v = lengths[idx]
        j = 0
        while j + 1 < len(kept) and v > 0.5 * (kept[j] + kept[j + 1]):
            j += 1
        pindex[idx] = j
    counts = np.array([(pindex == j).sum() for j in range(len(kept))])
    return pindex, kept, counts


def hartley(p):
    f = np.fft.fftn(np.asarray(p, dtype=np.float64))
    return f.real + f.imag


def fields(amp, xi, offsets, pindex):
    amp = np.asarray(amp, float)
    xi = np.asarray(xi, float)
    return np.stack([offsets[b] + hartley(amp[b][pindex] * xi[b]) for b in range(xi.shape[0])])


def log_rel_ebin_centers(e_min, e_max, e_ref):
    return 0.5 * np.log(np.asarray(e_max, float) * np.asarray(e_min, float)) - np.log(e_ref)


def logsky(flds, coef, crop):
    nx, ny = crop
    out = np.zeros((coef.shape[0], nx, ny))
    for e in range(coef.shape[0]):
        for b in range(flds.shape[0]):
            out[e] += coef[e, b] * flds[b, :nx, :ny]
    return out


def logsky_cotangent_to_fields(g_logsky, coef, shape):
    nf = coef.shape[1]
    nx, ny = g_logsky.shape[1:]
    g = np.zeros((nf,) + tuple(shape))
    for b in range(nf):
        for e in range(coef.shape[0]):
            g[b, :nx, :ny] += coef[e, b] * g_logsky[e]
    return g


def fields_vjp(amp, xi, pindex, g_fields):
    amp = np.asarray(amp, float)
    xi = np.asarray(xi, float)
    nf, n_modes = amp.shape
    dxi = np.empty_like(xi)
    damp = np.zeros((nf, n_modes))
    doff = np.empty(nf)
    for b in range(nf):
        h = hartley(g_fields[b])  # the Hartley matrix is symmetric
        dxi[b] = amp[b][pindex] * h
        damp[b] = np.bincount(pindex.ravel(), weights=(xi[b] * h).ravel(), minlength=n_modes)
        doff[b] = g_fields[b].sum()
    return dxi, damp, doff
