"""CPU oracle for the callers around the response (TEST INFRASTRUCTURE).

This module is the oracle (test infrastructure), never the product: only ``tests/`` may import it.
It restates in numpy:

* the Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
  "Parallel random numbers: as easy as 1, 2, 3", SC'11), pinned by the
  published known-answer vectors of that paper's Random123 distribution (the
  three vectors asserted in ``tests/test_callers.py``);
* the counter layout, Box-Muller transform and Poisson draws (inversion below
  10, Hormann's PTRS above) that the GPU sampler documents, element by
  element, so that the GPU draws can be compared draw for draw;
* the mock-data step of ``jubik/data.py:138-159`` (expected counts of each
  module -> Poisson draw -> int; transpose of the readout for plotting);
* the noise-weighted residuals of ``jubik/diagnostics.py:62-124``:
  ``(R(x) - d) / sqrt(R(x))`` per sample, back-projected by the readout
  transpose, with the minimum-count and zero-exposure masks;
* a conjugate-gradient solve of a symmetric positive definite system with
  the stopping rules that ``jubik/minimization_parser.py:337-420`` configures
  (absdelta, tol, atol, miniter, maxiter) for NIFTy.re's
  ``conjugate_gradient`` (third-party, ``nifty >= 9.0.0``, not vendored;
  its exact stopping semantics are restated here from the names, so CG
  iteration counts are parity unpinned -- the solution is pinned by a
  direct dense solve).
"""
from __future__ import annotations

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
MASK32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """ctr: (..., 4) uint32-valued; key: (2,) -> (..., 4) uint32 (numpy uint64 math)."""
    c = [np.asarray(ctr, np.uint64)[..., i] & MASK32 for i in range(4)]
    k0 = np.uint64(int(key[0]) & 0xFFFFFFFF)
    k1 = np.uint64(int(key[1]) & 0xFFFFFFFF)
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
        k0 = (k0 + W0) & MASK32
        k1 = (k1 + W1) & MASK32
    return np.stack(c, axis=-1).astype(np.uint32)


def _u01f(x):
    return ((x >> np.uint32(9)).astype(np.float64) + 0.5) * (1.0 / 8388608.0)


def _u01d(hi, lo):
    m = ((hi.astype(np.uint64) >> np.uint64(5)) << np.uint64(26)) | (lo.astype(np.uint64)
                                                                      >> np.uint64(6))
    return (m.astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def _key(seed):
    return (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)


def random_normal(n, dtype, seed, offset=0):
    """Element-by-element restatement of the GPU normal draws (float64 math)."""
    per = 4 if dtype == np.float32 else 2
    g = np.arange((n + per - 1) // per, dtype=np.uint64)
    ctr = np.stack([g & MASK32, g >> np.uint64(32),
                    np.full_like(g, offset & 0xFFFFFFFF), np.full_like(g, offset >> 32)], -1)
    r = philox4x32_10(ctr, _key(seed))
    if per == 4:
        u = [_u01f(r[:, i]) for i in range(4)]
        z = []
        for a, b in ((u[0], u[1]), (u[2], u[3])):
            rad = np.sqrt(-2.0 * np.log(a))
            z += [rad * np.cos(2 * np.pi * b), rad * np.sin(2 * np.pi * b)]
        out = np.stack(z, -1).reshape(-1)
    else:
        a, b = _u01d(r[:, 0], r[:, 1]), _u01d(r[:, 2], r[:, 3])
        rad = np.sqrt(-2.0 * np.log(a))
        out = np.stack([rad * np.cos(2 * np.pi * b), rad * np.sin(2 * np.pi * b)], -1).reshape(-1)
    return out[:n]


def _poisson_one(lam, i, off, key):
    from math import exp, floor, lgamma, log, sqrt
    if not lam >= 0.0 or lam >= 2.0e9:
        return -1
    if lam == 0.0:
        return 0

    def draw(att):
        c = np.array([[i & 0xFFFFFFFF, i >> 32, off, att]], np.uint64)
        return philox4x32_10(c, key)[0]

    if lam < 10.0:
        r = draw(0)
        u = float(_u01d(r[0:1], r[1:2])[0])
        p = exp(-lam)
        F, k = p, 0
        while u > F and k < 1000:
            k += 1
            p *= lam / k
            F += p
            if p == 0.0:
                break
        return k
    slam, loglam = sqrt(lam), log(lam)
    b = 0.931 + 2.53 * slam
    a = -0.059 + 0.02483 * b
    inv_alpha = 1.1239 + 1.1328 / (b - 3.4)
    vr = 0.9277 - 3.6224 / (b - 2.0)
    for att in range(256):
        r = draw(att + 1)
        U = float(_u01d(r[0:1], r[1:2])[0]) - 0.5
        V = float(_u01d(r[2:3], r[3:4])[0])
        us = 0.5 - abs(U)
        kd = floor((2.0 * a / us + b) * U + lam + 0.43)
        if us >= 0.07 and V <= vr:
            return int(kd)
        if kd < 0 or (us < 0.013 and V > us):
            continue
        if log(V) + log(inv_alpha) - log(a / (us * us) + b) <= -lam + kd * loglam - lgamma(kd + 1):
            return int(kd)
    return int(floor(lam + 0.5))


def random_poisson(lam, seed, offset=0):
    """Element-by-element restatement of the GPU Poisson draws (slow: tests only)."""
    lam = np.asarray(lam, np.float64).reshape(-1)
    key = _key(seed)
    return np.array([_poisson_one(float(l), i, offset, key) for i, l in enumerate(lam)],
                    np.int64)


def mock_data(lam_per_module, draw):
    """``jubik/data.py:143-146``: a Poisson draw of each module's expected
    counts, as int (``draw(lam, module_index)`` supplies the draws)."""
    return [np.asarray(draw(l, i)).astype(int) for i, l in enumerate(lam_per_module)]


def calculate_nwr(lam_samples, data, readmask, exposure_images=None, abs_=False,
                  min_counts=None, exposure_mask=True):
    """``jubik/diagnostics.py:62-124`` for one module list.

    lam_samples: list over samples of per-module readout vectors R(op(x));
    data: per-module readout vectors; readmask (M, E, N, N) bool (True = read
    out).  Returns (res (M, S, E, N, N), mask) where the residuals are
    ``(lam - d) / sqrt(lam)`` back-projected by the readout transpose
    (zeros at masked pixels) and the mask is True where a pixel is excluded:
    data below ``min_counts`` (back-projected) or exposure == 0."""
    M = readmask.shape[0]
    S = len(lam_samples)
    res = np.zeros((M, S) + readmask.shape[1:])
    for s, lam in enumerate(lam_samples):
        for m in range(M):
            v = (lam[m] - np.asarray(data[m], np.float64)) / np.sqrt(lam[m])
            res[m, s][readmask[m]] = np.abs(v) if abs_ else v
    mask = None
    if min_counts is not None:
        mc = np.zeros(readmask.shape)
        for m in range(M):
            mc[m][readmask[m]] = (np.asarray(data[m]) < min_counts).astype(float)
        mask = mc.astype(bool)
    if exposure_mask:
        em = np.asarray(exposure_images) == 0.0
        mask = em if mask is None else np.logical_or(mask, em)
    return res, mask


def conjugate_gradient(mat, j, x0=None, absdelta=None, tol=1e-5, atol=0.0, miniter=None,
                       maxiter=None):
    """Conjugate gradients for ``mat(x) = j`` (float64), minimising
    ``E(x) = 0.5 <x, mat x> - <j, x>``.  Stops after at least ``miniter``
    iterations when the energy decrease of an iteration is below ``absdelta``
    or the residual norm is at most ``max(tol |j|, atol)``; at most
    ``maxiter`` iterations.  Returns (x, iterations)."""
    j = np.asarray(j, np.float64)
    x = np.zeros_like(j) if x0 is None else np.array(x0, np.float64)
    r = j - mat(x) if x0 is not None else j.copy()
    d = r.copy()
    gamma = float(np.vdot(r, r))
    energy = -0.5 * float(np.vdot(x, r + j))
    miniter = miniter or 0
    maxiter = maxiter if maxiter is not None else 10 * j.size
    bound = max(tol * float(np.linalg.norm(j)), atol)
    it = 0
    while it < maxiter:
        if np.sqrt(gamma) <= bound and it >= miniter:
            break
        q = mat(d)
        curv = float(np.vdot(d, q))
        if curv <= 0:
            raise ValueError("matrix not positive definite")
        alpha = gamma / curv
        x = x + alpha * d
        r = r - alpha * q
        new_gamma = float(np.vdot(r, r))
        new_energy = -0.5 * float(np.vdot(x, r + j))
        it += 1
        delta = energy - new_energy
        energy = new_energy
        if absdelta is not None and it >= miniter and delta < absdelta:
            break
        d = r + (new_gamma / gamma) * d
        gamma = new_gamma
    return x, it
