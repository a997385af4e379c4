"""CPU oracle for the J-UBIK spatially-variant response (TEST INFRASTRUCTURE).

This module is the oracle (test infrastructure), never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it.
It restates, in float64 numpy / scipy.fft, the reference algorithm of

* ``jubik/convolve.py:18-184``  (``_bilinear_weights``, ``slice_patches``,
  ``linpatch_convolve``, ``convolve``, ``integrate``),
* ``jubik/response.py:12-112``  (``build_exposure_function``,
  ``build_readout_function``),
* ``jubik/utils.py:185-207``    (``coord_center``),
* ``jubik/instruments/erosita/erosita_response.py:209-212,349-350`` and
  ``jubik/instruments/chandra/chandra_response.py:127-142`` (composition
  ``R(x) = mask(exposure(psf(x * pixel_area)))``),
* the Poisson likelihood used at ``erosita_likelihood.py:89`` /
  ``chandra_likelihood.py:37``: NIFTy.re ``jft.Poissonian`` (third-party,
  ``nifty >= 9.0.0`` per ``pyproject.toml:14``, not vendored).  Its
  published energy is ``H(lam) = sum(lam) - sum(d * log(lam))``
  (stated at ``demos/x-ray-imaging.py:312-315``); gradient ``1 - d/lam``,
  Fisher metric ``t / lam``, left square-root metric ``t / sqrt(lam)``,
  normalised residual ``(d - lam)/sqrt(lam)``.  Parity of these Poisson
  values is unpinned: no reference test fixes them (the only test swaps in
  a fake, ``test/instruments/chandra/test_chandra_response_wrappers.py:80-88``).

Parity pins:
* outputs of the reference's own ``convolve.py`` / ``response.py`` /
  ``utils.py``, run unmodified through a numpy stand-in of the JAX calls they
  make (``tests/golden/make_ref_fixtures.py``, which first runs the reference's
  tests for those files through the stand-in): ``tests/test_ref_fixtures.py``
  checks this module against them (slicing, readout and patch centres
  bit-exact, ``linpatch_convolve`` and its VJP to 1e-13 / 1e-12);
* the known answers of the reference's own tests
  (``test/test_convolve.py``, ``test/test_slice_patches.py``,
  ``test/test_build_exposure_function.py``,
  ``test/test_build_exposure_readout_function.py``, ``test/test_utils.py:66-68``),
  re-asserted against this module in ``tests/test_oracle_pins.py``;
* an independent direct (non-FFT) C restatement in ``oracle/direct_linpatch.c``
  that cross-checks ``linpatch_convolve`` end to end.
"""
from __future__ import annotations

import os
from functools import reduce
from typing import NamedTuple

import numpy as np

try:  # scipy.fft is pocketfft, the same FFT family as JAX's CPU backend
    import scipy.fft as _sfft
except ImportError:  # pragma: no cover
    _sfft = None

_WORKERS = os.cpu_count() or 1


def _fftn(a, axes):
    if _sfft is not None:
        return _sfft.fftn(a, axes=axes, workers=_WORKERS)
    return np.fft.fftn(a, axes=axes)


def _ifftn(a, axes):
    if _sfft is not None:
        return _sfft.ifftn(a, axes=axes, workers=_WORKERS)
    return np.fft.ifftn(a, axes=axes)


class Domain(NamedTuple):
    """``jubik/data.py:19-29``."""

    shape: tuple
    distances: tuple


# ---------------------------------------------------------------- convolve.py
def bilinear_weights(shape):
    """``jubik/convolve.py:18-25``: outer(b, b), b = [linspace(0,1,h), flip]."""
    if shape[0] / 2 != int(shape[0] / 2):
        raise ValueError("this should happen")
    a = np.linspace(0, 1, int(shape[0] / 2), dtype="float64")
    b = np.concatenate([a, np.flip(a)])
    return np.outer(b, b)


def _slice_geometry(shape, n, dr):
    """Patch stride, window and clamped starts of ``convolve.py:43-63``.

    ``jax.lax.dynamic_slice`` clamps a start so the slice fits inside the
    padded operand; the clamp matters only for odd strides.
    """
    dx = int((shape[-2] - 2 * dr) / n)
    dy = int((shape[-1] - 2 * dr) / n)
    ph = shape[-2] + 2 * (dx // 2)
    pw = shape[-1] + 2 * (dy // 2)
    sh, sw = 2 * dx + 2 * dr, 2 * dy + 2 * dr
    if sh > ph or sw > pw or sh <= 0 or sw <= 0:
        raise ValueError("patch window does not fit the padded field")
    k = np.arange(n * n)
    r0 = np.minimum((k % n) * dx, ph - sh)
    c0 = np.minimum((k // n) * dy, pw - sw)
    return dx, dy, ph, pw, sh, sw, r0, c0


def slice_patches(x, shape, n_patches_per_axis, additional_margin):
    """``jubik/convolve.py:28-63``: pad by stride//2, gather n^2 windows.

    Patch k starts at padded row ``(k % n) * dx`` and column ``(k // n) * dy``
    (meshgrid with ``indexing="xy"`` flattened in C order).
    """
    x = np.asarray(x)
    dx, dy, ph, pw, sh, sw, r0, c0 = _slice_geometry(
        shape, n_patches_per_axis, additional_margin)
    pad = [(0, 0)] * (x.ndim - 2) + [(dx // 2, dx // 2), (dy // 2, dy // 2)]
    padded = np.pad(x, pad)
    out = np.empty((n_patches_per_axis ** 2,) + x.shape[:-2] + (sh, sw),
                   dtype=x.dtype)
    for k in range(n_patches_per_axis ** 2):
        out[k] = padded[..., r0[k]:r0[k] + sh, c0[k]:c0[k] + sw]
    return out


def slice_patches_adjoint(patches, shape, n_patches_per_axis,
                          additional_margin):
    """Transpose of :func:`slice_patches` (``jax.linear_transpose`` at
    ``convolve.py:138-143``): scatter-add every window, then drop the pad."""
    patches = np.asarray(patches)
    dx, dy, ph, pw, sh, sw, r0, c0 = _slice_geometry(
        shape, n_patches_per_axis, additional_margin)
    lead = patches.shape[1:-2]
    acc = np.zeros(lead + (ph, pw), dtype=patches.dtype)
    for k in range(n_patches_per_axis ** 2):
        acc[..., r0[k]:r0[k] + sh, c0[k]:c0[k] + sw] += patches[k]
    return acc[..., dx // 2:dx // 2 + shape[-2], dy // 2:dy // 2 + shape[-1]]


def cut_kernel(kernel, shape, n_patches_per_axis):
    """``convolve.py:104-111``: fftshift, then keep the central (2dx, 2dy)."""
    dx = int(shape[-2] / n_patches_per_axis)
    dy = int(shape[-1] / n_patches_per_axis)
    kcx = (shape[-2] - 2 * dx) // 2
    kcy = (shape[-1] - 2 * dy) // 2
    rolled = np.fft.fftshift(kernel, axes=(-2, -1))
    cut = rolled[..., kcx:-kcx, kcy:-kcy]
    if cut.shape[-2:] != (2 * dx, 2 * dy):
        raise ValueError("kernel cut does not give a (2dx, 2dy) window")
    return cut


def prepare_kernel(kernel, domain, n_patches_per_axis, margin,
                   precut=False):
    """``convolve.py:104-131``: cut, pad by the margin, ifftshift, and divide
    by ``sum * dvol`` per (patch, energy)."""
    shape = domain.shape
    cut = kernel if precut else cut_kernel(kernel, shape, n_patches_per_axis)
    pad = [(0, 0)] * (cut.ndim - 2) + [(margin, margin)] * 2
    pk = np.pad(cut, pad)
    rb = np.fft.ifftshift(pk, axes=(-2, -1))
    summed = rb.sum((-2, -1))
    dvol = domain.distances[-2] * domain.distances[-1]
    norm = (summed * np.array(dvol))[..., None, None]
    return rb * norm ** -1


def convolve(x, y, domain, axes, verbose=True):
    """``jubik/convolve.py:148-176``: ``dvol * ifftn(fftn(x) fftn(y)).real``.

    ``x`` is the kernel, ``y`` the signal; a kernel with fewer dims is
    broadcast over the signal's extra leading axis (with the reference's
    message)."""
    dlist = [domain.distances[i] for i in axes]
    dvol = float(reduce(lambda a, b: a * b, dlist))
    hx = _fftn(np.asarray(x, dtype=np.float64), axes)
    hy = _fftn(np.asarray(y, dtype=np.float64), axes)
    if len(np.shape(y)) > len(np.shape(x)):
        if verbose:
            print("kernel_shape:", np.shape(x))
            print("signal_shape:", np.shape(y))
            print("Dimension Inconsistency. Broadcasting PSFs")
        prod = hx[..., np.newaxis, :, :] * hy
    else:
        prod = hx * hy
    res = _ifftn(prod, axes)
    return (dvol * res).real


def integrate(x, domain, axes):
    """``jubik/convolve.py:179-184``."""
    s = np.sum(x, axis=tuple(axes))
    dlist = [domain.distances[i] for i in axes]
    return float(reduce(lambda a, b: a * b, dlist)) * s


def linpatch_convolve(x, domain, kernel, n_patches_per_axis, margin,
                      precut=False):
    """``jubik/convolve.py:66-145`` (float64).

    ``precut=True`` accepts kernels already cut to the (2dx, 2dy) window
    (the result of ``convolve.py:107-111``), which is what the GB300 path
    stores; the two forms agree exactly (tested)."""
    if not isinstance(domain, (Domain,)) and not (
            hasattr(domain, "shape") and hasattr(domain, "distances")):
        raise ValueError("domain has to be an instance of jubik.Domain")
    shape = domain.shape
    x = np.asarray(x, dtype=np.float64)
    slices = slice_patches(x, shape, n_patches_per_axis, 0)
    weights = bilinear_weights(slices.shape[-2:])
    weighted = weights * slices
    pad = [(0, 0)] * (weighted.ndim - 2) + [(margin, margin)] * 2
    padded = np.pad(weighted, pad)
    nk = prepare_kernel(np.asarray(kernel, dtype=np.float64), domain,
                        n_patches_per_axis, margin, precut=precut)
    ndom = Domain((1, *shape), (None, *domain.distances))
    conv = convolve(nk, padded, ndom, axes=(-2, -1), verbose=False)
    padded_shape = list(shape[:-2]) + [s + 2 * margin for s in shape[-2:]]
    pr = slice_patches_adjoint(conv, padded_shape, n_patches_per_axis, margin)
    return pr[..., margin:-margin, margin:-margin]


def linpatch_convolve_adjoint(g, domain, kernel, n_patches_per_axis, margin,
                              precut=False):
    """Transpose of :func:`linpatch_convolve` in ``x`` (what ``jax.vjp`` of
    ``convolve.py:66-145`` computes): correlation with the normalised kernel
    (``conj`` of its spectrum), crop the margin, weight, transpose-slice."""
    shape = domain.shape
    g = np.asarray(g, dtype=np.float64)
    padded_shape = list(shape[:-2]) + [s + 2 * margin for s in shape[-2:]]
    gp = np.pad(g, [(0, 0)] * (g.ndim - 2) + [(margin, margin)] * 2)
    win = slice_patches(gp, padded_shape, n_patches_per_axis, margin)
    nk = prepare_kernel(np.asarray(kernel, dtype=np.float64), domain,
                        n_patches_per_axis, margin, precut=precut)
    dvol = domain.distances[-2] * domain.distances[-1]
    hk = np.conj(_fftn(nk, (-2, -1)))
    hw = _fftn(win, (-2, -1))
    if nk.ndim < win.ndim:
        hk = hk[..., np.newaxis, :, :]
    corr = (dvol * _ifftn(hk * hw, (-2, -1))).real
    crop = corr[..., margin:corr.shape[-2] - margin,
                margin:corr.shape[-1] - margin]
    weighted = bilinear_weights(crop.shape[-2:]) * crop
    return slice_patches_adjoint(weighted, shape, n_patches_per_axis, 0)


# ---------------------------------------------------------------- response.py
def build_exposure_function(exposures, exposure_cut=None):
    """``jubik/response.py:12-45`` (threshold applied in place)."""
    if exposure_cut is not None:
        if exposure_cut < 0:
            raise ValueError("exposure_cut should be non-negative or None!")
        exposures[exposures < exposure_cut] = 0

    def exposure(x):
        return exposures * x
    return exposure


def build_readout_function(flags, threshold=None, keys=None):
    """``jubik/response.py:48-112``: returns a dict key -> x[i][~mask[i]]."""
    if threshold is not None and threshold < 0:
        raise ValueError("threshold should be positive!")
    if threshold is not None:
        flags[flags < threshold] = 0
    mask = flags == 0
    if keys is None:
        keys = ['masked input']
    elif len(keys) != flags.shape[0]:
        raise ValueError(
            "length of keys should match the number of flag maps.")

    def _apply_readout(x):
        if len(mask.shape) != 4:
            raise ValueError("flags should have shape (n, m, q, l)!")
        if len(x.shape) != 4:
            raise ValueError("input should have shape (n, m, q, l)!")
        return {key: np.asarray(x[i])[~mask[i]] for i, key in enumerate(keys)}
    return _apply_readout


def readout_adjoint(vec, mask_flags_zero, keys):
    """Transpose of the readout (``jax.linear_transpose`` at
    ``jubik/data.py:156-159``): scatter each module's vector back."""
    mask = mask_flags_zero
    out = np.zeros(mask.shape, dtype=np.float64)
    for i, key in enumerate(keys):
        out[i][~mask[i]] = vec[key]
    return out


# ---------------------------------------------------------------- utils.py
def coord_center(side_length, side_n):
    """``jubik/utils.py:185-207``."""
    tdx = tdy = side_length // side_n
    xc = np.arange(tdx // 2, tdx * side_n, tdx)
    yc = np.arange(tdy // 2, tdy * side_n, tdy)
    co = np.array(np.meshgrid(xc, yc)).reshape(2, -1)
    return np.ravel_multi_index(co, [side_length, side_length])


# ---------------------------------------------------------------- Poisson
def poisson_energy(lam, data):
    """NIFTy.re ``Poissonian`` energy: ``sum(lam) - vdot(data, log(lam))``."""
    lam = np.asarray(lam, dtype=np.float64)
    return float(np.sum(lam) - np.vdot(np.asarray(data, np.float64),
                                       np.log(lam)))


def poisson_grad(lam, data):
    """dH/dlam = 1 - d/lam."""
    lam = np.asarray(lam, dtype=np.float64)
    return 1.0 - np.asarray(data, np.float64) / lam


def poisson_metric(lam, t):
    """Fisher metric of the Poisson likelihood: t / lam."""
    return np.asarray(t, np.float64) / np.asarray(lam, np.float64)


def poisson_left_sqrt_metric(lam, t):
    return np.asarray(t, np.float64) / np.sqrt(np.asarray(lam, np.float64))


def poisson_normalized_residual(lam, data):
    lam = np.asarray(lam, np.float64)
    return (np.asarray(data, np.float64) - lam) / np.sqrt(lam)


# ---------------------------------------------------------------- response
class Response:
    """Full instrument response of ``erosita_response.py:349-350``:
    ``R(x) = mask(exposure(psf(x * pixel_area)))`` where ``psf`` is
    ``linpatch_convolve`` vmapped over the module axis of ``kernel``
    (``erosita_response.py:209-212``).  Kernels are pre-cut (M, n^2, E, K, K)
    or full (M, n^2, E, N, N); exposures (M, E, N, N); ``readmask`` True
    where a pixel is read out (``~mask`` of ``response.py:87,110``)."""

    def __init__(self, domain, kernel, n_patches_per_axis, margin,
                 exposures, readmask, pixel_area=1.0, precut=True):
        self.domain = domain
        self.kernel = np.asarray(kernel, np.float64)
        self.n = n_patches_per_axis
        self.margin = margin
        self.exposures = np.asarray(exposures, np.float64)
        self.readmask = np.asarray(readmask, bool)
        self.pixel_area = float(pixel_area)
        self.precut = precut

    @property
    def n_modules(self):
        return self.kernel.shape[0]

    def psf(self, x):
        return np.stack([linpatch_convolve(x, self.domain, self.kernel[i],
                                           self.n, self.margin, self.precut)
                         for i in range(self.n_modules)])

    def psf_adjoint(self, g):
        return sum(linpatch_convolve_adjoint(g[i], self.domain,
                                             self.kernel[i], self.n,
                                             self.margin, self.precut)
                   for i in range(self.n_modules))

    def readout(self, img):
        return [img[i][self.readmask[i]] for i in range(self.n_modules)]

    def readout_adjoint(self, vecs):
        out = np.zeros(self.readmask.shape, np.float64)
        for i in range(self.n_modules):
            out[i][self.readmask[i]] = vecs[i]
        return out

    def __call__(self, x):
        conv = self.psf(np.asarray(x, np.float64) * self.pixel_area)
        return self.readout(self.exposures * conv)

    def image(self, x):
        """exposure * psf(x * pixel_area) before the readout (M, E, N, N)."""
        return self.exposures * self.psf(np.asarray(x, np.float64)
                                         * self.pixel_area)

    def adjoint(self, vecs):
        g = self.exposures * self.readout_adjoint(vecs)
        return self.pixel_area * self.psf_adjoint(g)

    def energy_and_grad(self, x, data):
        lam = self(x)
        e = sum(poisson_energy(l, d) for l, d in zip(lam, data))
        g = self.adjoint([poisson_grad(l, d) for l, d in zip(lam, data)])
        return e, g

    def metric(self, x, v):
        lam = self(x)
        rv = self(v)
        return self.adjoint([poisson_metric(l, t) for l, t in zip(lam, rv)])


# ---------------------------------------------------------------- C restatement
def linpatch_direct_c(x, kernel_precut, n_patches_per_axis, margin):
    """Direct (non-FFT) C restatement of ``linpatch_convolve`` (oracle/direct_linpatch.c),
    built by ``make -C oracle``.  x: (E, nx, ny); kernel (n^2, E, 2dx, 2dx)."""
    import ctypes

    here = os.path.dirname(os.path.abspath(__file__))
    lib = ctypes.CDLL(os.path.join(here, "_build", "libjubik_oracle_c.so"))
    x = np.ascontiguousarray(x, dtype=np.float64)
    k = np.ascontiguousarray(kernel_precut, dtype=np.float64)
    E, nx, ny = x.shape
    out = np.empty_like(x)
    dp = ctypes.POINTER(ctypes.c_double)
    st = lib.oracle_linpatch_direct(x.ctypes.data_as(dp), E, nx, ny, int(n_patches_per_axis),
                                    int(margin), k.ctypes.data_as(dp), out.ctypes.data_as(dp))
    if st != 0:
        raise ValueError("invalid geometry")
    return out
