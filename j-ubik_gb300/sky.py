"""Diffuse sky from correlated fields, on the GPU (C ABI ``jubik_cf_*``).

J-UBIK's diffuse sky (``jubik/sky_models.py:205-225,306-341``) is the
exponential of a log-sky built from NIFTy.re correlated fields on a padded
grid: a spatial field plus, with a ``plaw`` prior, a spectral-index field
times the log energy-bin centres (``_apply_slope``, :593-602), cropped to the
data grid (``exp_padding``, :340-341).  Each field is

    field = offset + hartley(amp[pindex] * xi),   hartley(p) = Re fftn(p) + Im fftn(p),

with ``pindex`` the Fourier-mode length index of every pixel (NIFTy.re's
power distributor) and ``amp`` the amplitude spectrum over those lengths.
The field-sized work -- the distribution over modes, the Hartley transform on
the padded grid, the offsets, the energy combination and the crop, and the
vector-Jacobian product back to ``xi``, ``amp`` and the offsets -- runs in
``j-ubik_gb300/csrc/sky_cf.cu``.  The amplitude spectrum (a 1-D function of
the fluctuation parameters, NIFTy.re's non-parametric amplitude model) is an
input: the caller computes it, and differentiates it with the ``damp`` this
module returns.

:meth:`CorrelatedFieldSky.energy_and_grad` chains the log-sky into the
response's log-sky entry (the exp and the crop fused into its first kernel),
so one call gives the Poisson energy and its gradient with respect to the
excitations, amplitudes and offsets.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .plan import as_device, dtype_code, ptr, require_cuda, stream_handle

MAX_FIELDS = 4
MAX_ENERGIES = 32


def good_fft_size(n: int) -> int:
    """Smallest size >= n whose prime factors are 2, 3, 5, 7 and 11: the
    padded-grid size ``ducc0.fft.good_size`` gives (``sky_models.py:306-307``
    pads ``int(sdim * s_padding_ratio)`` to it)."""
    n = int(n)
    if n < 1:
        raise ValueError("size must be positive")
    m = n
    while True:
        r = m
        for p in (2, 3, 5, 7, 11):
            while r % p == 0:
                r //= p
        if r == 1:
            return m
        m += 1


def fourier_mode_distributor(shape, distances) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(pindex, unique mode lengths, multiplicity) of a regular grid, as
    NIFTy.re's ``get_fourier_mode_distributor``: the length of the Fourier
    mode of pixel (i0, i1, ...) is sqrt(sum_a (min(i_a, n_a - i_a) / (n_a d_a))^2);
    lengths that differ by at most 1e-12 times the largest length count as one
    (the last of such a run is kept), and every pixel is assigned to the
    nearest kept length by the midpoints between them."""
    shape = (int(shape),) if np.isscalar(shape) else tuple(int(s) for s in shape)
    dist = np.broadcast_to(np.asarray(distances, dtype=np.float64), (len(shape),))
    inv = 1.0 / (np.asarray(shape, dtype=np.float64) * dist)
    m = np.arange(shape[0], dtype=np.float64)
    m = np.minimum(m, shape[0] - m) * inv[0]
    if len(shape) > 1:
        m = m * m
        for a in range(1, len(shape)):
            t = np.arange(shape[a], dtype=np.float64)
            t = np.minimum(t, shape[a] - t) * inv[a]
            m = m[..., None] + t * t
        m = np.sqrt(m)
    um = np.unique(m)
    tol = 1e-12 * um[-1]
    um = um[np.diff(np.append(um, 2 * um[-1])) > tol]
    idx = np.searchsorted(0.5 * (um[:-1] + um[1:]), m)
    count = np.bincount(idx.ravel(), minlength=um.size)
    if np.any(count == 0) or count.shape != um.shape:
        raise RuntimeError("invalid harmonic mode(s) encountered")
    return idx.astype(np.int32), um, count


def log_rel_ebin_centers(e_min: Sequence[float], e_max: Sequence[float], e_ref: float) -> np.ndarray:
    """log of the energy-bin centres relative to e_ref: 0.5 log(e_max e_min) -
    log(e_ref) (``sky_models.py:455-466``)."""
    e_min = np.asarray(e_min, dtype=np.float64)
    e_max = np.asarray(e_max, dtype=np.float64)
    return 0.5 * np.log(e_max * e_min) - np.log(e_ref)


def diffuse_coefficients(e_min, e_max, e_ref, plaw: bool = True) -> np.ndarray:
    """Energy coefficients (E, n_fields) of the diffuse log-sky: the spatial
    field enters every bin with 1; the spectral-index field (``plaw``) with the
    bin's log relative centre, the outer product of ``_apply_slope``."""
    lr = log_rel_ebin_centers(e_min, e_max, e_ref)
    cols = [np.ones_like(lr)] + ([lr] if plaw else [])
    return np.stack(cols, axis=1)


class CorrelatedFieldSky:
    """``n_fields`` correlated fields on one padded grid and the log-sky they
    make.

    ``shape`` / ``distances``: the padded grid (``ext_s_shp`` of
    ``sky_models.py:306``) and its pixel distances.  ``crop``: the data grid
    (nx, ny) the log-sky keeps (the corner ``[:nx, :ny]``).  ``coefficients``:
    (E, n_fields) energy coefficients, e.g. :func:`diffuse_coefficients`;
    without them only the fields are available."""

    def __init__(self, shape, distances, n_fields: int = 1, crop=None, coefficients=None,
                 dtype: torch.dtype = torch.float32, device: Optional[torch.device] = None):
        shape = tuple(int(s) for s in shape)
        if len(shape) == 1:
            shape = (1,) + shape
        if len(shape) != 2:
            raise ValueError("correlated fields here are 1-D or 2-D")
        if not 1 <= n_fields <= MAX_FIELDS:
            raise ValueError(f"1 <= n_fields <= {MAX_FIELDS}")
        self.device = device or require_cuda()
        self.dtype = dtype
        self.shape = shape
        self.n_fields = int(n_fields)
        dist = np.broadcast_to(np.asarray(distances, dtype=np.float64), (2,))
        grid = shape if shape[0] > 1 else shape[1:]
        pidx, self.mode_lengths, self.mode_multiplicity = fourier_mode_distributor(
            grid, dist if shape[0] > 1 else dist[1:])
        self.pindex = np.ascontiguousarray(pidx.reshape(shape), dtype=np.int32)
        self.n_modes = int(self.mode_lengths.size)
        self.crop = tuple(int(c) for c in (crop if crop is not None else shape))
        if len(self.crop) != 2 or not (1 <= self.crop[0] <= shape[0] and 1 <= self.crop[1] <= shape[1]):
            raise ValueError("crop must be (nx, ny) within the padded grid")
        self.coefficients = None
        if coefficients is not None:
            c = np.ascontiguousarray(np.asarray(coefficients, dtype=np.float64))
            if c.ndim != 2 or c.shape[1] != self.n_fields or not 1 <= c.shape[0] <= MAX_ENERGIES:
                raise ValueError(f"coefficients must be (E <= {MAX_ENERGIES}, n_fields)")
            self.coefficients = c
        self._h = C.c_void_p()
        _lib.call("jubik_cf_create", self.n_fields, shape[0], shape[1],
                  self.pindex.ctypes.data_as(C.c_void_p), self.n_modes, dtype_code(dtype),
                  C.byref(self._h))

    @property
    def n_energies(self) -> int:
        return 0 if self.coefficients is None else int(self.coefficients.shape[0])

    def _s(self):
        return stream_handle(self.device)

    def _in(self, amp, xi, offsets=None):
        nf = self.n_fields
        a = as_device(amp, self.dtype, self.device).reshape(nf, self.n_modes)
        x = as_device(xi, self.dtype, self.device).reshape((nf,) + self.shape)
        o = None if offsets is None else as_device(offsets, self.dtype, self.device).reshape(nf)
        return a, x, o

    def _coef(self):
        if self.coefficients is None:
            raise ValueError("this sky has no energy coefficients")
        return self.coefficients.ctypes.data_as(C.c_void_p)

    def fields(self, amp, xi, offsets, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """(n_fields, s0, s1): offset_b + hartley(amp_b[pindex] * xi_b)."""
        a, x, o = self._in(amp, xi, offsets)
        if out is None:
            out = torch.empty((self.n_fields,) + self.shape, dtype=self.dtype, device=self.device)
        _lib.call("jubik_cf_apply", self._h, ptr(a), ptr(x), ptr(o), ptr(out), None, 0, 0, 0,
                  None, self._s())
        return out

    def logsky(self, amp, xi, offsets, out: Optional[torch.Tensor] = None,
               fields_out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """(E, nx, ny): sum_b coefficients[e, b] field_b[:nx, :ny]."""
        a, x, o = self._in(amp, xi, offsets)
        if out is None:
            out = torch.empty((self.n_energies,) + self.crop, dtype=self.dtype, device=self.device)
        _lib.call("jubik_cf_apply", self._h, ptr(a), ptr(x), ptr(o), ptr(fields_out),
                  self._coef(), self.n_energies, self.crop[0], self.crop[1], ptr(out), self._s())
        return out

    def vjp(self, amp, xi, g_fields=None, g_logsky=None):
        """(dxi, damp, doffsets) for the cotangent of the fields (n_fields, s0,
        s1) or of the log-sky (E, nx, ny)."""
        if (g_fields is None) == (g_logsky is None):
            raise ValueError("give exactly one of g_fields, g_logsky")
        a, x, _ = self._in(amp, xi)
        dxi = torch.empty_like(x)
        damp = torch.empty_like(a)
        doff = torch.empty(self.n_fields, dtype=self.dtype, device=self.device)
        if g_fields is not None:
            g = as_device(g_fields, self.dtype, self.device).reshape((self.n_fields,) + self.shape)
            _lib.call("jubik_cf_vjp", self._h, ptr(a), ptr(x), ptr(g), None, 0, 0, 0, None,
                      ptr(dxi), ptr(damp), ptr(doff), self._s())
        else:
            g = as_device(g_logsky, self.dtype, self.device).reshape(
                (self.n_energies,) + self.crop)
            _lib.call("jubik_cf_vjp", self._h, ptr(a), ptr(x), None, self._coef(),
                      self.n_energies, self.crop[0], self.crop[1], ptr(g), ptr(dxi), ptr(damp),
                      ptr(doff), self._s())
        return dxi, damp, doff

    def energy_and_grad(self, plan, amp, xi, offsets):
        """Poisson energy of the response ``plan`` at the sky exp(logsky) and
        its gradient with respect to (xi, amp, offsets)."""
        ls = self.logsky(amp, xi, offsets)
        energy, g = plan.energy_and_grad_logsky(ls)
        dxi, damp, doff = self.vjp(amp, xi, g_logsky=g)
        return energy, dxi, damp, doff

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().jubik_cf_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CorrelatedFieldLogSky(torch.autograd.Function):
    """logsky(amp, xi, offsets) of a :class:`CorrelatedFieldSky`, differentiable
    in all three inputs."""

    @staticmethod
    def forward(ctx, sky: CorrelatedFieldSky, amp, xi, offsets):
        ctx.sky = sky
        ctx.offsets_shape = offsets.shape
        ctx.save_for_backward(amp, xi)
        return sky.logsky(amp.detach(), xi.detach(), offsets.detach())

    @staticmethod
    def backward(ctx, g):
        amp, xi = ctx.saved_tensors
        dxi, damp, doff = ctx.sky.vjp(amp.detach(), xi.detach(), g_logsky=g.contiguous())
        return (None, damp.reshape(amp.shape), dxi.reshape(xi.shape),
                doff.reshape(ctx.offsets_shape))


def correlated_field_logsky(sky: CorrelatedFieldSky, amp, xi, offsets) -> torch.Tensor:
    return CorrelatedFieldLogSky.apply(sky, amp, xi, offsets)
