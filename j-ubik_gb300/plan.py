"""Host-side plan object over the C ABI (``jubik_plan_*``).

A :class:`ResponsePlan` holds, on one GPU, everything the response needs
between calls: the normalised PSF spectra (computed once, where the
reference recomputes the kernel preparation of ``jubik/convolve.py:104-131``
on every call), the exposure, the readout index map and the Poisson counts.
All arrays are PyTorch CUDA tensors; the library only sees raw pointers.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib

_DTYPES = {torch.float32: _lib.F32, torch.float64: _lib.F64}
_PATHS = {"auto": _lib.PATH_AUTO, "fused": _lib.PATH_FUSED, "plain": _lib.PATH_PLAIN,
          "fused_unit": _lib.PATH_FUSED_UNIT}


def dtype_code(dtype: torch.dtype) -> int:
    try:
        return _DTYPES[dtype]
    except KeyError:
        raise TypeError(f"unsupported dtype {dtype}; use float32 or float64") from None


def stream_handle(device: torch.device) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise _lib.JubikError("the GB300 response needs a CUDA device; none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def as_device(x, dtype: Optional[torch.dtype], device: torch.device) -> torch.Tensor:
    """Contiguous CUDA tensor view/copy of ``x`` (numpy array or tensor)."""
    if isinstance(x, torch.Tensor):
        t = x
    else:
        t = torch.as_tensor(np.asarray(x))
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    if t.device != device:
        t = t.to(device)
    return t.contiguous()


def ptr(t: Optional[torch.Tensor]) -> C.c_void_p:
    return C.c_void_p(0 if t is None else t.data_ptr())


class PsfSnapshot:
    """The PSF a plan held when an operator ran: its key and a way to set it
    again.  Autograd nodes keep one, so that a backward pass that runs after the
    plan was given another kernel first restores the kernel of its forward."""

    __slots__ = ("key", "source", "layout", "watch", "version")

    def __init__(self, key, source, layout, watch=None):
        self.key, self.source, self.layout = key, source, layout
        # in-place edits of a tensor kernel after the forward are an error, as
        # for any tensor that autograd saved
        if watch is None and isinstance(source, torch.Tensor):
            watch = source
        self.watch = watch if isinstance(watch, torch.Tensor) else None
        self.version = self.watch._version if self.watch is not None else None

    def kernel(self):
        if self.watch is not None and self.watch._version != self.version:
            raise RuntimeError("the PSF kernel of this response was modified in place after the "
                               "forward pass; its gradient cannot be computed")
        return self.source() if callable(self.source) else self.source


class ResponsePlan:
    """Plan for ``R(x) = mask(exposure(psf(x * pixel_area)))`` on one GPU.

    Parameters mirror the reference: ``n_modules`` is the vmapped module axis
    of ``erosita_response.py:209-212``, ``shape`` the field ``Domain.shape[-2:]``,
    ``n_patches`` / ``margin`` those of ``linpatch_convolve``
    (``jubik/convolve.py:66``).  ``path`` picks the fused path ("auto"/"fused":
    patch spectra shared across modules when there are several), the fused path
    with one kernel per unit and no sharing ("fused_unit"), or the unfused one
    ("plain").  With ``path="auto"`` the environment variable ``JUBIK_PATH``
    (one of the path names) overrides the automatic choice, for debugging.
    """

    def __init__(self, n_modules: int, n_energies: int, shape: Sequence[int], n_patches: int,
                 margin: int, dtype: torch.dtype = torch.float32, path: str = "auto",
                 pixel_area: float = 1.0, device: Optional[torch.device] = None):
        self.device = device if device is not None else require_cuda()
        self.dtype = dtype
        if path == "auto":  # debugging override of the automatic choice
            path = os.environ.get("JUBIK_PATH", "auto")
        if path not in _PATHS:
            raise ValueError(f"path must be one of {sorted(_PATHS)}, got {path!r}")
        self.n_modules, self.n_energies = int(n_modules), int(n_energies)
        self.shape = (int(shape[0]), int(shape[1]))
        self.n_patches, self.margin = int(n_patches), int(margin)
        self.pixel_area = float(pixel_area)
        self.dx = self.shape[0] // self.n_patches
        self.K = 2 * self.dx
        self.P = self.K + 2 * self.margin
        desc = _lib.PlanDesc(self.n_modules, self.n_energies, self.shape[0], self.shape[1],
                             self.n_patches, self.margin, dtype_code(dtype), _PATHS[path],
                             self.pixel_area)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().jubik_plan_create(C.byref(desc), C.byref(h)),
                       "jubik_plan_create")
        self._h = h
        p = C.c_int32()
        _lib.call("jubik_plan_path", self._h, C.byref(p))
        self.path = {1: "fused", 2: "plain"}[p.value]
        self.shared_spectra = self.path == "fused" and path != "fused_unit" and self.n_modules >= 2
        self._refresh_readout()
        self._keep = []  # tensors the plan reads asynchronously
        self.psf_key = None  # identifies the PSF spectra the plan holds
        self._psf = None     # PsfSnapshot of them

    # -------------------------------------------------------------- state
    def close(self):
        if getattr(self, "_h", None):
            torch.cuda.synchronize(self.device)
            _lib.load().jubik_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def workspace_bytes(self) -> int:
        b = C.c_int64()
        _lib.call("jubik_plan_workspace_bytes", self._h, C.byref(b))
        return b.value

    def _s(self):
        return stream_handle(self.device)

    PHASES = ("forward", "adjoint", "likelihood", "memset", "forward_patch", "adjoint_patch",
              "finish")

    def set_dependent_launch(self, on: bool = True) -> "ResponsePlan":
        """Programmatic dependent launch between the kernels of a call (default on)."""
        _lib.call("jubik_plan_set_dependent_launch", self._h, 1 if on else 0)
        return self

    def set_forward_run(self, run_len: int = 0) -> "ResponsePlan":
        """Patches per run of the module-shared FP32 forward at FFT side 192: 4
        reduces the fewest field rows, 2 and 1 give more work items for small
        fields, 0 lets the library choose (the default).  Raises
        JubikUnsupported for runs the geometry cannot take, ValueError for
        other lengths."""
        _lib.call("jubik_plan_set_forward_run", self._h, int(run_len))
        return self

    @property
    def forward_run(self) -> int:
        """The run length the forward uses (1 where it does not run in runs)."""
        r = C.c_int32()
        _lib.call("jubik_plan_forward_run", self._h, C.byref(r))
        return int(r.value)

    def autotune(self, x, candidates: Sequence[int] = (1, 2, 4), reps: int = 5) -> dict:
        """Time one energy-and-gradient pass on sky x (the plan's data must be
        set) for each applicable forward run length, keep the fastest, and
        return {run length: ms per pass}."""
        x = self._sky(x)
        grad = torch.empty((self.n_energies,) + self.shape, dtype=self.dtype,
                           device=self.device)
        energy = torch.empty((), dtype=torch.float64, device=self.device)
        times = {}
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device)
            for r in candidates:
                try:
                    self.set_forward_run(r)
                except _lib.JubikUnsupported:
                    continue
                for _ in range(2):
                    self.energy_and_grad(x, energy=energy, grad=grad)
                t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                t0.record(stream)
                for _ in range(reps):
                    self.energy_and_grad(x, energy=energy, grad=grad)
                t1.record(stream)
                t1.synchronize()
                times[int(r)] = t0.elapsed_time(t1) / reps
        if times:
            self.set_forward_run(min(times, key=times.get))
        return times

    def set_profiling(self, on: bool = True) -> None:
        """Bracket every kernel phase with CUDA events (resets the totals)."""
        _lib.call("jubik_plan_set_profiling", self._h, int(bool(on)))

    def profile(self) -> dict:
        """{phase: (total ms, launches)} since profiling was switched on."""
        ms = (C.c_double * len(self.PHASES))()
        n = (C.c_int64 * len(self.PHASES))()
        _lib.call("jubik_plan_profile", self._h, ms, n)
        return {name: (float(ms[i]), int(n[i])) for i, name in enumerate(self.PHASES)}

    def _refresh_readout(self):
        sizes = (C.c_int64 * self.n_modules)()
        tot = C.c_int64()
        _lib.call("jubik_plan_readout_sizes", self._h, sizes, C.byref(tot))
        self.readout_sizes = [int(v) for v in sizes]
        self.readout_total = int(tot.value)

    def set_psf(self, psf, layout: str = "auto", key=None, source=None,
                watch=None) -> "ResponsePlan":
        """PSF kernels: (M, n^2, E, K, K) pre-cut windows or (M, n^2, E, nx, ny)
        full-field kernels; an array without the E axis is broadcast over
        energies (``convolve.py:167-171``).

        ``key`` names these kernels (a fresh token when None) and becomes
        ``psf_key``; ``source`` (default: ``psf`` itself) is what
        :meth:`restore_psf` sets again -- a tensor, or a callable returning the
        kernels, so that a snapshot need not hold a device copy; ``watch`` is
        the caller's tensor whose in-place edits invalidate the snapshot."""
        self._set_psf(psf, layout)
        self.psf_key = key if key is not None else object()
        self._psf = PsfSnapshot(self.psf_key, psf if source is None else source, layout,
                                watch=watch)
        return self

    def psf_snapshot(self) -> Optional[PsfSnapshot]:
        """The PSF the plan holds now (for :meth:`restore_psf`)."""
        return self._psf

    def restore_psf(self, snap: Optional[PsfSnapshot]) -> None:
        """Set the PSF of ``snap`` again if the plan holds another one."""
        if snap is None or (self.psf_key is snap.key or self.psf_key == snap.key):
            return
        self._set_psf(snap.kernel(), snap.layout)
        self.psf_key, self._psf = snap.key, snap

    def _set_psf(self, psf, layout: str) -> None:
        t = as_device(psf, self.dtype, self.device)
        n2 = self.n_patches ** 2
        if t.dim() == 4:
            t = t.unsqueeze(2)
            bcast = 1
        elif t.dim() == 5:
            bcast = 0
        else:
            raise ValueError("kernel must have shape (M, n^2, [E,] k, k)")
        if t.shape[0] != self.n_modules or t.shape[1] != n2:
            raise ValueError(f"kernel leading shape {tuple(t.shape[:2])} does not match "
                             f"(modules, n^2) = ({self.n_modules}, {n2})")
        if not bcast and t.shape[2] != self.n_energies:
            raise ValueError("kernel energy axis does not match the plan")
        win = tuple(t.shape[-2:])
        if layout == "auto":
            layout = "precut" if win == (self.K, self.K) else "full"
        if layout == "precut" and win != (self.K, self.K):
            raise ValueError(f"pre-cut kernels must be ({self.K}, {self.K}), got {win}")
        if layout == "full" and win != self.shape:
            raise ValueError(f"full-field kernels must be {self.shape}, got {win}")
        code = _lib.PSF_PRECUT if layout == "precut" else _lib.PSF_FULL
        _lib.call("jubik_plan_set_psf", self._h, ptr(t), code, bcast, self._s())
        torch.cuda.current_stream(self.device).synchronize()

    def set_exposure(self, exposure=None, readmask=None) -> "ResponsePlan":
        """exposure (M,E,nx,ny) (None = ones); readmask (M,E,nx,ny) bool, True
        where the pixel is read out (None = all)."""
        full = (self.n_modules, self.n_energies) + self.shape
        e = None
        if exposure is not None:
            e = as_device(exposure, self.dtype, self.device)
            e = e.expand(full).contiguous() if tuple(e.shape) != full else e
        m = None
        if readmask is not None:
            m = as_device(readmask, None, self.device)
            m = m.expand(full) if tuple(m.shape) != full else m
            m = m.to(torch.uint8).contiguous()
        _lib.call("jubik_plan_set_exposure", self._h, ptr(e), ptr(m), self._s())
        self._refresh_readout()
        return self

    def readout_index(self) -> torch.Tensor:
        """Flat (M,E,nx,ny) indices of the read-out pixels (device int64 view)."""
        p = C.c_void_p()
        _lib.call("jubik_plan_readout_index", self._h, C.byref(p))
        if self.readout_total == 0:
            return torch.empty(0, dtype=torch.int64, device=self.device)
        return _wrap_device(p.value, self.readout_total, "<i8", self.device).clone()

    def set_data(self, counts) -> "ResponsePlan":
        """Poisson counts in readout order (total,) -> int32 on the device."""
        d = as_device(counts, torch.int32, self.device).reshape(-1)
        if d.numel() != self.readout_total:
            raise ValueError(f"data has {d.numel()} entries, the readout has {self.readout_total}")
        if torch.any(d < 0):
            raise ValueError("`data` may not be negative")
        _lib.call("jubik_plan_set_data", self._h, ptr(d), self._s())
        torch.cuda.current_stream(self.device).synchronize()
        return self

    # -------------------------------------------------------------- operators
    def _sky(self, x) -> torch.Tensor:
        t = as_device(x, self.dtype, self.device)
        want = (self.n_energies,) + self.shape
        if tuple(t.shape) != want:
            t = t.reshape(want)
        return t

    def psf_forward(self, x, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        x = self._sky(x)
        if out is None:
            out = torch.empty((self.n_modules, self.n_energies) + self.shape, dtype=self.dtype,
                              device=self.device)
        _lib.call("jubik_psf_forward", self._h, ptr(x), ptr(out), self._s())
        return out

    def psf_adjoint(self, cot, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        c = as_device(cot, self.dtype, self.device).reshape(
            (self.n_modules, self.n_energies) + self.shape)
        if out is None:
            out = torch.empty((self.n_energies,) + self.shape, dtype=self.dtype,
                              device=self.device)
        _lib.call("jubik_psf_adjoint", self._h, ptr(c), ptr(out), self._s())
        return out

    def response(self, x, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        x = self._sky(x)
        if out is None:
            out = torch.empty(self.readout_total, dtype=self.dtype, device=self.device)
        _lib.call("jubik_response_forward", self._h, ptr(x), ptr(out), self._s())
        return out

    def response_jvp(self, t, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Tangent of the (linear) response at any point: R(t)."""
        t = self._sky(t)
        if out is None:
            out = torch.empty(self.readout_total, dtype=self.dtype, device=self.device)
        _lib.call("jubik_response_jvp", self._h, ptr(t), ptr(out), self._s())
        return out

    def response_vjp(self, cot, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        c = as_device(cot, self.dtype, self.device).reshape(-1)
        if c.numel() != self.readout_total:
            raise ValueError("cotangent size does not match the readout")
        if out is None:
            out = torch.empty((self.n_energies,) + self.shape, dtype=self.dtype,
                              device=self.device)
        _lib.call("jubik_response_vjp", self._h, ptr(c), ptr(out), self._s())
        return out

    def energy_and_grad(self, x, need_grad: bool = True, energy: Optional[torch.Tensor] = None,
                        grad: Optional[torch.Tensor] = None):
        """Poisson energy (float64 0-d device tensor) and dE/dx, one fused pass."""
        x = self._sky(x)
        if energy is None:
            energy = torch.empty((), dtype=torch.float64, device=self.device)
        if need_grad and grad is None:
            grad = torch.empty((self.n_energies,) + self.shape, dtype=self.dtype,
                               device=self.device)
        _lib.call("jubik_poisson_energy_grad", self._h, ptr(x), ptr(energy),
                  ptr(grad if need_grad else None), self._s())
        return energy, (grad if need_grad else None)

    def energy_and_grad_logsky(self, s, need_grad: bool = True,
                               energy: Optional[torch.Tensor] = None,
                               grad: Optional[torch.Tensor] = None):
        """Poisson energy and gradient for the sky exp(s[:E, :nx, :ny]) of a
        (possibly padded) log-sky array s (``sky_models.py:340-341``): the exp
        and the crop run inside the response's first kernel.  Returns the energy
        (float64 0-d) and dE/ds (shape of s, zero outside the crop)."""
        t = as_device(s, self.dtype, self.device)
        if t.dim() == 2:
            t = t.unsqueeze(0)
        if t.dim() != 3:
            raise ValueError("log-sky must have shape (E', nx', ny')")
        ep, n0, n1 = (int(v) for v in t.shape)
        if energy is None:
            energy = torch.empty((), dtype=torch.float64, device=self.device)
        if need_grad and grad is None:
            grad = torch.empty_like(t)
        _lib.call("jubik_poisson_energy_grad_logsky", self._h, ptr(t), ep, n0, n1, ptr(energy),
                  ptr(grad if need_grad else None), self._s())
        return energy, (grad if need_grad else None)

    def set_metric_lambda(self, lam) -> "ResponsePlan":
        """Take the metric weights eps^2/lam from ``lam`` (expected counts in
        readout order, float32 or float64; e.g. the response of a float64 plan of
        the same instrument) for the next ``metric(None, v)`` calls.  An FP32
        plan's own lam carries the FP32 forward's error, which 1/lam amplifies at
        faint pixels; a float64 lam leaves the FP32 metric only its own rounding."""
        t = lam if isinstance(lam, torch.Tensor) else torch.as_tensor(np.asarray(lam))
        if t.dtype not in (torch.float32, torch.float64):
            t = t.to(torch.float64)
        t = t.to(self.device).contiguous().reshape(-1)
        if t.numel() != self.readout_total:
            raise ValueError("lam size does not match the readout")
        self._metric_lam = t  # read by a kernel queued on the current stream
        _lib.call("jubik_plan_set_metric_lambda", self._h, ptr(t), dtype_code(t.dtype), self._s())
        return self

    def metric(self, x, v, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """R^T diag(1/lam) R v with lam = R(x); x=None reuses the last lam."""
        xx = None if x is None else self._sky(x)
        vv = self._sky(v)
        if out is None:
            out = torch.empty((self.n_energies,) + self.shape, dtype=self.dtype,
                              device=self.device)
        _lib.call("jubik_metric_apply", self._h, ptr(xx), ptr(vv), ptr(out), self._s())
        return out

    def split_readout(self, flat: torch.Tensor):
        """Split a flat readout vector into the per-module pieces."""
        return list(torch.split(flat, self.readout_sizes))


def _wrap_device(address: int, n: int, typestr: str, device: torch.device) -> torch.Tensor:
    """Tensor view of n elements at a raw device address (callers copy it)."""

    class _View:
        __cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                    "data": (address, False), "version": 3}

    return torch.as_tensor(_View(), device=device)
