"""Independent imaging problems of uneven size, evaluated as one batch.

A survey fits many fields, each with its own sky, patch grid, PSFs and data
(one ``jft.Poissonian(data).amend(response)`` per field in J-UBIK).  Small
fields fill only a part of the GPU, and launching their kernels one field
after another leaves it idle between launches.  :class:`ProblemBatch` keeps
one :class:`~.plan.ResponsePlan` per problem and evaluates the Poisson energy
and gradient of all of them in one pass.  :meth:`ProblemBatch.capture` records
that pass once as a CUDA graph: the problems are spread round-robin over
several streams forked from the capture stream, so the graph's branches run
side by side, and one graph launch replaces every per-problem launch.

:meth:`ProblemBatch.autotune` picks the kernel path for each FFT side by
timing the candidates (module-shared fused, per-unit fused, unfused) on the
largest problem of that side.  Problems with one module take the same kernels
on both fused paths.

When every problem runs on a fused FFT side, :meth:`ProblemBatch.group`
switches the pass to grouped launches (``jubik_group_*``): one clearing
kernel; per FFT side, one forward and one adjoint launch over all of that
side's one-module problems and two of each over its several-module problems
(patch spectra shared by the modules, then the units); and one likelihood
pass over all problems -- a handful of launches in place of five per problem.
The grouped pass can be captured too.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from .plan import ResponsePlan, require_cuda, stream_handle


def _fft_side(inst) -> int:
    return 2 * (inst.shape[0] // inst.n_patches) + 2 * inst.margin


class ProblemBatch:
    """Energy and gradient of many independent response problems.

    ``instruments`` are objects with the fields of
    :class:`jubik_gb300.synthetic.Instrument` (n_modules, n_energies, shape,
    n_patches, margin, sky, psf, exposure, readmask, pixel_area).  ``paths``
    maps an FFT side to a kernel path ('auto', 'fused', 'fused_unit', 'plain');
    sides not listed use 'auto'."""

    def __init__(self, instruments: Sequence, dtype: torch.dtype = torch.float32,
                 n_streams: int = 8, paths: Optional[Dict[int, str]] = None,
                 device: Optional[torch.device] = None):
        if len(instruments) == 0:
            raise ValueError("a batch needs at least one problem")
        if n_streams < 1:
            raise ValueError("n_streams must be >= 1")
        self.device = device or require_cuda()
        self.dtype = dtype
        self.instruments = list(instruments)
        self.n_streams = n_streams
        self.paths = dict(paths or {})
        self.plans: List[ResponsePlan] = [self._make_plan(i) for i in self.instruments]
        self.x = [torch.as_tensor(np.asarray(i.sky), device=self.device).to(dtype).contiguous()
                  for i in self.instruments]
        self.energy = torch.zeros(len(self.plans), dtype=torch.float64, device=self.device)
        self.grad = [torch.empty_like(x) for x in self.x]
        self._graph = None
        self._streams: List[torch.cuda.Stream] = []
        self._group = None

    # ------------------------------------------------------------ set-up
    def _make_plan(self, inst, path: Optional[str] = None) -> ResponsePlan:
        P = _fft_side(inst)
        plan = ResponsePlan(inst.n_modules, inst.n_energies, inst.shape, inst.n_patches,
                            inst.margin, dtype=self.dtype,
                            path=path or self.paths.get(P, "auto"),
                            pixel_area=getattr(inst, "pixel_area", 1.0), device=self.device)
        plan.set_psf(inst.psf)
        plan.set_exposure(inst.exposure, inst.readmask)
        return plan

    @property
    def mpix(self) -> float:
        """Data-space Mpix of one pass (modules x energies x field, before masking)."""
        return sum(i.n_modules * i.n_energies * i.shape[0] * i.shape[1]
                   for i in self.instruments) / 1e6

    def set_data(self, counts: Sequence) -> "ProblemBatch":
        """Poisson counts per problem, in each problem's readout order."""
        if len(counts) != len(self.plans):
            raise ValueError("one count vector per problem")
        for plan, d in zip(self.plans, counts):
            plan.set_data(d)
        self._data = [np.asarray(d) for d in counts]
        return self

    def expected_counts(self) -> List[np.ndarray]:
        """R(x) of every problem at the stored skies (host float64)."""
        return [p.response(x).double().cpu().numpy() for p, x in zip(self.plans, self.x)]

    def autotune(self, candidates: Sequence[str] = ("fused", "fused_unit", "plain"),
                 reps: int = 5) -> Dict[int, str]:
        """Time each candidate path on the largest problem of every FFT side
        and rebuild the plans with the fastest.  Needs the data set first."""
        if not hasattr(self, "_data"):
            raise RuntimeError("set_data before autotune")
        lib = _lib.load()
        code = _lib.F32 if self.dtype == torch.float32 else _lib.F64
        by_side: Dict[int, List[int]] = {}
        for k, inst in enumerate(self.instruments):
            by_side.setdefault(_fft_side(inst), []).append(k)
        chosen: Dict[int, str] = {}
        timings: Dict[int, Dict[str, float]] = {}
        for P, ks in sorted(by_side.items()):
            k = max(ks, key=lambda j: self.instruments[j].n_energies * self.instruments[j].shape[0]
                    * self.instruments[j].shape[1])
            res = {}
            for path in candidates:
                if path != "plain" and not lib.jubik_fused_supported(P, code):
                    continue
                plan = self._make_plan(self.instruments[k], path)
                try:
                    plan.set_data(self._data[k])
                    e = torch.empty((), dtype=torch.float64, device=self.device)
                    g = torch.empty_like(self.x[k])
                    for _ in range(2):
                        plan.energy_and_grad(self.x[k], energy=e, grad=g)
                    s = torch.cuda.current_stream(self.device)
                    t0 = torch.cuda.Event(enable_timing=True)
                    t1 = torch.cuda.Event(enable_timing=True)
                    t0.record(s)
                    for _ in range(reps):
                        plan.energy_and_grad(self.x[k], energy=e, grad=g)
                    t1.record(s)
                    t1.synchronize()
                    res[path] = t0.elapsed_time(t1) / reps
                finally:
                    plan.close()
            best = min(res, key=res.get)
            # near ties go to the module-shared kernels: they do less work in all
            # (one sky spectrum per patch for all modules), which counts once the
            # problems share the GPU in a graph or a grouped pass
            if "fused" in res and res["fused"] <= 1.05 * res[best]:
                best = "fused"
            chosen[P] = best
            timings[P] = res
        self.timings = timings
        if chosen != {P: self.paths.get(P, "auto") for P in chosen}:
            self.paths.update(chosen)
            self._rebuild()
        # the forward's run length (patches whose shared block rows meet in TMEM)
        # on every plan that runs the module-shared FP32 kernels at FFT side 192
        self.run_timings = {}
        for k, plan in enumerate(self.plans):
            if plan.shared_spectra and plan.dtype == torch.float32 and plan.P == 192:
                self.run_timings[k] = plan.autotune(self.x[k], reps=reps)
        return chosen

    def group(self) -> bool:
        """Switch the pass to grouped launches; False (and the per-problem pass
        stays) when a problem takes the unfused path."""
        self._drop_group()
        lib = _lib.load()
        n = len(self.plans)
        handles = (C.c_void_p * n)(*[p._h.value for p in self.plans])
        g = C.c_void_p()
        if lib.jubik_group_create(handles, n, C.byref(g)) != _lib.OK:
            return False
        xs = (C.c_void_p * n)(*[x.data_ptr() for x in self.x])
        gs = (C.c_void_p * n)(*[t.data_ptr() for t in self.grad])
        st = lib.jubik_group_set_io(g, xs, gs, C.c_void_p(self.energy.data_ptr()))
        if st != _lib.OK:
            lib.jubik_group_destroy(g)
            _lib.check(st, "jubik_group_set_io")
        self._group = g
        self._graph = None
        return True

    @property
    def grouped(self) -> bool:
        return self._group is not None

    def launches_per_pass(self) -> int:
        """Kernel launches of one pass (grouped, or five per problem)."""
        if self._group is None:
            return 5 * len(self.plans)
        n = C.c_int32()
        _lib.call("jubik_group_launches", self._group, C.byref(n))
        return int(n.value)

    def _drop_group(self):
        if self._group is not None:
            _lib.load().jubik_group_destroy(self._group)
            self._group = None

    def _rebuild(self):
        self._drop_group()
        for p in self.plans:
            p.close()
        self.plans = [self._make_plan(i) for i in self.instruments]
        if hasattr(self, "_data"):
            for plan, d in zip(self.plans, self._data):
                plan.set_data(d)
        self._graph = None

    # ------------------------------------------------------------ evaluation
    def _pass(self, streams: Optional[List[torch.cuda.Stream]]):
        if self._group is not None:
            _lib.call("jubik_group_energy_grad", self._group, stream_handle(self.device))
            return
        if not streams:
            for k, plan in enumerate(self.plans):
                plan.energy_and_grad(self.x[k], energy=self.energy[k], grad=self.grad[k])
            return
        main = torch.cuda.current_stream(self.device)
        for s in streams:
            s.wait_stream(main)
        for k, plan in enumerate(self.plans):
            with torch.cuda.stream(streams[k % len(streams)]):
                plan.energy_and_grad(self.x[k], energy=self.energy[k], grad=self.grad[k])
        for s in streams:
            main.wait_stream(s)

    def energy_and_grad(self):
        """One pass over all problems, problem after problem on the current
        stream.  Returns (energies (float64, one per problem), gradients)."""
        self._pass(None)
        return self.energy, self.grad

    def capture(self) -> "ProblemBatch":
        """Record one pass as a CUDA graph with the problems spread over
        ``n_streams`` branches.  Runs one eager pass first so that every
        kernel's one-time set-up happens outside the capture."""
        self._pass(None)
        torch.cuda.synchronize(self.device)
        self._streams = ([] if self._group is not None else
                         [torch.cuda.Stream(self.device) for _ in range(self.n_streams)])
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            self._pass(self._streams)
        self._graph = graph
        return self

    def replay(self):
        """Launch the captured pass on the current stream (inputs are read
        from the batch's sky buffers ``x``, which callers may overwrite in
        place).  Returns (energies, gradients)."""
        if self._graph is None:
            raise RuntimeError("capture() first")
        self._graph.replay()
        return self.energy, self.grad

    def close(self):
        self._graph = None
        self._drop_group()
        for p in self.plans:
            p.close()
        self.plans = []
