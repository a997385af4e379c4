"""Benchmark: Mpix/s of the FP32 fused response forward + VJP with the Poisson
likelihood (energy + gradient) on the 1024^2 x 7 modules x 3 energies
workload (16x16 patches of stride 64, margin 32, FFT side 192).

One step = lam = R(x); H = sum(lam - d log lam); grad = R^T(1 - d/lam), i.e.
one ``jubik_poisson_energy_grad`` call: 22.02 Mpix of data-space pixels.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  ``--impl reference`` times the float64 CPU
restatement of the reference path on the host cores (the reference itself is
JAX, which is not installed) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {"workload": "response_fwd_vjp_poisson", "field": [1024, 1024], "modules": 7,
            "energies": 3, "patches_per_axis": 16, "patch_stride": 64, "margin": 32,
            "fft_side": 192, "psf": "Moffat beta 2.5, FWHM 2-8 px, per-module rotation",
            "l2": "inputs larger than L2 (801 MB of PSF spectra per pass)"}
METRIC = "Mpix/s response fwd+VJP (1024²×7 modules×3 E); FP32 vs FP64, rel err ≤1e-6"


def workload(nx):
    """The workload dict for field side ``nx`` (n = nx / 64 patches per axis)."""
    if nx == WORKLOAD["field"][0]:
        return dict(WORKLOAD)
    n = nx // WORKLOAD["patch_stride"]
    return dict(WORKLOAD, field=[nx, nx], patches_per_axis=n,
                l2=f"PSF spectra {7 * 3 * n * n * (192 * 96 + 192) * 8 / 1e6:.0f} MB per pass")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--path", choices=["auto", "fused", "fused_unit", "plain"], default="auto")
    ap.add_argument("--nx", type=int, default=1024)
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the FP64 comparison and the CPU baseline")
    ap.add_argument("--profile-only", action="store_true",
                    help="one warm-up and two steps (for a launch list under a profiler)")
    ap.add_argument("--leg", choices=["step", "sky", "batch", "batch7", "fp64", "psf", "sampling",
                                      "p384"],
                    default="step",
                    help="with --profile-only: the response step, the correlated-field sky "
                         "(log-sky and VJP), the grouped uneven batch (one module per field, "
                         "or batch7: seven), the FP64 unfused step, "
                         "the PSF-patch interpolation, the sampling kernels (dot products, "
                         "Poisson draws), or the FP32 step at FFT side 384 (1024^2 x 7 x 3, "
                         "8 x 8 patches, margin 64: the unfused path)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the GPU works."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: str):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", index, f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def _rows(self):
        with open(self.file.name) as f:
            return [r.split(",") for r in f.read().splitlines() if r.count(",") >= 8]

    def wait_first(self, limit_s: float = 5.0):
        """Wait (at most limit_s) until nvidia-smi has written its first row, so
        that its samples cover what runs next."""
        t0 = time.time()
        while self.proc is not None and time.time() - t0 < limit_s and not self._rows():
            time.sleep(0.02)

    def mark(self) -> int:
        """Number of rows written so far: brackets a region of the run."""
        return len(self._rows()) if self.proc is not None else 0

    def stop(self, window=None):
        """Median SM clock and the throttle reasons seen over the rows written
        inside window = (mark at start, mark at end); the whole run when no row
        fell inside it."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = self._rows()
        os.unlink(self.file.name)
        scope = "whole run"
        if window is not None and window[1] > window[0]:
            rows, scope = rows[window[0]:window[1]], "timed region"
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm), "scope": scope}


def replica_throughput(ms_local: float, mpix_per_rank: float, pg=None, device=None):
    """Whole-job throughput of N independent replicas: the slowest rank's
    ms per step (max over ranks) and N x Mpix per step / that time."""
    ms = ms_local
    world = 1
    if pg is not None:
        import torch

        world = pg.get_world_size()
        t = torch.tensor([ms_local], dtype=torch.float64, device=device)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * mpix_per_rank / (ms / 1e3)


# ------------------------------------------------------------------ CPU legs
def cpu_workload(inst, data):
    """One step of the float64 CPU restatement on the whole workload (every
    module and energy: the same 22.02 Mpix as a GPU step at 1024^2): returns a
    callable running lam = R(x), the Poisson energy and R^T(1 - d/lam)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import jubik_oracle as O

    M, E, nx = inst.n_modules, inst.n_energies, inst.shape[0]
    dom = O.Domain((E, nx, nx), (1.0, 1.0, 1.0))
    R = O.Response(dom, inst.psf, inst.n_patches, inst.margin, inst.exposure, inst.readmask)
    x = inst.sky.astype(np.float64)
    sizes = [int(inst.readmask[m].sum()) for m in range(M)]
    parts = np.split(np.asarray(data), np.cumsum(sizes)[:-1])

    def step():
        return R.energy_and_grad(x, parts)

    return step


def cpu_sample(inst, data, min_seconds=0.0, max_reps=100):
    """Whole-workload CPU steps until ``min_seconds`` have passed (at least
    one).  Returns (Mpix/s over all steps, seconds, steps)."""
    step = cpu_workload(inst, data)
    mpix = inst.n_modules * inst.n_energies * inst.shape[0] * inst.shape[1] / 1e6
    reps, t0 = 0, time.perf_counter()
    while True:
        step()
        reps += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds or reps >= max_reps:
            break
    return reps * mpix / dt, dt, reps


def workload_data(inst):
    """Poisson counts of the workload, drawn from lam = R(x) on the CPU."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import jubik_oracle as O
    from jubik_gb300 import synthetic

    E, nx = inst.n_energies, inst.shape[0]
    R = O.Response(O.Domain((E, nx, nx), (1.0, 1.0, 1.0)), inst.psf, inst.n_patches,
                   inst.margin, inst.exposure, inst.readmask)
    lam = np.concatenate(R(inst.sky.astype(np.float64)))
    return synthetic.poisson_data(lam, seed=1)


def run_reference(args, rank, world):
    if rank != 0:
        return
    from jubik_gb300 import synthetic

    inst = synthetic.config2(nx=args.nx)
    data = workload_data(inst)
    step = cpu_workload(inst, data)
    mpix = inst.n_modules * inst.n_energies * inst.shape[0] * inst.shape[1] / 1e6
    # one step = the whole workload (about 5 s on 16 cores); warm-up (at most 3)
    # and timed steps are capped so that the run stays within about two minutes
    warm = max(1, min(args.warmup, 3))
    t_one = None
    for _ in range(warm):
        t0 = time.perf_counter()
        step()
        dt = time.perf_counter() - t0
        t_one = dt if t_one is None else min(t_one, dt)
    steps = max(1, min(args.steps, int(100.0 / max(t_one, 1e-3))))
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    value = mpix / t
    cores = os.cpu_count()
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mpix/s",
            "n_gpus": world, "steps": steps, "warmup": warm,
            "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload(args.nx),
            "cpu_baseline": {"value": value, "unit": "Mpix/s", "cores": cores, "kind": "port",
                             "sample": "float64 numpy/scipy.fft restatement of the whole "
                                       f"workload per step ({inst.n_modules} modules x "
                                       f"{inst.n_energies} energies x {args.nx}^2 px, "
                                       f"{inst.n_modules * inst.n_energies * inst.n_patches ** 2}"
                                       " patch units); median of the timed steps"},
            "e2e": {"value": value, "unit": "Mpix/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def uneven_batch_leg(dev, n_streams=8, passes=10, modules=1, count=64):
    """Independent problems of uneven size (the config-5 geometry: sides
    144..896, FFT sides 32/64/128, 1..3 energies; ``count`` of them, each with
    ``modules`` telescope modules): energy + gradient of all of them, problem
    after problem on one stream, as one CUDA-graph launch of the same pass with
    the problems spread over ``n_streams`` branches, and as grouped launches."""
    import torch

    import jubik_gb300 as ju
    from jubik_gb300 import synthetic

    if modules == 1:
        insts = synthetic.config5(count=count)
    else:
        insts = [synthetic.config2(nx=g["nx"], dx=g["dx"], margin=g["margin"],
                                   n_modules=modules, n_energies=g["E"], seed=g["seed"])
                 for g in synthetic.config5_geometry(count=count)]
    b = ju.ProblemBatch(insts, dtype=torch.float32, n_streams=n_streams, device=dev)
    try:
        lam = b.expected_counts()
        b.set_data([synthetic.poisson_data(l, 7 + k) for k, l in enumerate(lam)])
        chosen = b.autotune()
        s = torch.cuda.current_stream(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)

        def timed(fn):
            for _ in range(3):
                fn()
            torch.cuda.synchronize(dev)
            e0.record(s)
            for _ in range(passes):
                fn()
            e1.record(s)
            torch.cuda.synchronize(dev)
            return e0.elapsed_time(e1) / passes

        loop_ms = timed(b.energy_and_grad)
        b.capture()
        graph_ms = timed(b.replay)
        out = {"problems": len(insts), "modules": modules, "mpix_per_pass": b.mpix,
               "streams": n_streams,
               "paths": {str(k): v for k, v in chosen.items()},
               "autotune_ms": {str(k): v for k, v in b.timings.items()},
               "loop_ms": loop_ms, "graph_ms": graph_ms, "loop_launches": 5 * len(insts),
               "loop_mpix_s": b.mpix / (loop_ms / 1e3), "graph_mpix_s": b.mpix / (graph_ms / 1e3),
               "graph_speedup": loop_ms / graph_ms}
        if b.group():  # one launch per stage and FFT side over all problems
            grouped_ms = timed(b.energy_and_grad)
            b.capture()
            grouped_graph_ms = timed(b.replay)
            out.update({"grouped_launches": b.launches_per_pass(), "grouped_ms": grouped_ms,
                        "grouped_graph_ms": grouped_graph_ms,
                        "grouped_mpix_s": b.mpix / (grouped_ms / 1e3),
                        "grouped_graph_mpix_s": b.mpix / (grouped_graph_ms / 1e3)})
        return out
    finally:
        b.close()


def unfused_leg(dev, nx, dx, margin, n_modules, n_energies, geometry, passes=20):
    """Energy + gradient steps (FP32) of a geometry whose FFT side is beyond the
    fused tile, on synthetic inputs: the unfused path, event-timed."""
    import torch

    import jubik_gb300 as ju
    from jubik_gb300 import synthetic

    inst = synthetic.config2(nx=nx, dx=dx, margin=margin, n_modules=n_modules,
                             n_energies=n_energies, dtype=np.float32)
    mpix = inst.n_modules * inst.n_energies * inst.shape[0] * inst.shape[1] / 1e6
    plan = ju.ResponsePlan(n_modules, n_energies, inst.shape, inst.n_patches, inst.margin,
                           dtype=torch.float32, device=dev)
    try:
        plan.set_psf(inst.psf)
        plan.set_exposure(inst.exposure, inst.readmask)
        x = torch.as_tensor(inst.sky, device=dev)
        plan.set_data(synthetic.poisson_data(plan.response(x).double().cpu().numpy(), seed=1))
        energy = torch.empty((), dtype=torch.float64, device=dev)
        grad = torch.empty_like(x)
        s = torch.cuda.current_stream(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        for _ in range(5):
            plan.energy_and_grad(x, energy=energy, grad=grad)
        torch.cuda.synchronize(dev)
        e0.record(s)
        for _ in range(passes):
            plan.energy_and_grad(x, energy=energy, grad=grad)
        e1.record(s)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / passes
        return {"geometry": geometry, "path": plan.path, "mpix": mpix, "ms": ms,
                "mpix_s": mpix / (ms / 1e3)}
    finally:
        plan.close()


def chandra_demo_leg(dev, passes=20):
    """The geometry of the reference's Chandra demo (demos/configs/chandra_demo.yaml:
    a 512^2 sky, one observation, 3 energy bins, 4 x 4 patches and margin fraction
    0.062, i.e. margin 32 and FFT side 320, beyond the fused tile)."""
    return unfused_leg(dev, 512, 128, 32, 1, 3,
                       "512^2 x 1 observation x 3 energies, 4 x 4 patches, margin 32, P 320",
                       passes)


def p384_leg(dev, passes=10):
    """The benchmark field (1024^2 x 7 modules x 3 energies) cut into 8 x 8
    patches: margin 64 (erosita_response.py:207's rule) and FFT side 384."""
    return unfused_leg(dev, 1024, 128, 64, 7, 3,
                       "1024^2 x 7 modules x 3 energies, 8 x 8 patches, margin 64, P 384",
                       passes)


def erosita_demo_leg(dev, passes=20):
    """The geometry of the reference's eROSITA demo (demos/configs/eROSITA_demo.yaml:
    a 512^2 sky, telescope modules 1 and 2, 3 energy bins, 8 x 8 patches and margin
    fraction 0.062, i.e. margin 32 and FFT side 192) on synthetic inputs:
    energy + gradient steps with the library's forward run length, then with the
    one ResponsePlan.autotune measures fastest."""
    import torch

    import jubik_gb300 as ju
    from jubik_gb300 import synthetic

    inst = synthetic.config2(nx=512, n_modules=2, n_energies=3, dtype=np.float32)
    M, E, nx = inst.n_modules, inst.n_energies, inst.shape[0]
    mpix = M * E * nx * nx / 1e6
    plan = ju.ResponsePlan(M, E, inst.shape, inst.n_patches, inst.margin, dtype=torch.float32,
                           device=dev)
    try:
        plan.set_psf(inst.psf)
        plan.set_exposure(inst.exposure, inst.readmask)
        x = torch.as_tensor(inst.sky, device=dev)
        plan.set_data(synthetic.poisson_data(plan.response(x).double().cpu().numpy(), seed=1))
        energy = torch.empty((), dtype=torch.float64, device=dev)
        grad = torch.empty_like(x)
        s = torch.cuda.current_stream(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)

        def timed():
            for _ in range(5):
                plan.energy_and_grad(x, energy=energy, grad=grad)
            torch.cuda.synchronize(dev)
            e0.record(s)
            for _ in range(passes):
                plan.energy_and_grad(x, energy=energy, grad=grad)
            e1.record(s)
            torch.cuda.synchronize(dev)
            return e0.elapsed_time(e1) / passes

        auto_run = plan.forward_run
        auto_ms = timed()
        tuned = plan.autotune(x, reps=passes)
        tuned_ms = timed()
        return {"geometry": "512^2 x 2 modules x 3 energies, 8 x 8 patches, margin 32, P 192",
                "mpix": mpix, "auto_run": auto_run, "auto_ms": auto_ms,
                "auto_mpix_s": mpix / (auto_ms / 1e3),
                "autotune_ms": {str(k): v for k, v in tuned.items()},
                "tuned_run": plan.forward_run, "tuned_ms": tuned_ms,
                "tuned_mpix_s": mpix / (tuned_ms / 1e3)}
    finally:
        plan.close()


# ------------------------------------------------------------------ GPU leg
def sky_model_leg(plan, dev, nx, E, mpix, reps=20):
    """The diffuse sky model in front of the response: two correlated fields
    (spatial, spectral index) on the padded grid good_fft_size(1.1075 nx)^2
    (the demos' s_padding_ratio), the log-sky of E energy bins cropped to
    nx^2, and the Poisson energy and gradient back to the excitations."""
    import torch

    from jubik_gb300 import sky as jsky
    shape = (jsky.good_fft_size(int(nx * 1.1075)),) * 2
    e_min = np.geomspace(0.2, 2.0, E)
    coef = jsky.diffuse_coefficients(e_min, 2.0 * e_min, 1.0)
    sky = jsky.CorrelatedFieldSky(shape, 1.0, n_fields=2, crop=(nx, nx), coefficients=coef,
                                  dtype=torch.float32, device=dev)
    rng = np.random.default_rng(12)
    k = sky.mode_lengths / sky.mode_lengths[-1]
    base = (1 + (k / 0.05) ** 2) ** -1.0 * 8 / np.sqrt(sky.pindex.size)
    amp = torch.as_tensor(np.stack([0.4 * base, 0.05 * base]), dtype=torch.float32, device=dev)
    xi = torch.as_tensor(rng.standard_normal((2,) + shape), dtype=torch.float32, device=dev)
    off = torch.tensor([0.3, -0.2], dtype=torch.float32, device=dev)
    ls = sky.logsky(amp, xi, off)
    g = torch.randn_like(ls)
    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(reps):
            fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / reps

    out = {"padded_grid": list(shape), "fields": 2, "energies": E, "modes": sky.n_modes,
           "logsky_ms": timed(lambda: sky.logsky(amp, xi, off, out=ls)),
           "vjp_ms": timed(lambda: sky.vjp(amp, xi, g_logsky=g)),
           "response_energy_grad_ms": timed(lambda: plan.energy_and_grad_logsky(ls)),
           "chain_energy_grad_ms": timed(lambda: sky.energy_and_grad(plan, amp, xi, off))}
    out["chain_mpix_s"] = mpix / (out["chain_energy_grad_ms"] / 1e3)
    sky.close()
    return out


def profile_sky_leg(dev, nx, E, passes=3):
    """Log-sky and VJP of the sky-model leg, ``passes`` times (for ncu)."""
    import torch

    from jubik_gb300 import sky as jsky
    shape = (jsky.good_fft_size(int(nx * 1.1075)),) * 2
    e_min = np.geomspace(0.2, 2.0, E)
    sky = jsky.CorrelatedFieldSky(shape, 1.0, n_fields=2, crop=(nx, nx),
                                  coefficients=jsky.diffuse_coefficients(e_min, 2 * e_min, 1.0),
                                  dtype=torch.float32, device=dev)
    amp = torch.rand(2, sky.n_modes, device=dev) * 1e-3
    xi = torch.randn((2,) + shape, device=dev)
    off = torch.zeros(2, device=dev)
    ls = sky.logsky(amp, xi, off)
    g = torch.randn_like(ls)
    for _ in range(passes):
        sky.logsky(amp, xi, off, out=ls)
        sky.vjp(amp, xi, g_logsky=g)
    torch.cuda.synchronize()
    sky.close()


def profile_batch_leg(dev, passes=3, modules=1):
    """The grouped pass over the config-5 uneven batch, ``passes`` times (for ncu):
    64 one-module fields on the per-unit kernels, or (modules = 7) 16 fields of
    seven modules on the module-shared kernels."""
    import torch

    import jubik_gb300 as ju
    from jubik_gb300 import synthetic
    if modules == 1:
        insts = synthetic.config5()
        paths = {32: "fused_unit", 64: "fused_unit", 128: "fused_unit"}
    else:
        insts = [synthetic.config2(nx=g["nx"], dx=g["dx"], margin=g["margin"],
                                   n_modules=modules, n_energies=g["E"], seed=g["seed"])
                 for g in synthetic.config5_geometry(count=16)]
        paths = {64: "fused", 128: "fused"}
    b = ju.ProblemBatch(insts, dtype=torch.float32, device=dev, paths=paths)
    b.set_data([synthetic.poisson_data(l, 1) for l in b.expected_counts()])
    if not b.group():
        raise RuntimeError("the config-5 batch did not group")
    for _ in range(passes):
        b.energy_and_grad()
    torch.cuda.synchronize()
    b.close()


def profile_fp64_leg(dev, inst, data, passes=2):
    """The FP64 unfused energy + gradient step on the workload, ``passes`` times."""
    import torch

    import jubik_gb300 as ju
    M, E = inst.n_modules, inst.n_energies
    plan = ju.ResponsePlan(M, E, inst.shape, inst.n_patches, inst.margin, dtype=torch.float64,
                           path="plain", device=dev)
    plan.set_psf(inst.psf.astype(np.float64))
    plan.set_exposure(inst.exposure.astype(np.float64), inst.readmask)
    plan.set_data(data)
    x = torch.as_tensor(inst.sky, dtype=torch.float64, device=dev)
    for _ in range(passes):
        plan.energy_and_grad(x)
    torch.cuda.synchronize()
    plan.close()


def profile_psf_leg(dev, nx, passes=2):
    """PSF patches of one eROSITA-like module (16 x 16 patches, 3 energies, pre-cut
    windows) interpolated from gridded PSFs, ``passes`` times."""
    import torch

    from jubik_gb300 import psf as jpsf
    from jubik_gb300 import synthetic
    infos = synthetic.erosita_like_psf_infos(n_energies=3, field=(nx, nx), grid=128, seed=1)
    dom = ju_domain((3, nx, nx), (1.0, 1.0, 1.0))
    for _ in range(passes):
        jpsf.psf_interpolator(dom, nx // 64, infos, layout="precut", dtype=torch.float64)
    torch.cuda.synchronize()


def profile_p384_leg(dev, nx=1024, passes=2):
    """The FP32 energy+gradient step at FFT side 384 (nx^2 x 7 modules x 3
    energies, patches of stride 128, margin 64: 8 x 8 patches at 1024^2), which
    the fused tile does not hold: the unfused path, ``passes`` times."""
    import torch

    import jubik_gb300 as ju
    from jubik_gb300 import synthetic
    inst = synthetic.config2(nx=nx, dx=128, margin=64, dtype=np.float32)
    plan = ju.ResponsePlan(inst.n_modules, inst.n_energies, inst.shape, inst.n_patches,
                           inst.margin, dtype=torch.float32, device=dev)
    plan.set_psf(inst.psf)
    plan.set_exposure(inst.exposure, inst.readmask)
    x = torch.as_tensor(inst.sky, device=dev)
    plan.set_data(synthetic.poisson_data(plan.response(x).double().cpu().numpy(), seed=1))
    for _ in range(passes):
        plan.energy_and_grad(x)
    torch.cuda.synchronize()
    plan.close()


def ju_domain(shape, distances):
    import jubik_gb300 as ju
    return ju.Domain(shape, distances)


def profile_sampling_leg(dev, lam, passes=2):
    """The sampling kernels of the MGVI loop on workload-sized vectors: FP64 dot
    products of FP32 vectors and Poisson draws of the expected counts."""
    import torch

    from jubik_gb300 import sampling
    a = torch.randn(lam.numel(), device=dev)
    b = torch.randn(lam.numel(), device=dev)
    for i in range(passes):
        sampling.dot(a, b)
        sampling.random_poisson(lam, seed=7, offset=i)
    torch.cuda.synchronize()


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch

    import jubik_gb300 as ju
    from jubik_gb300 import synthetic

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist

    inst = synthetic.config2(nx=args.nx, dtype=np.float32)
    M, E, nx = inst.n_modules, inst.n_energies, inst.shape[0]
    mpix = M * E * nx * nx / 1e6
    plan = ju.ResponsePlan(M, E, inst.shape, inst.n_patches, inst.margin, dtype=torch.float32,
                           path=args.path, pixel_area=1.0, device=dev)
    plan.set_psf(inst.psf)
    plan.set_exposure(inst.exposure, inst.readmask)
    x = torch.as_tensor(inst.sky, device=dev)
    lam = plan.response(x).double().cpu().numpy()
    data = synthetic.poisson_data(lam, seed=1)
    plan.set_data(data)
    energy = torch.empty((), dtype=torch.float64, device=dev)
    grad = torch.empty_like(x)

    def step():
        plan.energy_and_grad(x, need_grad=True, energy=energy, grad=grad)

    if args.profile_only:
        if args.leg == "sky":
            profile_sky_leg(dev, nx, E)
        elif args.leg == "batch":
            profile_batch_leg(dev)
        elif args.leg == "batch7":
            profile_batch_leg(dev, modules=7)
        elif args.leg == "fp64":
            profile_fp64_leg(dev, inst, data)
        elif args.leg == "psf":
            profile_psf_leg(dev, nx)
        elif args.leg == "sampling":
            profile_sampling_leg(dev, plan.response(x))
        elif args.leg == "p384":
            profile_p384_leg(dev, nx)
        else:
            step()
            step()
            step()
        torch.cuda.synchronize()
        if rank == 0:
            print(json.dumps({"profile_only": True, "leg": args.leg, "path": plan.path}))
        return

    index = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local if world > 1
                                                                          else 0]
    sampler = ClockSampler(index.strip() or "0")
    sampler.wait_first()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    stream = torch.cuda.current_stream(dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    row0 = sampler.mark()
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    row1 = sampler.mark()
    if pg:
        pg.barrier()
    clocks = sampler.stop((row0, row1))
    ms, value = replica_throughput(ev0.elapsed_time(ev1) / args.steps, mpix, pg, dev)

    # per-kernel durations (events on the launch stream, inside the library)
    plan.set_profiling(True)
    nprof = min(args.steps, 20)
    for _ in range(nprof):
        step()
    prof = plan.profile()
    plan.set_profiling(False)
    per_launch = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in prof.items()}
    launches_per_step = sum(v[1] for k, v in prof.items() if k != "memset") / nprof

    # end-to-end through the public API with pinned host buffers: every step
    # copies its sky in and its energy and gradient out.  The copies run on
    # their own streams, double-buffered, so that step i+1's upload and step
    # i-1's download overlap step i's kernels.
    xh = torch.as_tensor(inst.sky).pin_memory()
    gh = [torch.empty_like(xh).pin_memory() for _ in range(2)]
    eh = [torch.empty((), dtype=torch.float64).pin_memory() for _ in range(2)]
    xd = [torch.empty_like(x) for _ in range(2)]
    gd = [torch.empty_like(x) for _ in range(2)]
    ed = [torch.empty((), dtype=torch.float64, device=dev) for _ in range(2)]
    up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    ev = {k: [torch.cuda.Event() for _ in range(2)] for k in ("in", "done", "out")}
    fresh = [True, True]

    def e2e_step(i):
        b = i % 2
        with torch.cuda.stream(up):
            if not fresh[b]:
                up.wait_event(ev["done"][b])          # step i-2 finished reading xd[b]
            xd[b].copy_(xh, non_blocking=True)
            ev["in"][b].record(up)
        stream.wait_event(ev["in"][b])
        if not fresh[b]:
            stream.wait_event(ev["out"][b])           # step i-2's result downloaded
        plan.energy_and_grad(xd[b], need_grad=True, energy=ed[b], grad=gd[b])
        ev["done"][b].record(stream)
        with torch.cuda.stream(down):
            down.wait_event(ev["done"][b])
            gh[b].copy_(gd[b], non_blocking=True)
            eh[b].copy_(ed[b], non_blocking=True)
            ev["out"][b].record(down)
        fresh[b] = False

    def e2e_run(k, i0=0):
        up.wait_stream(stream)  # no upload starts before the timed region does
        for i in range(k):
            e2e_step(i0 + i)
        stream.wait_stream(down)

    e2e_run(4)
    torch.cuda.synchronize()
    ke = max(1, min(args.steps, 50))
    ev0.record(stream)
    e2e_run(ke, 4)
    ev1.record(stream)
    torch.cuda.synchronize()
    e2e_ms, e2e_value = replica_throughput(ev0.elapsed_time(ev1) / ke, mpix, pg, dev)
    h2d = xh.numel() * xh.element_size()
    d2h = gh[0].numel() * gh[0].element_size() + 8

    # roofline of the dominant kernel (algorithmic = compulsory DRAM bytes per launch)
    U = M * E * inst.n_patches ** 2
    NP = E * inst.n_patches ** 2
    P = inst.P
    spec = U * (P * P // 2 + P) * 8          # PSF spectra, read once per launch
    pspec = NP * P * (P // 2) * 8            # shared patch spectra
    img, sky = M * E * nx * nx * 4, E * nx * nx * 4
    fft_unit = 5.0 * P * P * np.log2(P)      # one real 2-D FFT of side P (5 N log2 N / 2)
    mul_unit = 6.0 * P * (P // 2)
    shared = plan.shared_spectra
    # whole 64-row block rows per patch output (P 192, stride 64, margin 32, runs of
    # 4 patch rows, 2+ modules): the forward runs the run-ordered kernel
    run = (P == 192 and inst.dx == 64 and inst.margin == 32 and nx == inst.n_patches * 64
           and inst.n_patches % 4 == 0 and M >= 2)
    fwd_kernel = "k_fwd_run<float,192>" if run else "k_fwd_from_spec<float,192>"
    kinfo = {  # phase -> (kernel, bytes, flops)
        # the forward leaves both words of the exact two-word image sum
        "forward": (fwd_kernel if shared else "k_fused<float,192,fwd>",
                    spec + (pspec if shared else sky) + 2 * img,
                    U * (fft_unit * (1 if shared else 2) + mul_unit)),
        "adjoint": ("k_adj_to_spec_ord<float,192>" if shared else "k_fused<float,192,adj>",
                    spec + img + (pspec if shared else sky),
                    U * (fft_unit * (1 if shared else 2) + mul_unit)),
        "forward_patch": ("k_sky_spec<float,192>", sky + pspec, NP * fft_unit),
        "adjoint_patch": ("k_adj_from_spec<float,192>", pspec + sky, NP * fft_unit),
    }
    dom = max((k for k in kinfo if per_launch.get(k, 0.0) > 0), key=lambda k: per_launch[k])
    dom_name, dom_bytes, flops = kinfo[dom]
    dom_ms = per_launch[dom]
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    sm_mhz = clocks.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * sm_mhz * 1e6 / 1e12
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "fused_config2_traffic.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            traffic = json.load(f).get(dom_name)

    line = {
        "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded GRF sky, Moffat PSFs, Poisson counts)",
        "config": dict(workload(args.nx), path=plan.path, forward_run=plan.forward_run,
                       parallelism="replicas" if world > 1 else "1gpu"),
        "e2e": {"value": e2e_value, "unit": "Mpix/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                "copies": "pinned host buffers; upload of step i+1 and download of step "
                          "i-1 overlap step i (double-buffered copy streams)"},
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "clocks": clocks,
        "kernels_ms": {(kinfo[k][0] if k in kinfo else k): v for k, v in per_launch.items()
                       if prof[k][1]},
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved,
                     "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                     "traffic": traffic, "algorithmic_bytes": dom_bytes,
                     "peak_source": peak_src,
                     "fp32": {"achieved": flops / (dom_ms / 1e3) / 1e12, "peak": fp32_peak,
                              "unit": "TFLOP/s",
                              "frac": flops / (dom_ms / 1e3) / 1e12 / fp32_peak,
                              "flops": flops,
                              "peak_source": f"{n_sm} SMs x 128 FP32 lanes x 2 x median SM "
                                             "clock"}},
    }

    if rank == 0 and not args.no_extras:
        # accuracy vs the GPU FP64 unfused path and its speed
        plan64 = ju.ResponsePlan(M, E, inst.shape, inst.n_patches, inst.margin,
                                 dtype=torch.float64, path="plain", pixel_area=1.0, device=dev)
        plan64.set_psf(inst.psf.astype(np.float64))
        plan64.set_exposure(inst.exposure.astype(np.float64), inst.readmask)
        plan64.set_data(data)
        x64 = x.double()
        rng = np.random.default_rng(5)
        cot = torch.as_tensor(rng.normal(size=plan.readout_total), device=dev)

        def rel(a, b):
            return float(torch.linalg.norm(a.double() - b) / torch.linalg.norm(b))

        err = {"forward": rel(plan.response(x), plan64.response(x64)),
               "vjp": rel(plan.response_vjp(cot.float()), plan64.response_vjp(cot))}
        e32, g32 = plan.energy_and_grad(x)
        e64, g64 = plan64.energy_and_grad(x64)
        err["energy"] = abs(float(e32) - float(e64)) / abs(float(e64))
        err["grad"] = rel(g32, g64)
        # the floor that lam's FP32 representation sets: the exact (FP64) lam
        # rounded once to FP32, everything else in FP64
        lam64 = plan64.response(x64)
        lam_r = lam64.float().double()
        dd = torch.as_tensor(data, device=dev, dtype=torch.float64)
        err["grad_floor_fp32_lambda"] = rel(plan64.response_vjp(1.0 - dd / lam_r), g64)
        vm = torch.as_tensor(rng.normal(size=x.shape), device=dev)
        m64 = plan64.metric(x64, vm)
        err["metric"] = rel(plan.metric(x, vm.float()), m64)
        err["metric_floor_fp32_lambda"] = rel(plan64.response_vjp(plan64.response(vm) / lam_r),
                                              m64)
        # the FP32 metric with its weights from the FP64 plan's lam (set once per
        # linearisation point): only the FP32 products' own rounding remains
        plan.set_metric_lambda(lam64)
        err["metric_fp64_lambda"] = rel(plan.metric(None, vm.float()), m64)
        # bitwise reproducibility of the FP32 step
        e_a, g_a = plan.energy_and_grad(x)
        e_a, g_a = float(e_a), g_a.clone()
        e_b, g_b = plan.energy_and_grad(x)
        torch.cuda.synchronize()
        line["bitwise_repeatable"] = bool(e_a == float(e_b) and torch.equal(g_a, g_b))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(2):
            plan64.energy_and_grad(x64)
        torch.cuda.synchronize()
        fp64_ms = (time.perf_counter() - t0) / 2 * 1e3
        plan64.close()
        # the other operator calls of the workload, each timed alone (Mpix/s of 22.02 Mpix)
        cot32 = cot.float()
        vt = torch.as_tensor(rng.normal(size=x.shape), device=dev, dtype=torch.float32)
        rout = torch.empty(plan.readout_total, dtype=torch.float32, device=dev)
        xout = torch.empty_like(x)
        calls = {"forward R(x)": lambda: plan.response(x, out=rout),
                 "vjp R^T(c)": lambda: plan.response_vjp(cot32, out=xout),
                 "energy only": lambda: plan.energy_and_grad(x, need_grad=False, energy=energy),
                 "metric R^T diag(1/lam) R v": lambda: plan.metric(None, vt, out=xout)}
        comp = {}
        for name, fn in calls.items():
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            ev0.record(stream)
            for _ in range(20):
                fn()
            ev1.record(stream)
            torch.cuda.synchronize()
            t = ev0.elapsed_time(ev1) / 20
            comp[name] = {"ms": t, "mpix_s": mpix / (t / 1e3)}
        line["operators"] = comp
        line["uneven_batch"] = uneven_batch_leg(dev)
        # the same geometry with the 7 modules of an eROSITA field, 16 fields
        line["uneven_batch_7_modules"] = uneven_batch_leg(dev, modules=7, count=16)
        line["erosita_demo"] = erosita_demo_leg(dev)
        line["chandra_demo"] = chandra_demo_leg(dev)
        line["p384_8x8"] = p384_leg(dev)
        line["sky_model"] = sky_model_leg(plan, dev, nx, E, mpix)
        line["rel_err_vs_fp64_gpu"] = err
        line["fp64_plain_ms_per_step"] = fp64_ms
        line["speedup_vs_fp64_plain"] = fp64_ms / ms
        # CPU baseline: the float64 restatement on whole steps of the workload
        v, dt, reps = cpu_sample(inst, data, min_seconds=10.0, max_reps=3)
        line["cpu_baseline"] = {"value": v, "unit": "Mpix/s", "cores": os.cpu_count(),
                                "kind": "port",
                                "sample": f"float64 numpy/scipy.fft restatement of the whole "
                                          f"workload ({M} modules x {E} energies x {nx}^2 px, "
                                          f"{U} units), {reps} steps in {dt:.1f} s"}
    plan.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
