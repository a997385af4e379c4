"""Uneven batch of independent problems: per-problem parity with the oracle,
and the CUDA-graph pass (problems spread over several streams) against the
eager problem-after-problem pass."""
import numpy as np
import pytest
import torch

import jubik_oracle as O
import jubik_gb300 as ju
from jubik_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _bits(t):
    return t.detach().reshape(-1).contiguous().view(torch.uint8).cpu().numpy().tobytes()


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def small_batch():
    insts = synthetic.config5(count=6, seed=11, min_side=96, max_side=256)
    refs = []
    for k, inst in enumerate(insts):
        E, nx = inst.n_energies, inst.shape[0]
        psf = np.broadcast_to(inst.psf[:, :, None], inst.psf.shape[:2] + (E,) + inst.psf.shape[2:])
        R = O.Response(O.Domain((E, nx, nx), (1.0, 1.0, 1.0)), psf, inst.n_patches, inst.margin,
                       inst.exposure, inst.readmask)
        lam = R(inst.sky)
        data = [synthetic.poisson_data(lam[0], 50 + k)]
        e, g = R.energy_and_grad(inst.sky, data)
        refs.append(dict(data=data[0], energy=e, grad=g))
    return insts, refs


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_batch_eager_and_graph_match_oracle(cuda, small_batch, dtype):
    insts, refs = small_batch
    assert len({2 * (i.shape[0] // i.n_patches) + 2 * i.margin for i in insts}) >= 2
    b = ju.ProblemBatch(insts, dtype=dtype, n_streams=3)
    try:
        b.set_data([r["data"] for r in refs])
        tol, gtol = (1e-12, 1e-11) if dtype == torch.float64 else (1e-6, 5e-4)
        e, g = b.energy_and_grad()
        torch.cuda.synchronize()
        eager_e = e.clone()
        eager_g = [t.clone() for t in g]
        for k, r in enumerate(refs):
            assert abs(float(e[k]) - r["energy"]) / abs(r["energy"]) < tol
            assert rel(g[k], r["grad"]) < gtol
        b.capture()
        for _ in range(2):  # two replays in a row
            b.energy.zero_()
            for t in b.grad:
                t.zero_()
            e2, g2 = b.replay()
            torch.cuda.synchronize()
            # every problem's pass is bitwise reproducible (exact two-word sums,
            # fixed-order reductions), also as branches of one graph
            for k in range(len(insts)):
                assert float(e2[k]) == float(eager_e[k])
                assert torch.equal(g2[k], eager_g[k])
        # the graph reads the sky buffers: new skies give the new energies
        b.x[0].mul_(1.5)
        e3, _ = b.replay()
        plan_e, _ = b.plans[0].energy_and_grad(b.x[0])
        torch.cuda.synchronize()
        assert float(e3[0]) == float(plan_e)
        assert abs(float(e3[0]) - float(eager_e[0])) > 1e-6 * abs(float(eager_e[0]))
    finally:
        b.close()


def test_batch_autotune_picks_a_covering_path(cuda, small_batch):
    insts, refs = small_batch
    b = ju.ProblemBatch(insts, dtype=torch.float32, n_streams=2)
    try:
        with pytest.raises(RuntimeError):
            b.autotune()
        b.set_data([r["data"] for r in refs])
        chosen = b.autotune(reps=2)
        # run lengths are tuned on the module-shared FP32 plans at FFT side 192
        for k, times in b.run_timings.items():
            assert b.plans[k].forward_run == min(times, key=times.get)
        sides = {2 * (i.shape[0] // i.n_patches) + 2 * i.margin for i in insts}
        assert set(chosen) == sides
        assert all(p in ("fused", "fused_unit", "plain") for p in chosen.values())
        e, g = b.energy_and_grad()
        for k, r in enumerate(refs):
            assert abs(float(e[k]) - r["energy"]) / abs(r["energy"]) < 1e-6
    finally:
        b.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_grouped_launches_match_per_problem(cuda, small_batch, dtype):
    """One grouped launch per stage and FFT side gives the per-problem results,
    eagerly and captured in a graph."""
    insts, refs = small_batch
    b = ju.ProblemBatch(insts, dtype=dtype, n_streams=2)
    try:
        b.set_data([r["data"] for r in refs])
        e0, g0 = b.energy_and_grad()
        torch.cuda.synchronize()
        e0 = e0.clone()
        g0 = [t.clone() for t in g0]
        assert b.group()
        sides = {2 * (i.shape[0] // i.n_patches) + 2 * i.margin for i in insts}
        assert b.launches_per_pass() == 4 + 2 * len(sides) < 5 * len(insts)
        # exact two-word sums: every grouped pass gives the same bits.  Against
        # the per-problem pass, the FP32 energy differs by ~1e-9: the grouped
        # likelihood pass splits each image into other blocks, whose per-thread
        # compensated FP32 sums round differently
        etol = 1e-13 if dtype == torch.float64 else 1e-8
        gtol = 1e-13 if dtype == torch.float64 else 1e-6
        first = None
        for run in ("eager", "graph", "graph again"):
            if run == "graph":
                b.capture()
            for t in b.grad:
                t.fill_(float("nan"))  # the grouped pass clears and fills every gradient
            e, g = b.replay() if run.startswith("graph") else b.energy_and_grad()
            torch.cuda.synchronize()
            bits = (_bits(e), [_bits(t) for t in g])
            first = first or bits
            assert bits == first, run
            for k, r in enumerate(refs):
                assert abs(float(e[k]) - float(e0[k])) <= etol * abs(float(e0[k])), (run, k)
                assert rel(g[k], g0[k].double().cpu().numpy()) < gtol, (run, k)
                assert abs(float(e[k]) - r["energy"]) / abs(r["energy"]) < (
                    1e-12 if dtype == torch.float64 else 1e-6)
    finally:
        b.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_grouped_module_shared_and_mixed_problems(cuda, dtype):
    """Problems with several modules (patch spectra shared by the modules) and
    one-module problems of the same FFT side group into separate classes; the
    grouped pass matches the per-problem pass and the oracle."""
    # (nx, dx, margin, M, E): FFT sides 64, 96, 64, 96, 96
    geos = [(64, 16, 16, 2, 2), (96, 32, 16, 3, 1), (64, 16, 16, 1, 2), (128, 32, 16, 2, 2),
            (128, 32, 16, 1, 1)]
    insts, refs = [], []
    for k, (nx, dx, m, M, E) in enumerate(geos):
        inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E, seed=k)
        R = O.Response(O.Domain((E, nx, nx), (1.0, 1.0, 1.0)), inst.psf, nx // dx, m,
                       inst.exposure, inst.readmask)
        lam = R(inst.sky)
        data = [synthetic.poisson_data(l, 60 + 7 * k + i) for i, l in enumerate(lam)]
        e, g = R.energy_and_grad(inst.sky, data)
        insts.append(inst)
        refs.append(dict(data=np.concatenate(data), energy=e, grad=g))
    b = ju.ProblemBatch(insts, dtype=dtype, n_streams=2)
    try:
        b.set_data([r["data"] for r in refs])
        e0, g0 = b.energy_and_grad()
        torch.cuda.synchronize()
        e0 = e0.clone()
        g0 = [t.clone() for t in g0]
        assert b.group()
        # classes: (64, shared), (96, shared), (64, per-unit), (96, per-unit)
        assert b.launches_per_pass() == 4 + 4 + 4 + 2 + 2
        # the same bits on every grouped pass (module sums in module order, exact
        # two-word sums).  Against the per-problem pass the FP32 energy differs by
        # the likelihood pass's other block split (~1e-9), and the gradient by the
        # ordered adjoint's other CTA count: a patch whose modules are split over
        # two CTAs adds its FP32 partial sums in another grouping (~1e-6 here,
        # after the cancellation in 1 - d/lam)
        etol = 1e-13 if dtype == torch.float64 else 1e-8
        gtol = 1e-13 if dtype == torch.float64 else 2e-5
        first = None
        for run in ("eager", "graph", "graph again"):
            if run == "graph":
                b.capture()
            for t in b.grad:
                t.fill_(float("nan"))
            e, g = b.replay() if run.startswith("graph") else b.energy_and_grad()
            torch.cuda.synchronize()
            bits = (_bits(e), [_bits(t) for t in g])
            first = first or bits
            assert bits == first, run
            for k, r in enumerate(refs):
                assert abs(float(e[k]) - float(e0[k])) <= etol * abs(float(e0[k])), (run, k)
                assert rel(g[k], g0[k].double().cpu().numpy()) < gtol, (run, k)
                assert abs(float(e[k]) - r["energy"]) / abs(r["energy"]) < (
                    1e-12 if dtype == torch.float64 else 1e-6)
                if dtype == torch.float64:
                    assert rel(g[k], r["grad"]) < 1e-11
    finally:
        b.close()


def test_group_refuses_unfused_problems(cuda):
    """A problem whose FFT side takes the unfused path keeps the per-problem pass."""
    inst = synthetic.config2(nx=64, dx=16, margin=8, n_modules=2, n_energies=1)  # side 48
    b = ju.ProblemBatch([inst], dtype=torch.float32)
    try:
        lam = b.expected_counts()
        b.set_data([synthetic.poisson_data(lam[0], 1)])
        assert not b.group()
        assert not b.grouped
        e, _ = b.energy_and_grad()
        assert np.isfinite(float(e[0]))
    finally:
        b.close()


def test_group_refuses_plans_changed_after_set_io(cuda, small_batch):
    """A group copies its plans' buffer addresses and readout maps at set_io: a
    plan that gets a new exposure afterwards makes the group's calls fail with
    a state error (instead of reading freed or stale buffers) until set_io."""
    insts, refs = small_batch
    b = ju.ProblemBatch(insts, dtype=torch.float32, n_streams=2)
    try:
        b.set_data([r["data"] for r in refs])
        assert b.group()
        b.energy_and_grad()
        b.plans[0].set_exposure(None, insts[0].readmask)  # drops the exposure buffer
        with pytest.raises(ju.JubikStateError, match="set_io"):
            b.energy_and_grad()
        b.plans[0].set_exposure(insts[0].exposure, insts[0].readmask)
        b.plans[0].set_data(refs[0]["data"])
        assert b.group()  # set_io again
        e, _ = b.energy_and_grad()
        torch.cuda.synchronize()
        for k, r in enumerate(refs):
            assert abs(float(e[k]) - r["energy"]) / abs(r["energy"]) < 1e-6
    finally:
        b.close()
