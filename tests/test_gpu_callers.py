"""GPU callers around the response: samplers against their element-by-element
oracle, the FP64 dot, mock data, noise-weighted residuals and the MGVI
linear-sample CG solve."""
import math

import numpy as np
import pytest
import torch
from scipy.sparse.linalg import LinearOperator, cg as scipy_cg

import callers_oracle as CO
import jubik_oracle as O
import jubik_gb300 as ju
from jubik_gb300 import diagnostics, minimization, sampling, synthetic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 2e-6), (torch.float64, 1e-13)],
                         ids=["f32", "f64"])
def test_random_normal_matches_oracle(cuda, dtype, tol):
    n = 100003
    z = sampling.random_normal(n, dtype, seed=12345, offset=7)
    ref = CO.random_normal(n, np.float32 if dtype == torch.float32 else np.float64, 12345, 7)
    got = z.double().cpu().numpy()
    assert np.max(np.abs(got - ref) / np.maximum(1.0, np.abs(ref))) < tol
    # launch-shape independence: a prefix of a longer draw is the shorter draw
    z2 = sampling.random_normal(n + 50, dtype, seed=12345, offset=7)
    assert torch.equal(z, z2[:n])
    assert not torch.equal(z, sampling.random_normal(n, dtype, seed=12345, offset=8))


def test_random_poisson_matches_oracle_draw_for_draw(cuda):
    rng = np.random.default_rng(4)
    lam = np.concatenate([np.zeros(10), rng.uniform(0, 10, 1500), [9.999, 10.0, 10.001],
                          rng.uniform(10, 100, 1500), 10 ** rng.uniform(2, 6, 1000)])
    got = sampling.random_poisson(torch.as_tensor(lam, device=cuda), seed=99, offset=3)
    ref = CO.random_poisson(lam, 99, 3)
    got = got.cpu().numpy().astype(np.int64)
    # libm and CUDA round exp/log/lgamma differently in the last ulp, which can
    # flip an accept/reject decision at a boundary: allow a few in 1e3
    assert np.mean(got != ref) < 3e-3
    with pytest.raises(ValueError):
        sampling.random_poisson(torch.tensor([1.0, -2.0], device=cuda))


@pytest.mark.parametrize("lam", [0.7, 4.0, 12.0, 300.0])
def test_random_poisson_distribution(cuda, lam):
    from scipy import stats
    n = 400000
    d = sampling.random_poisson(torch.full((n,), lam, dtype=torch.float32, device=cuda),
                                seed=int(lam * 10)).cpu().numpy()
    lo, hi = int(stats.poisson.ppf(1e-4, lam)), int(stats.poisson.ppf(1 - 1e-4, lam))
    ks = np.arange(lo, hi + 1)
    obs = np.array([(d == k).sum() for k in ks], float)
    obs[0] += (d < lo).sum()
    obs[-1] += (d > hi).sum()
    p = stats.poisson.pmf(ks, lam)
    p[0] = stats.poisson.cdf(lo, lam)
    p[-1] = stats.poisson.sf(hi - 1, lam)
    chi2 = ((obs - n * p) ** 2 / (n * p)).sum()
    assert stats.chi2.sf(chi2, len(ks) - 1) > 1e-4


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64], ids=["f32", "f64"])
def test_dot_fp64_deterministic(cuda, dtype):
    rng = np.random.default_rng(2)
    a = rng.normal(size=3_000_001)
    b = rng.normal(size=3_000_001)
    ta = torch.as_tensor(a, device=cuda).to(dtype)
    tb = torch.as_tensor(b, device=cuda).to(dtype)
    ref = float(np.dot(ta.double().cpu().numpy(), tb.double().cpu().numpy()))
    d1 = float(sampling.dot(ta, tb))
    d2 = float(sampling.dot(ta, tb))
    assert d1 == d2
    assert abs(d1 - ref) <= 1e-13 * np.sqrt(a.size)
    assert float(sampling.dot(ta[:0], tb[:0])) == 0.0


def _fsum_dot(a, b):
    return math.fsum((np.asarray(a, np.float64) * np.asarray(b, np.float64)).tolist())


def test_dot_fp32_compensated_sums(cuda):
    """FP32 operands: exact product splits in compensated FP32 sums; groups with a
    non-finite word, or whose products all underflow, are summed again in FP64."""
    rng = np.random.default_rng(3)
    n = 20_000_003
    a = rng.normal(size=n).astype(np.float32)
    b = rng.normal(size=n).astype(np.float32)
    ta, tb = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    ref = _fsum_dot(a, b)
    assert abs(float(sampling.dot(ta, tb)) - ref) <= 1e-13 * np.sqrt(n)
    # unaligned views take the element-wise loop
    ref1 = _fsum_dot(a[1:], b[1:])
    assert abs(float(sampling.dot(ta[1:], tb[1:])) - ref1) <= 1e-13 * np.sqrt(n)
    # heavy cancellation: the error scales with the terms, not the result
    c = np.concatenate([a[:1000], -a[:1000]])
    d = np.concatenate([b[:1000], b[:1000]])
    got = float(sampling.dot(torch.from_numpy(c).to(cuda), torch.from_numpy(d).to(cuda)))
    assert abs(got) <= 1e-15 * float(np.abs(c.astype(np.float64) * d).sum())
    # products below the FP32 range (1e-25 * 1e-25) go through the FP64 path
    t = np.full(4096, 1e-25, np.float32)
    got = float(sampling.dot(torch.from_numpy(t).to(cuda), torch.from_numpy(t).to(cuda)))
    assert got == pytest.approx(_fsum_dot(t, t), rel=1e-12)
    # an infinite or NaN operand
    e = a[:5000].copy()
    e[1234] = np.inf
    te = torch.from_numpy(e).to(cuda)
    tb5 = torch.from_numpy(np.abs(b[:5000]) + 1.0).to(cuda)
    assert float(sampling.dot(te, tb5)) == np.inf
    e[1234] = np.nan
    assert np.isnan(float(sampling.dot(torch.from_numpy(e).to(cuda), tb5)))
    # products beyond the FP32 range (1e30 * 1e30) are finite in FP64
    big = np.full(1000, 1e30, np.float32)
    tbig = torch.from_numpy(big).to(cuda)
    assert float(sampling.dot(tbig, tbig)) == pytest.approx(_fsum_dot(big, big), rel=1e-12)


@pytest.fixture(scope="module")
def small_response():
    nx, dx, m, M, E = 64, 16, 8, 2, 2
    inst = synthetic.config2(nx=nx, dx=dx, margin=m, n_modules=M, n_energies=E)
    rd = ju.build_response(ju.Domain((E, nx, nx), (1.0, 1.0, 1.0)), inst.psf, nx // dx, m,
                           exposures=inst.exposure.copy(), flags=inst.readmask.astype(float),
                           keys=["tm1", "tm2"], pixel_area=0.5, dtype=torch.float64)
    ref = O.Response(O.Domain((E, nx, nx), (1.0, 1.0, 1.0)), inst.psf, nx // dx, m,
                     inst.exposure, inst.readmask, pixel_area=0.5)
    return inst, rd, ref


def test_mock_data_is_poisson_of_expected_counts(cuda, small_response):
    inst, rd, ref = small_response
    d = diagnostics.generate_mock_data(rd, inst.sky, seed=5)
    lam = ref(inst.sky)
    assert list(d.tree.keys()) == ["tm1", "tm2"]
    for i, k in enumerate(["tm1", "tm2"]):
        v = d.tree[k].cpu().numpy()
        assert v.dtype == np.int64 and v.shape == lam[i].shape and (v >= 0).all()
        z = (v - lam[i]) / np.sqrt(lam[i])
        assert abs(z.mean()) < 5 / np.sqrt(z.size) and abs(z.std() - 1) < 0.05
        # draw for draw: module i is the oracle's stream (seed, offset i)
        assert np.mean(v != CO.random_poisson(lam[i], 5, i)) < 3e-3
    # the readout transpose puts the counts back on the image
    img = rd["mask_adj"](d)[0].cpu().numpy()
    assert img.shape == inst.readmask.shape
    np.testing.assert_array_equal(img[inst.readmask], np.concatenate(
        [d.tree[k].cpu().numpy() for k in ["tm1", "tm2"]]).astype(float))
    assert (img[~inst.readmask] == 0).all()


@pytest.mark.parametrize("absolute,min_counts", [(False, None), (True, 3000)])
def test_nwr_matches_oracle(cuda, small_response, absolute, min_counts):
    inst, rd, ref = small_response
    data = diagnostics.generate_mock_data(rd, inst.sky, seed=6)
    dl = [data.tree[k].cpu().numpy() for k in ["tm1", "tm2"]]
    rng = np.random.default_rng(8)
    pos = [inst.sky * np.exp(0.05 * rng.normal(size=inst.sky.shape)) for _ in range(3)]
    res, mask = diagnostics.calculate_nwr(pos, lambda x: x, data, rd, abs=absolute,
                                          min_counts=min_counts)
    ref_res, ref_mask = CO.calculate_nwr([ref(p) for p in pos], dl, inst.readmask,
                                         exposure_images=inst.exposure, abs_=absolute,
                                         min_counts=min_counts)
    assert res.shape == ref_res.shape == (2, 3, 2, 64, 64)
    np.testing.assert_allclose(res.cpu().numpy(), ref_res, rtol=1e-10, atol=1e-12)
    ref_mask = np.broadcast_to(ref_mask[:, None], ref_res.shape)
    np.testing.assert_array_equal(mask.cpu().numpy(), ref_mask)


def test_cg_solves_metric_system_like_scipy(cuda, small_response):
    inst, rd, ref = small_response
    R = rd["R"]
    lam = R.flat(inst.sky).cpu().numpy()
    data = synthetic.poisson_data(lam, 3)
    lh = ju.Poissonian(ju.Vector({"tm1": data[:R.plan.readout_sizes[0]],
                                  "tm2": data[R.plan.readout_sizes[0]:]})).amend(R)
    x = torch.as_tensor(inst.sky, device=cuda)
    lh.energy_and_gradient(x)
    rng = np.random.default_rng(3)
    j = torch.as_tensor(rng.normal(size=inst.sky.shape), device=cuda)
    mat = lambda v: lh.metric(None, v) + v
    sol, info = minimization.conjugate_gradient(mat, j, tol=1e-10, maxiter=500)
    n = inst.sky.size

    def ref_mat(v):
        v = v.reshape(inst.sky.shape)
        return (ref.metric(inst.sky, v) + v).reshape(-1)

    op = LinearOperator((n, n), matvec=ref_mat)
    try:
        xs, st = scipy_cg(op, j.cpu().numpy().reshape(-1), rtol=1e-12, maxiter=2000)
    except TypeError:  # scipy before 1.12 names the tolerance tol
        xs, st = scipy_cg(op, j.cpu().numpy().reshape(-1), tol=1e-12, maxiter=2000)
    assert st == 0
    np.testing.assert_allclose(sol.cpu().numpy().reshape(-1), xs, rtol=1e-7, atol=1e-9)
    assert info["residual_norm"] <= 1e-10 * float(torch.linalg.norm(j)) * 1.0001
    # the same iteration through the oracle's CG restatement
    xo, it = CO.conjugate_gradient(lambda v: ref_mat(v), j.cpu().numpy().reshape(-1), tol=1e-10)
    assert abs(it - info["iterations"]) <= 2


def test_draw_linear_sample(cuda, small_response):
    inst, rd, ref = small_response
    R = rd["R"]
    lam = R.flat(inst.sky).cpu().numpy()
    data = synthetic.poisson_data(lam, 4)
    s0 = R.plan.readout_sizes[0]
    lh = ju.Poissonian(ju.Vector({"tm1": data[:s0], "tm2": data[s0:]})).amend(R)
    x = torch.as_tensor(inst.sky, device=cuda)
    s, info = minimization.draw_linear_sample(lh, x, seed=10, tol=1e-8, maxiter=300)
    assert s.shape == x.shape and info["iterations"] > 0
    # (M + 1) s reproduces the right-hand side built from the same draws
    lamd = R.plan.response(x)
    xi_d = sampling.random_normal(lamd.shape, lamd.dtype, seed=10, offset=0)
    xi_x = sampling.random_normal(x.shape, x.dtype, seed=10, offset=1)
    z = R.plan.response_vjp(xi_d / torch.sqrt(lamd)) + xi_x
    lhs = R.plan.metric(None, s) + s
    assert float(torch.linalg.norm(lhs - z) / torch.linalg.norm(z)) < 1e-7
    s2, _ = minimization.draw_linear_sample(lh, x, seed=10, tol=1e-8, maxiter=300)
    assert torch.allclose(s, s2, rtol=1e-12, atol=0)
