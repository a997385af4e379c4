"""Host-side logic of the drop-ins that runs before any GPU work (no GPU)."""
import numpy as np
import pytest

import jubik_gb300 as ju


def test_coord_center_matches_reference_known_answer():
    np.testing.assert_array_equal(ju.coord_center(4, 2), np.array([5, 13, 7, 15]))


def test_bilinear_weights_drop_in():
    w = ju._bilinear_weights((4, 4))
    assert w.shape == (4, 4) and np.all(w >= 0)
    np.testing.assert_allclose(w, w[::-1, :])
    with pytest.raises(ValueError):
        ju._bilinear_weights((3, 3))


def test_exposure_negative_cut_raises_before_gpu():
    with pytest.raises(ValueError):
        ju.build_exposure_function(np.ones((2, 4, 4)), -1)


def test_exposure_cut_is_applied_in_place():
    exp = np.array([[1.0, 5.0], [10.0, 0.5]])
    try:
        ju.build_exposure_function(exp, 2.0)
    except Exception:
        pass  # no GPU here: the in-place threshold happens first
    np.testing.assert_array_equal(exp, [[0.0, 5.0], [10.0, 0.0]])


def test_readout_validation_before_gpu():
    flags = np.ones((2, 3, 4, 4))
    with pytest.raises(ValueError):
        ju.build_readout_function(flags.copy(), -1, ("a", "b"))
    with pytest.raises(ValueError):
        ju.build_readout_function(flags.copy(), None, ("a",))
    f = ju.build_readout_function(np.ones((1, 4, 4)), None, ("a",))
    with pytest.raises(ValueError, match="flags should have shape"):
        f(np.ones((1, 2, 4, 4)))
    g = ju.build_readout_function(flags.copy(), None, ("a", "b"))
    with pytest.raises(ValueError, match="input should have shape"):
        g(np.ones((3, 4, 4)))


def test_readout_threshold_in_place():
    flags = np.array([[[[1.0, 30.0], [50.0, 5.0]]]])
    ju.build_readout_function(flags, 20, None)
    np.testing.assert_array_equal(flags, [[[[0.0, 30.0], [50.0, 0.0]]]])


def test_poissonian_rejects_float_data():
    with pytest.raises(TypeError):
        ju.Poissonian(np.array([1.0, 2.0]))


def test_vector_tree_interface():
    v = ju.Vector({"a": np.ones(2), "b": np.zeros(3)})
    assert list(v.keys()) == ["a", "b"]
    w = v * 2.0 + v
    np.testing.assert_array_equal(w.tree["a"], [3.0, 3.0])


def test_linpatch_domain_type_checked():
    with pytest.raises(ValueError, match="domain has to be"):
        ju.linpatch_convolve(np.ones((8, 8)), (8, 8), np.ones((4, 8, 8)), 2, 1)


def test_uneven_batch_geometry():
    from jubik_gb300 import synthetic
    geo = synthetic.config5_geometry()
    assert len(geo) == 64
    assert geo == synthetic.config5_geometry()  # seeded
    assert {g["P"] for g in geo} == {32, 64, 128}
    for g in geo:
        assert g["P"] == 2 * g["dx"] + 2 * g["margin"]
        assert g["nx"] == g["n"] * g["dx"] and 4 <= g["n"] <= 16
        assert g["dx"] % 2 == 0 and g["margin"] >= 3 * g["sigma"][1] - 1e-9
        assert 1 <= g["E"] <= 3 and 0.8 <= g["sigma"][1] <= 4.0
        assert 96 <= g["nx"] <= 1024


def test_problem_batch_needs_a_gpu_and_problems():
    if ju.plan.torch.cuda.is_available():
        pytest.skip("CUDA device present")
    with pytest.raises(ValueError):
        ju.ProblemBatch([])
    from jubik_gb300 import synthetic
    with pytest.raises(ju.JubikError):
        ju.ProblemBatch(synthetic.config5(count=1, max_side=160))


def test_kernel_cache_keys_distinguish_new_arrays():
    """The PSF-spectrum cache must not take a new kernel for an old one when
    memory or object identities are reused."""
    import torch
    from jubik_gb300.convolve import _kernel_key
    a = np.ones((4, 8, 8))
    ka, keep = _kernel_key(a)
    assert keep is a
    assert _kernel_key(a)[0] == ka                      # same object, same values
    b = a.copy()
    b[0, 0, 0] = 2.0
    assert _kernel_key(b)[0] != ka                      # a different array
    t = torch.ones(4, 8, 8)
    kt, _ = _kernel_key(t)
    t.mul_(2.0)                                         # in-place edit bumps the version
    assert _kernel_key(t)[0] != kt


def test_psf_snapshot_restore_logic():
    """Host logic of the PSF snapshots that autograd nodes keep (no GPU): a
    plan given another kernel re-applies the snapshot's kernel, and only then."""
    import torch
    from jubik_gb300.plan import PsfSnapshot, ResponsePlan

    plan = ResponsePlan.__new__(ResponsePlan)  # no device plan: record the uploads
    applied = []
    plan._set_psf = lambda psf, layout: applied.append((psf, layout))
    plan.psf_key, plan._psf = None, None
    ka, kb = torch.ones(3), torch.zeros(3)
    ResponsePlan.set_psf(plan, ka, "precut", key=("a",))
    snap_a = plan.psf_snapshot()
    ResponsePlan.set_psf(plan, kb, "precut", key=("b",))
    assert plan.psf_key == ("b",) and len(applied) == 2
    plan.restore_psf(snap_a)
    assert plan.psf_key == ("a",) and applied[-1][0] is ka and len(applied) == 3
    plan.restore_psf(snap_a)  # already held: nothing is uploaded
    assert len(applied) == 3
    # a callable source is evaluated when the snapshot is restored
    ResponsePlan.set_psf(plan, kb, "full", source=lambda: "again")
    snap_c = plan.psf_snapshot()
    ResponsePlan.set_psf(plan, ka, "precut")
    plan.restore_psf(snap_c)
    assert applied[-1] == ("again", "full")
    # an in-place edit of the watched tensor invalidates the snapshot
    w = torch.ones(2)
    s = PsfSnapshot(("w",), lambda: w, "precut", watch=w)
    w.add_(1.0)
    try:
        s.kernel()
    except RuntimeError as e:
        assert "modified in place" in str(e)
    else:
        raise AssertionError("expected RuntimeError")
