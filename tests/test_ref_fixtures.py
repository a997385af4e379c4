"""The oracle against outputs of J-UBIK's own code (CPU, no GPU).

``tests/golden/ref_*.npz`` hold outputs of the reference's unmodified
``jubik/convolve.py``, ``jubik/response.py`` and ``jubik/utils.py``, evaluated
through a numpy-backed JAX stand-in that passes the reference's own tests for
those files (``tests/golden/make_ref_fixtures.py``).  These tests pin the
float64 oracle to them: slicing, readout and patch centres bit-exact,
convolutions to 1e-13.
"""
import os

import numpy as np
import pytest

import jubik_oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases(name):
    d = np.load(os.path.join(HERE, name + ".npz"))
    out = {}
    for k in d.files:
        if "/" in k:
            c, f = k.split("/", 1)
            out.setdefault(c, {})[f] = d[k]
    return out, str(d["standin_check"])


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def test_fixtures_record_the_standin_check():
    for name in ("ref_slice", "ref_linpatch", "ref_convolve", "ref_response", "ref_utils"):
        _, check = cases(name)
        assert "passed" in check and "failed" not in check


@pytest.mark.parametrize("case", sorted(cases("ref_slice")[0]))
def test_oracle_slice_patches_bit_exact(case):
    c = cases("ref_slice")[0][case]
    n, dr = int(c["n"]), int(c["dr"])
    p = O.slice_patches(c["x"], c["x"].shape, n, dr)
    assert p.shape == c["patches"].shape and np.array_equal(p, c["patches"])
    a = O.slice_patches_adjoint(c["patches"], c["x"].shape, n, dr)
    assert np.array_equal(a, c["adjoint"])


@pytest.mark.parametrize("case", sorted(cases("ref_linpatch")[0]))
def test_oracle_linpatch_matches_reference(case, capsys):
    c = cases("ref_linpatch")[0][case]
    dom = O.Domain(c["x"].shape, tuple(c["distances"]))
    n, m = int(c["n"]), int(c["margin"])
    y = O.linpatch_convolve(c["x"], dom, c["kernel"], n, m)
    assert rel(y, c["y"]) < 1e-13
    if "xt" in c:
        xt = O.linpatch_convolve_adjoint(c["cot"], dom, c["kernel"], n, m)
        assert rel(xt, c["xt"]) < 1e-12


@pytest.mark.parametrize("case", sorted(cases("ref_convolve")[0]))
def test_oracle_convolve_matches_reference(case, capsys):
    c = cases("ref_convolve")[0][case]
    dom = O.Domain(c["y"].shape, tuple(c["distances"]))
    out = O.convolve(c["x"], c["y"], dom, tuple(int(a) for a in c["axes"]))
    assert out.shape == c["out"].shape
    assert np.max(np.abs(out - c["out"])) <= 1e-13 * max(1.0, np.max(np.abs(c["out"])))
    assert capsys.readouterr().out == str(c["printed"])


def test_oracle_exposure_and_readout_bit_exact():
    cs = cases("ref_response")[0]
    for name in ("e0", "e20"):
        c = cs[name]
        ex = c["exposures"].copy()
        cut = None if np.isnan(c["cut"]) else float(c["cut"])
        out = O.build_exposure_function(ex, cut)(c["x"])
        assert np.array_equal(out, c["out"]) and np.array_equal(ex, c["thresholded"])
    for name in ("r0", "r500"):
        c = cs[name]
        flags = c["flags"].copy()
        thr = None if np.isnan(c["threshold"]) else float(c["threshold"])
        keys = None if name == "r0" else tuple(str(k) for k in c["keys"])
        vec = O.build_readout_function(flags, thr, keys)(c["x"])
        tree = vec.tree if hasattr(vec, "tree") else vec
        assert [str(k) for k in tree] == [str(k) for k in c["keys"]]
        assert np.array_equal(np.concatenate([np.asarray(v) for v in tree.values()]), c["values"])
        assert np.array_equal(flags, c["thresholded"])


def test_oracle_coord_center_matches_reference():
    c = cases("ref_utils")[0]["coord"]
    for (a, b), row in zip(c["args"], c["out"]):
        assert np.array_equal(O.coord_center(int(a), int(b)), row[: b * b])


def test_package_coord_center_matches_reference():
    import jubik_gb300 as ju

    c = cases("ref_utils")[0]["coord"]
    for (a, b), row in zip(c["args"], c["out"]):
        assert np.array_equal(ju.coord_center(int(a), int(b)), row[: b * b])
