"""Freeze outputs of J-UBIK's own code as fixtures: ``tests/golden/ref_*.npz``.

Loads the reference's ``jubik/convolve.py``, ``jubik/response.py`` and
``jubik/utils.py`` unmodified through the numpy-backed JAX / NIFTy.re
stand-in of ``reference_standin.py``, checks the stand-in by running the
reference's own tests for these files through it, then evaluates seeded
small cases and writes inputs and outputs.  The VJP of ``linpatch_convolve``
(what ``jax.vjp`` returns) is the transposed Jacobian, assembled column by
column from the reference's forward at small sizes.

Run in a checkout that holds the reference sources:
``python tests/golden/make_ref_fixtures.py [reference root]``.  The fixtures
travel with the repository; nothing at test time reads the reference.
"""
from __future__ import annotations

import io
import os
import sys
from contextlib import redirect_stdout

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import reference_standin  # noqa: E402

REF_TESTS = ["test_convolve.py", "test_slice_patches.py", "test_build_exposure_function.py",
             "test_build_exposure_readout_function.py",
             "test_utils.py::test_coord_center_small_grid"]


def run_reference_tests(root) -> str:
    """The reference's own tests of these files, through the stand-in."""
    import pytest

    class _Standin:
        def pytest_configure(self, config):
            reference_standin.load_reference(root)

    sys.dont_write_bytecode = True
    tdir = os.path.join(root, "test")
    args = ["-q", "-p", "no:cacheprovider", "-c", os.devnull, "--rootdir", tdir]
    args += [os.path.join(tdir, t) for t in REF_TESTS]
    out = io.StringIO()
    with redirect_stdout(out):
        rc = pytest.main(args, plugins=[_Standin()])
    summary = [ln for ln in out.getvalue().splitlines() if "passed" in ln or "failed" in ln]
    if rc != 0:
        raise SystemExit("the reference's tests fail through the stand-in:\n" + out.getvalue())
    return summary[-1].strip("= ")


def grid(a, bits=10):
    """Values rounded to multiples of 2**-bits (exact in float64; compress well)."""
    return np.round(np.asarray(a) * 2.0 ** bits) / 2.0 ** bits


def slice_cases(ju):
    out = {}
    cases = {  # name: (x shape, n, dr)
        "s36": ((36, 36), 16, 2),            # the reference's own test geometry
        "s40e": ((2, 40, 40), 4, 3),         # a leading energy axis
        "s45c": ((1, 45, 45), 3, 0),         # odd stride 15: clamped last start
        "s45m": ((1, 45 + 10, 45 + 10), 3, 5),  # the same with a margin (overlap-add form)
        "s24": ((24, 24), 3, 4),
    }
    for name, (shape, n, dr) in cases.items():
        x = np.arange(int(np.prod(shape)), dtype=float).reshape(shape)
        p = np.asarray(ju.slice_patches(x, shape, n, dr))
        import jax  # the stand-in
        (adj,) = jax.linear_transpose(lambda a: ju.slice_patches(a, shape, n, dr), x)(p)
        out[name] = {"x": x, "n": n, "dr": dr, "patches": p, "adjoint": np.asarray(adj)}
    return out


def _linpatch_vjp(ju, dom, kernel, n, m, g):
    """Transpose of the reference's linpatch_convolve in x, column by column."""
    shape = dom.shape
    size = int(np.prod(shape))
    out = np.empty(size)
    gflat = g.reshape(-1)
    basis = np.zeros(size)
    with redirect_stdout(io.StringIO()):  # the broadcast branch prints per call
        for j in range(size):
            basis[j] = 1.0
            col = np.asarray(ju.linpatch_convolve(basis.reshape(shape), dom, kernel, n, m))
            out[j] = np.dot(col.reshape(-1), gflat)
            basis[j] = 0.0
    return out.reshape(shape)


def linpatch_cases(ju):
    rng = np.random.default_rng(2026)
    out = {}
    cases = {  # name: (x shape, kernel shape kind, n, margin, distances, vjp)
        "l48": ((2, 48, 48), "full", 3, 8, (1.0, 0.5, 0.5), False),
        "l40": ((40, 40), "full", 4, 5, (1.0, 1.0), False),
        "l36b": ((2, 36, 36), "bcast", 3, 6, (1.0, 1.0, 1.0), False),
        "l30": ((1, 30, 30), "full", 5, 3, (1.0, 2.0, 2.0), False),
        "l64": ((1, 64, 64), "full", 4, 16, (1.0, 1.0, 1.0), False),
        "l24v": ((1, 24, 24), "full", 3, 4, (1.0, 1.0, 1.0), True),
        "l20v": ((2, 20, 20), "full", 4, 2, (1.0, 0.5, 0.5), True),
    }
    for name, (shape, kind, n, m, dist, vjp) in cases.items():
        N = shape[-1]
        E = shape[0] if len(shape) == 3 else None
        lead = () if (E is None or kind == "bcast") else (E,)
        # positive kernels with their origin at index (0, 0), wrapped around the
        # edges (the reference fftshifts them to the centre before the cut)
        yy, xx = np.meshgrid(np.arange(N) - N // 2, np.arange(N) - N // 2, indexing="ij")
        ker = np.empty((n * n,) + lead + (N, N))
        for idx in np.ndindex(ker.shape[:-2]):
            s = 1.0 + 2.0 * rng.random()
            ker[idx] = np.fft.ifftshift(np.exp(-0.5 * (yy ** 2 + (0.8 * xx) ** 2) / s ** 2) +
                                        0.01 * rng.random((N, N)))
        ker = grid(ker, 16)
        x = grid(rng.random(shape) + 0.25)
        dom = ju.Domain(shape, dist)
        buf = io.StringIO()
        with redirect_stdout(buf):
            y = np.asarray(ju.linpatch_convolve(x, dom, ker, n, m))
        case = {"x": x, "kernel": ker, "n": n, "margin": m, "distances": np.array(dist),
                "y": y, "printed": np.array(buf.getvalue())}
        if vjp:
            g = grid(rng.standard_normal(shape))
            case["cot"] = g
            case["xt"] = _linpatch_vjp(ju, dom, ker, n, m, g)
        out[name] = case
    return out


def convolve_cases(ju):
    rng = np.random.default_rng(7)
    out = {}
    k = np.zeros((4, 4))
    k[0, 0] = 1.0
    out["cid"] = {"x": k, "y": grid(rng.normal(size=(4, 4))), "axes": np.array([-2, -1]),
                  "distances": np.array([1.0, 1.0])}
    out["cb"] = {"x": k, "y": np.stack([np.ones((4, 4)), 2.0 * np.ones((4, 4))]),
                 "axes": np.array([-2, -1]), "distances": np.array([1.0, 1.0])}
    out["cr"] = {"x": grid(rng.random((3, 12, 10))), "y": grid(rng.random((3, 12, 10))),
                 "axes": np.array([-2, -1]), "distances": np.array([9.0, 0.5, 0.25])}
    out["c1"] = {"x": grid(rng.random((2, 16))), "y": grid(rng.random((2, 16))),
                 "axes": np.array([-1]), "distances": np.array([1.0, 0.5])}
    for c in out.values():
        dom = ju.Domain(c["y"].shape, tuple(c["distances"]))
        buf = io.StringIO()
        with redirect_stdout(buf):
            c["out"] = np.asarray(ju.convolve(c["x"], c["y"], dom, tuple(int(a) for a in c["axes"])))
        c["printed"] = np.array(buf.getvalue())
    return out


def response_cases(ju):
    rng = np.random.default_rng(11)
    M, E, N = 2, 3, 24
    exposures = grid(rng.uniform(0.0, 3e3, size=(M, E, N, N)), 4)
    x = grid(rng.random((M, E, N, N)) * 10.0)
    out = {}
    for name, cut in (("e0", None), ("e20", 20.0)):
        ex = exposures.copy()
        f = ju.build_exposure_function(ex, cut)
        out[name] = {"exposures": exposures, "cut": np.array(np.nan if cut is None else cut),
                     "x": x, "out": np.asarray(f(x)), "thresholded": ex}
    for name, thr, keys in (("r0", None, None), ("r500", 500.0, ("tm1", "tm2"))):
        flags = exposures.copy()
        fn = ju.build_readout_function(flags, thr, keys)
        vec = fn(x if keys is not None else x[:1])
        leaves = [np.asarray(v) for v in vec.tree.values()]
        out[name] = {"flags": exposures, "threshold": np.array(np.nan if thr is None else thr),
                     "x": x if keys is not None else x[:1],
                     "keys": np.array(list(vec.tree.keys())),
                     "values": np.concatenate(leaves), "sizes": np.array([len(v) for v in leaves]),
                     "thresholded": flags}
    return out


def coord_cases(ju):
    sizes = [(4, 2), (8, 2), (48, 3), (64, 4), (1024, 16), (36, 6)]
    return {"coord": {"args": np.array(sizes),
                      "out": np.stack([np.pad(np.asarray(ju.coord_center(a, b)), (0, 256 - b * b),
                                              constant_values=-1) for a, b in sizes])}}


def main(root):
    summary = run_reference_tests(root)
    ju = reference_standin.load_reference(root)
    groups = {"ref_slice": slice_cases(ju), "ref_linpatch": linpatch_cases(ju),
              "ref_convolve": convolve_cases(ju), "ref_response": response_cases(ju),
              "ref_utils": coord_cases(ju)}
    for fname, cases in groups.items():
        flat = {"standin_check": np.array(summary)}
        for cname, arrays in cases.items():
            for k, v in arrays.items():
                flat[f"{cname}/{k}"] = np.asarray(v)
        path = os.path.join(HERE, fname + ".npz")
        np.savez_compressed(path, **flat)
        print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KB)")
    print("stand-in check:", summary)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
