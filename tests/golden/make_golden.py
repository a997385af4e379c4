"""Generate the small golden fixtures of tests/golden/{slice36,linpatch48,response32}.npz.

These freeze the float64 oracle's outputs on seeded inputs, including the
composed response and Poisson energy that the reference's patch files do not
compute on their own.  The oracle itself is pinned to the reference's code by
the fixtures of ``make_ref_fixtures.py`` (outputs of the reference's own
``convolve.py`` / ``response.py`` / ``utils.py``) and by the reference's
known-answer tests (tests/test_oracle_pins.py).
Run: ``python tests/golden/make_golden.py``.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import jubik_oracle as O  # noqa: E402


def slice36():
    x = np.arange(36 * 36, dtype=float).reshape(36, 36)
    s = O.slice_patches(x, (36, 36), 16, 2)
    return {"x": x, "patches": s, "adjoint": O.slice_patches_adjoint(s, (36, 36), 16, 2)}


def linpatch48():
    rng = np.random.default_rng(7)
    E, N, n, m = 2, 48, 3, 8
    dx = N // n
    x = rng.random((E, N, N))
    ker = rng.random((n * n, E, 2 * dx, 2 * dx))
    dom = O.Domain((E, N, N), (1.0, 0.5, 0.5))
    g = rng.normal(size=(E, N, N))
    return {"x": x, "kernel": ker, "cot": g,
            "y": O.linpatch_convolve(x, dom, ker, n, m, precut=True),
            "xt": O.linpatch_convolve_adjoint(g, dom, ker, n, m, precut=True)}


def response32():
    rng = np.random.default_rng(11)
    M, E, N, n, m = 2, 1, 32, 2, 4
    dx = N // n
    dom = O.Domain((E, N, N), (1.0, 1.0, 1.0))
    ker = rng.random((M, n * n, E, 2 * dx, 2 * dx))
    exp = rng.uniform(500, 1500, size=(M, E, N, N))
    rm = rng.random((M, E, N, N)) > 0.1
    R = O.Response(dom, ker, n, m, exp, rm, pixel_area=0.25)
    x = np.exp(rng.normal(size=(E, N, N)))
    lam = R(x)
    data = [rng.poisson(l) for l in lam]
    e, g = R.energy_and_grad(x, data)
    return {"kernel": ker, "exposure": exp, "readmask": rm, "x": x,
            "lam": np.concatenate(lam), "data": np.concatenate(data),
            "energy": np.array(e), "grad": g}


CASES = {"slice36": slice36, "linpatch48": linpatch48, "response32": response32}

if __name__ == "__main__":
    for name, fn in CASES.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **fn())
        print("wrote", name)
