"""The exact two-word accumulation of the fused kernels, restated in numpy on
the CPU (no GPU): terms split as hi (multiple of Q1) + lo (multiple of Q2) add
to the same bits in every order, and hi + lo is within 2^L * Q2 / 2 of the
exact sum.  The device code is ``Split2`` in ``j-ubik_gb300/csrc/fused.cu``;
this restatement checks the arithmetic those kernels rely on."""
import math

import numpy as np
import pytest


def split2_constants(bound, L, D):
    e = math.frexp(bound)[1]  # bound < 2^e
    q1 = e - (D - 2)
    q2 = q1 + L + 1 - D
    return math.ldexp(1.5, q1 + D - 1), math.ldexp(1.5, q2 + D - 1), q1, q2


@pytest.mark.parametrize("dt, D", [(np.float32, 24), (np.float64, 53)])
@pytest.mark.parametrize("L", [2, 4, 6])
def test_two_word_sums_are_order_independent_and_near_exact(dt, D, L):
    rng = np.random.default_rng(L)
    n_terms, n_el = 2 ** L, 4096
    # terms of mixed signs over many decades, each partial sum below the bound
    mag = 10.0 ** rng.uniform(-9, 0, size=(n_terms, n_el))
    v = (rng.choice([-1.0, 1.0], size=mag.shape) * mag / n_terms).astype(dt)
    bound = 1.0
    m1, m2, q1, q2 = split2_constants(bound, L, D)
    m1, m2 = dt(m1), dt(m2)
    hi = (v + m1) - m1
    lo = ((v - hi) + m2) - m2
    assert np.all(np.mod(hi.astype(np.float64), 2.0 ** q1) == 0)
    assert np.all(np.mod(lo.astype(np.float64), 2.0 ** q2) == 0)
    sums = []
    for trial in range(6):
        order = rng.permutation(n_terms)
        sh = np.zeros(n_el, dt)
        sl = np.zeros(n_el, dt)
        for t in order:  # one rounding per addition, as a reduction performs it
            sh = (sh + hi[t]).astype(dt)
            sl = (sl + lo[t]).astype(dt)
        sums.append((sh + sl).astype(dt))
    for s in sums[1:]:
        assert np.array_equal(s.view(np.uint8), sums[0].view(np.uint8))
    # the exact sum, correctly rounded to float64 (fsum)
    exact = np.array([math.fsum(col) for col in v.astype(np.float64).T])
    err = np.abs(sums[0].astype(np.float64) - exact)
    # quantisation of the lo words, plus the final rounding of hi + lo (and, in
    # float64, the rounding of the reference itself)
    assert np.all(err <= n_terms * 2.0 ** q2 / 2 + 2 * np.abs(exact) * np.finfo(dt).eps)
    # the lo quantisation sits far below the result's own last bit: most
    # elements are the exact sum rounded once, the rest one ulp away
    assert np.mean(sums[0] == exact.astype(dt)) > 0.9


def test_split_of_a_nan_bound_poisons_every_term():
    m1 = np.float32(np.nan)
    v = np.float32(1.0)
    assert np.isnan((v + m1) - m1)
