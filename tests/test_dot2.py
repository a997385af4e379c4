"""The FP32 dot product's per-thread algorithm, restated on the CPU.

FP32 operands of ``jubik_dot`` are summed by each thread with the compensated
dot product "Dot2" (Ogita, Rump & Oishi, SIAM J. Sci. Comput. 26, 2005): each
product split exactly into p + e with p = fl(xy) and e = fma(x, y, -p), p added
with Knuth's TwoSum, and the error terms gathered in a second word.  Here the
same operations run in numpy float32 (an FP32 product is exact in float64, so
fma(x, y, -p) is (x*y - p) in float64, rounded once): the two words hold a
group's sum to about 2^-48 of its terms.
"""
import math

import numpy as np

f32 = np.float32


def dot2_words(x, y):
    """(s, c) of one thread's group: s + c is the compensated sum of x * y."""
    s = f32(0.0)
    c = f32(0.0)
    for a, b in zip(x.astype(f32), y.astype(f32)):
        p = f32(a * b)
        e = f32(np.float64(a) * np.float64(b) - np.float64(p))  # fma(a, b, -p), exact
        t = f32(s + p)
        bp = f32(t - s)
        sg = f32(f32(s - f32(t - bp)) + f32(p - bp))  # TwoSum's error of s + p
        s = t
        c = f32(c + f32(e + sg))
    return s, c


def exact_dot(x, y):
    return math.fsum((x.astype(np.float64) * y.astype(np.float64)).tolist())


def test_error_free_transformations():
    rng = np.random.default_rng(0)
    for _ in range(200):
        a, b = rng.normal(size=2).astype(f32)
        p = f32(a * b)
        e = f32(np.float64(a) * np.float64(b) - np.float64(p))
        assert np.float64(p) + np.float64(e) == np.float64(a) * np.float64(b)
        s, q = rng.normal(size=2).astype(f32) * f32(rng.uniform(1, 1e4))
        t = f32(s + q)
        bp = f32(t - s)
        sg = f32(f32(s - f32(t - bp)) + f32(q - bp))
        assert np.float64(t) + np.float64(sg) == np.float64(s) + np.float64(q)


def test_group_sum_to_2_to_minus_48_of_its_terms():
    rng = np.random.default_rng(1)
    for n in (1, 7, 128):
        for _ in range(20):
            x = rng.normal(size=n).astype(f32)
            y = rng.normal(size=n).astype(f32)
            s, c = dot2_words(x, y)
            got = np.float64(s) + np.float64(c)
            terms = float(np.abs(x.astype(np.float64) * y).sum())
            # Ogita-Rump-Oishi: |err| <= u |sum| + gamma_n^2 sum|xy|; the two words
            # are kept apart, so only the second term remains (u = 2^-24)
            gamma = n * 2.0 ** -24 / (1 - n * 2.0 ** -24)
            assert abs(got - exact_dot(x, y)) <= gamma ** 2 * terms + 1e-300


def test_cancellation_is_bounded_by_the_terms_not_the_result():
    rng = np.random.default_rng(2)
    x = rng.normal(size=64).astype(f32) * f32(1e3)
    y = rng.normal(size=64).astype(f32)
    xx = np.concatenate([x, -x])
    yy = np.concatenate([y, y])  # exact dot 0
    s, c = dot2_words(xx, yy)
    terms = float(np.abs(xx.astype(np.float64) * yy).sum())
    assert abs(np.float64(s) + np.float64(c)) <= 2.0 ** -44 * terms


def test_far_better_than_plain_fp32_accumulation():
    rng = np.random.default_rng(3)
    x = rng.normal(size=128).astype(f32)
    y = rng.normal(size=128).astype(f32)
    ref = exact_dot(x, y)
    s, c = dot2_words(x, y)
    naive = f32(0.0)
    for a, b in zip(x, y):
        naive = f32(naive + f32(a * b))
    assert abs(np.float64(s) + np.float64(c) - ref) * 1e4 < abs(float(naive) - ref) + 1e-12
