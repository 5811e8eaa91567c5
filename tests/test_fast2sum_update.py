"""The compensated update of the FP32 pair state, (hi + lo + inc) (1 - dp)
as a new (hi, lo) pair, restated in binary32 with numpy.

The step and tracer kernels (march.cu comp_damp, trc32.cu comp_update)
recover the update's two roundings by Fast2Sum (Dekker 1971).  That is
exact for s - c (c = s dp, 0 <= dp < 1).  It is exact for hi + inc wherever
|inc| <= |hi|, and elsewhere it is off by less than half an ulp of the
increment.  Checked here against TwoSum (Knuth), which is always exact, on
random operands covering both cases.
"""
import numpy as np

F = np.float32


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def _fast_two_sum(a, b):
    s = a + b
    return s, b - (s - a)


def _rng_operands(n, seed):
    rng = np.random.default_rng(seed)
    hi = (rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 2, n)).astype(F)
    # increments mostly far below the state, some comparable, some above it
    inc = (hi * rng.standard_normal(n).astype(F) * F(10.0) ** rng.uniform(-6, 1, n).astype(F)).astype(F)
    inc[: n // 10] = rng.standard_normal(n // 10).astype(F) * F(1e-3)  # states near zero
    hi[: n // 20] = F(0)
    dp = (10.0 ** rng.uniform(-7, -1, n)).astype(F)
    return hi, inc, dp


def test_fast2sum_of_the_increment_exact_where_it_is_below_the_state():
    with np.errstate(over='ignore', invalid='ignore'):
        hi, inc, _ = _rng_operands(200000, 1)
        s1, e1 = _two_sum(hi, inc)
        s2, e2 = _fast_two_sum(hi, inc)
    assert np.array_equal(s1, s2)
    below = np.abs(inc) <= np.abs(hi)
    assert below.sum() > 100000 and (~below).sum() > 10000
    assert np.array_equal(e1[below], e2[below])
    # elsewhere the error term is off by less than half an ulp of inc
    off = np.abs(e1[~below].astype(np.float64) - e2[~below].astype(np.float64))
    assert np.all(off <= 0.5 * np.spacing(np.abs(inc[~below])).astype(np.float64))


def test_fast2sum_of_the_damping_always_exact():
    hi, inc, dp = _rng_operands(200000, 2)
    s = hi + inc
    c = s * dp
    t1, e1 = _two_sum(s, -c)
    t = s - c
    e2 = (s - t) - c
    assert np.array_equal(t1, t) and np.array_equal(e1, e2)
    # the pair (t, e) is s - c exactly
    assert np.array_equal(t.astype(np.float64) + e2.astype(np.float64),
                          s.astype(np.float64) - c.astype(np.float64))
