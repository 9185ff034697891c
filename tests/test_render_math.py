"""The render pass evaluates the reference's `prev + (cur - prev) * 0.25` (float
operands, product and sum in double, stored as float; game.cpp:2041-2042) in float
for normal operands. These CPU checks confirm the two evaluations agree, with
numpy's IEEE float32/float64 arithmetic, on random operands of every magnitude."""
import numpy as np


def _double_path(prev, cur):
    d = (cur - prev).astype(np.float32)
    return (prev.astype(np.float64) + d.astype(np.float64) * 0.25).astype(np.float32)


def _float_path(prev, cur):
    d = (cur - prev).astype(np.float32)
    return (prev + d * np.float32(0.25)).astype(np.float32)


def _rand_floats(rng, n, lo, hi):
    mant = rng.uniform(1.0, 2.0, n)
    exp = rng.integers(lo, hi, n)
    sign = rng.choice([-1.0, 1.0], n)
    return (sign * mant * np.exp2(exp.astype(np.float64))).astype(np.float32)


def test_smoothing_float_equals_double_for_normal_operands():
    rng = np.random.default_rng(7)
    n = 2_000_000
    for lo, hi in ((-30, 10), (-119, 120), (-5, 5)):
        prev = _rand_floats(rng, n, lo, hi)
        cur = _rand_floats(rng, n, lo, hi)
        # the flows a world produces: multiples of 2^-16
        cur[::3] = (np.round(cur[::3].astype(np.float64) * 65536.0) / 65536.0).astype(np.float32)
        d = (cur - prev).astype(np.float32)
        ok = ((np.abs(prev) >= 2.0 ** -120) | (prev == 0)) & ((np.abs(d) >= 2.0 ** -120) | (d == 0))
        ok &= np.isfinite(d)
        a, b = _double_path(prev[ok], cur[ok]), _float_path(prev[ok], cur[ok])
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_decay_towards_zero_stays_on_the_double_path():
    # with no new flow the smoothed value decays by 3/4 per pass and reaches the
    # subnormal range, where only the double evaluation is the reference's
    v = np.float32(1.0)
    for _ in range(400):
        v = _double_path(np.array([v], np.float32), np.array([0.0], np.float32))[0]
    assert 0 < abs(v) < 2.0 ** -126 or v == 0
