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


def _byte(f, k):
    a = (f.astype(np.float64) * k) * 0.25 + 0.5
    out = np.where(a >= 1.0, 255.0, np.floor(np.clip(a, 0.0, 1.0) * 255.0))
    return np.where(a > 0.0, out, 0.0).astype(np.int64)


def _key(f):
    u = np.asarray(f, np.float32).view(np.uint32).astype(np.uint64)
    return np.where(u & 0x80000000, (~u) & 0xFFFFFFFF, u | 0x80000000)


def _unkey(k):
    k = np.asarray(k, np.uint64)
    u = np.where(k & 0x80000000, k & 0x7FFFFFFF, (~k) & 0xFFFFFFFF).astype(np.uint32)
    return u.view(np.float32)


def _thresholds(k):
    lo = np.full(255, int(_key(np.float32(-np.inf))), np.uint64)
    hi = np.full(255, int(_key(np.float32(np.inf))), np.uint64)
    j = np.arange(1, 256)
    for _ in range(34):  # bisection on all 255 thresholds at once
        mid = lo + (hi - lo) // 2
        ge = _byte(_unkey(mid), k) >= j
        hi = np.where(ge, mid, hi)
        lo = np.where(ge, lo, mid + 1)
    return np.concatenate([[np.float32(-np.inf)], _unkey(lo)])


def test_flow_byte_from_thresholds_equals_double_evaluation():
    # the render pass looks the flow texel byte up in per-material thresholds
    # instead of evaluating the reference's double expression
    rng = np.random.default_rng(3)
    for iterations in (1, 3, 6, 7):
        k = 3.0 / iterations + 0.5
        thr = _thresholds(k)
        f = np.concatenate([_rand_floats(rng, 500_000, -12, 4), thr[1:], np.nextafter(thr[1:], np.float32(-np.inf)),
                            np.float32([0.0, -0.0, 1e30, -1e30, np.inf, -np.inf])]).astype(np.float32)
        f = f[np.isfinite(f) | np.isinf(f)]
        looked_up = np.searchsorted(thr, f, side="right") - 1
        assert np.array_equal(looked_up, _byte(f, k))
