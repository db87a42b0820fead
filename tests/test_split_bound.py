"""The error bound behind the plain method on the tensor cores, checked on the
CPU: with x = hi + lo (hi = bf16(x), lo = bf16(x - hi), both round to
nearest even), hi.hi + lo.hi + hi.lo differs from x.q by at most
3.05 * 2^-16 * |x| |q| (the pieces left out: lo.lo, and each operand's
remainder below 2^-16 |x|).  The scan's completeness check adds the FP32
accumulation allowance on top of this constant."""
import numpy as np

C_SPLIT = 3.05 * 2.0 ** -16


def bf16_rne(a: np.ndarray) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def split(a: np.ndarray):
    hi = bf16_rne(a)
    lo = bf16_rne((a - hi).astype(np.float32))
    return hi, lo


def worst_ratio(X: np.ndarray, Q: np.ndarray) -> float:
    xh, xl = split(X)
    qh, ql = split(Q)
    f = np.float64
    approx = xh.astype(f) @ qh.astype(f).T + xl.astype(f) @ qh.astype(f).T + xh.astype(f) @ ql.astype(f).T
    exact = X.astype(f) @ Q.astype(f).T
    scale = np.linalg.norm(X.astype(f), axis=1)[:, None] * np.linalg.norm(Q.astype(f), axis=1)[None, :]
    return float(np.max(np.abs(approx - exact) / np.maximum(scale, 1e-300)))


def test_bf16_rounding_matches_known_values():
    v = np.float32([1.0, 1.00390625, 1.005859375, 3.0e-3, -2.5, 65504.0])
    r = bf16_rne(v)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa -> 1
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0078125)
    assert r[4] == -2.5
    # half an 8-bit ulp: at most 2^-8 of the value
    assert abs(float(r[3]) - 3.0e-3) <= 2.0 ** -8 * 3.0e-3
    hi, lo = split(v)
    assert np.all(np.abs((hi.astype(np.float64) + lo) - v) <= 2.0 ** -16 * np.abs(v))


def test_split_product_bound_gaussian():
    rng = np.random.default_rng(5)
    for d in (8, 33, 96, 128):
        X = rng.standard_normal((400, d), dtype=np.float32)
        Q = rng.standard_normal((50, d), dtype=np.float32)
        assert worst_ratio(X, Q) <= C_SPLIT


def test_split_product_bound_wide_magnitudes():
    # log-normal magnitudes over many binades, signs mixed, and rows whose
    # elements sit just below rounding ties
    rng = np.random.default_rng(6)
    d = 128
    X = (rng.lognormal(0.0, 3.0, (300, d)) * rng.choice([-1.0, 1.0], (300, d))).astype(np.float32)
    Q = (rng.lognormal(0.0, 3.0, (40, d)) * rng.choice([-1.0, 1.0], (40, d))).astype(np.float32)
    assert worst_ratio(X, Q) <= C_SPLIT
    base = rng.integers(1, 255, size=(64, d)).astype(np.float32) * 2.0 ** -7 + 1.0
    near_tie = (base + np.float32(2.0 ** -9) - np.float32(2.0 ** -24)).astype(np.float32)
    assert worst_ratio(near_tie, near_tie[:16]) <= C_SPLIT


def test_split_bound_is_not_loose_by_orders_of_magnitude():
    # the constant is a bound, not a guess: with every element of one sign
    # and its remainders pushed to the same side, the observed ratio comes
    # within a factor of 5 of it
    rng = np.random.default_rng(7)
    s = np.float32(2.0 ** -9 * 0.999)
    X = (np.float32(1.0) + s + rng.integers(0, 2**8, size=(200, 96)) * 2.0 ** -17).astype(np.float32)
    r = worst_ratio(X, X[:20])
    assert C_SPLIT / 5 <= r <= C_SPLIT
