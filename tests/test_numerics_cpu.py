"""CPU checks of the exact FP64 rewrites used by the GPU decision path, independent of
CUDA: Python floats are IEEE binary64 with correctly rounded +, *, /, and Fraction gives
the exact products and sums a fused multiply-add rounds once."""
from fractions import Fraction
import random
import struct

import numpy as np


def fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def div_by(a, b, y):
    """q = a y, r = a - b q exactly, RN(q + r y) (Markstein 1990)."""
    q = a * y
    r = fma(-b, q, a)
    return fma(r, y, q)


def test_division_by_known_reciprocal_is_correctly_rounded():
    rng = random.Random(5)
    cases = []
    for _ in range(6000):   # wide exponents
        a = rng.uniform(1, 2) * 2.0 ** rng.randint(-60, 60) * rng.choice([1, -1])
        b = rng.uniform(1, 2) * 2.0 ** rng.randint(-60, 60)
        cases.append((a, b))
    for _ in range(6000):   # move counters over integer tF / num_states
        cases.append((float(rng.randint(1, 2 ** 40)), float(rng.randint(1, 2 ** rng.randint(1, 40)))))
    for _ in range(6000):   # the SAD extrapolation (e - too_lo) / min_T
        cases.append((-300.0 * rng.random(), 0.01 + 2.0 * rng.random()))
    for _ in range(2000):   # divisors with near-all-ones / near-zero mantissas
        m = rng.getrandbits(12)
        bits = ((1023 + rng.randint(-20, 20)) << 52) | ((0xFFFFFFFFFFFFF ^ m) if rng.random() < 0.5 else m)
        cases.append((rng.uniform(-1e6, 1e6), struct.unpack("<d", struct.pack("<Q", bits))[0]))
    bad = [(a, b) for a, b in cases if div_by(a, b, 1.0 / b) != a / b]
    assert not bad, bad[:5]


def test_float_to_double_by_bits():
    """The integer float-to-double conversion of the GPU decision path, restated."""
    def f2d(f32):
        b = int(np.float32(f32).view(np.uint32))
        e = (b >> 23) & 0xFF
        if e == 0 and (b & 0x7FFFFFFF) == 0:
            return struct.unpack("<d", struct.pack("<Q", (b & 0x80000000) << 32))[0]
        if e in (0, 255):
            return float(np.float32(f32))
        d = ((b >> 31) << 63) | ((e + 1023 - 127) << 52) | ((b & 0x7FFFFF) << 29)
        return struct.unpack("<d", struct.pack("<Q", d))[0]
    rng = np.random.default_rng(2)
    for bits in rng.integers(0, 2 ** 32, 20000, dtype=np.uint64):
        f = np.uint32(bits).view(np.float32)
        if np.isnan(f):
            continue
        assert f2d(f) == float(f) and np.signbit(f2d(f)) == np.signbit(f)


def _trunc32(x):
    """binary32 value of float64 x with its mantissa truncated toward zero (f32_trunc)."""
    f = x.astype(np.float32)
    over = np.abs(f.astype(np.float64)) > np.abs(x)
    f[over] = np.nextafter(f[over], np.float32(0))
    return f


def test_log_space_metropolis_bounds_never_contradict_the_fp64_test():
    """The single-walker fast path decides rejected = lnw2 > lnw1 && u > exp(lnw1 - lnw2)
    (energy.rs:461-465) on binary32 truncations a, b of the weights, an error bound dd of
    a - b and bounds [lo, hi] of ln u, and falls back to FP64 only in between.  Whatever
    the bounds call sure must agree with the FP64 test, and they should call nearly every
    case.  binary32 arithmetic here is numpy's IEEE single (the kernels build with
    -fmad=false, so no contraction); logf's 1-ulp error is covered by the 2^-20 widening."""
    rng = np.random.default_rng(17)
    n = 1_000_000
    lnw1 = rng.uniform(0.0, 3000.0, n)
    gap = np.exp(rng.uniform(np.log(1e-12), np.log(60.0), n))
    sign = np.where(rng.random(n) < 0.8, 1.0, -1.0)        # mostly uphill, some downhill
    lnw2 = lnw1 + sign * gap
    same = rng.random(n) < 0.02                             # equal weights
    lnw2[same] = lnw1[same]
    u53 = rng.integers(0, 2 ** 53, n, dtype=np.uint64)
    u53[: n // 50] = rng.integers(0, 2 ** 24, n // 50, dtype=np.uint64)  # tiny uniforms
    u53[n // 50: n // 25] = np.uint64(2 ** 53 - 1) - rng.integers(0, 2 ** 30, n // 50, dtype=np.uint64)
    # the fast path's binary32 quantities
    a, b = _trunc32(lnw1), _trunc32(lnw2)
    df = (a - b).astype(np.float32)
    dd = ((np.abs(a) + np.abs(b)) * np.float32(1.2e-7) + np.abs(df) * np.float32(6.0e-8)
          + np.float32(1e-12)).astype(np.float32)
    top = (u53 >> np.uint64(29)).astype(np.float64)
    uf = (top * 2.0 ** -24).astype(np.float32)
    uh = ((top + 1.0) * 2.0 ** -24).astype(np.float32)
    with np.errstate(divide="ignore"):
        lo = np.where(top == 0, np.float32(-np.inf), np.log(uf) * np.float32(1.0 + 9.6e-7)).astype(np.float32)
    hi = (np.log(uh) * np.float32(1.0 - 9.6e-7)).astype(np.float32)
    acc_sure = (b < a) | (hi < df - dd)
    rej_sure = (b > a) & (lo > df + dd)
    # the reference's FP64 test
    u = u53.astype(np.float64) * 2.0 ** -53
    exact_rej = (lnw2 > lnw1) & (u > np.exp(lnw1 - lnw2))
    assert not (acc_sure & rej_sure).any()
    assert not (acc_sure & exact_rej).any(), np.flatnonzero(acc_sure & exact_rej)[:5]
    assert not (rej_sure & ~exact_rej).any(), np.flatnonzero(rej_sure & ~exact_rej)[:5]
    # the sample is deliberately hard (log-uniform gaps down to 1e-12, 2 % equal weights,
    # uniforms at both ends); the FP64 test still decides fewer than 2 % of the cases
    assert (acc_sure | rej_sure).mean() > 0.98


def test_integer_window_thresholds():
    """x < T <=> x < ceil(T) and x > T <=> x > floor(T) for integer x: the single-walker
    fast path compares Ising energies with the SAD window edges and energy bounds this way."""
    rng = np.random.default_rng(3)
    T = np.concatenate([rng.integers(-3000, 3000, 20000).astype(np.float64),
                        rng.integers(-3000, 3000, 20000) + 0.5,
                        rng.uniform(-3000, 3000, 20000)])
    x = rng.integers(-3010, 3010, T.size).astype(np.float64)
    assert np.array_equal(x < T, x < np.ceil(T))
    assert np.array_equal(x > T, x > np.floor(T))
