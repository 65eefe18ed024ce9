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
