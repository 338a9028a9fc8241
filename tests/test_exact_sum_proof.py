"""The proof rules of the exact Neumaier sums (``ExactSum`` in
``ndfiltrs_gb300/csrc/common.cuh``) restated with Python integers and checked
against the sequential Neumaier sum (Sum64, the reference's
``src/mean.rs:7-26``).

The device code sums terms exactly in 192-bit fixed point (lowest bit
2^(H - 158), magnitudes truncated toward zero) and returns a value only when
one of two rules proves it equal to the sequential sum:

* every term a multiple of 2^Q with Q >= 2k + H - 105 (n < 2^k terms): the
  correction sum is exact and the result is RN(S);
* otherwise both ends of [S - E, S + E], E = 2^(3k + 55) units, round to the
  same double.

These tests check that no proven value differs from the sequential sum, over
random families and over sums built so that Neumaier's result is not the
correctly rounded sum; the GPU parity tests check the device code itself.
"""

from __future__ import annotations

import math
import random
import struct
from fractions import Fraction


def _bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def neumaier(terms) -> float:
    value = correction = 0.0
    for x in terms:
        total = value + x
        if abs(value) >= abs(x):
            correction += (value - total) + x
        else:
            correction += (x - total) + value
        value = total
    return value + correction


def bound_exponent(x: float) -> int:
    """Smallest H with |x| < 2^H (the device's bound_exponent)."""
    if x == 0.0:
        return -1022
    _, e = math.frexp(abs(x))
    return max(e, -1022)


def _rn(units: int, low_bit: int) -> float | None:
    if units == 0:
        return None
    value = float(Fraction(units) * Fraction(2) ** low_bit)
    if value == 0.0 or math.isinf(value) or abs(value) < 2.2250738585072014e-308:
        return None
    return value


def proven_sum(terms, H: int) -> float | None:
    n = len(terms)
    k = n.bit_length()
    if n < 1 or k + H > 1000:
        return None
    L = H - 158
    total = 0
    low = None
    for x in terms:
        if math.isnan(x) or math.isinf(x):
            return None
        if x == 0.0:
            continue
        m, e = math.frexp(abs(x))
        mant, q = int(m * 2**53), e - 53
        while mant % 2 == 0:
            mant //= 2
            q += 1
        if abs(x) >= 2.0**H:
            return None
        low = q if low is None else min(low, q)
        units = mant << (q - L) if q >= L else mant >> (L - q)
        total += -units if x < 0 else units
    if low is None or low >= 2 * k + H - 105:
        if total == 0:
            return 0.0
        return _rn(total, L)
    reach = 2 ** (3 * k + 55)
    a, b = _rn(total - reach, L), _rn(total + reach, L)
    if a is None or b is None or _bits(a) != _bits(b):
        return None
    return a


def _families(rng: random.Random):
    yield "float32 sky", [float(struct.unpack("<f", struct.pack("<f", 500 + 20 * rng.gauss(0, 1)))[0])
                         for _ in range(rng.randint(1, 600))]
    yield "float64 sky", [100 + 5 * rng.gauss(0, 1) for _ in range(rng.randint(1, 600))]
    yield "wide exponents", [rng.gauss(0, 1) * 2.0 ** rng.randint(-100, 100) for _ in range(rng.randint(1, 200))]
    yield "cancelling powers", [rng.choice((-1, 1)) * 2.0 ** rng.randint(0, 60) for _ in range(rng.randint(1, 200))]
    yield "squares", sorted(min(1.0, (rng.gauss(0, 1) / 4) ** 2) for _ in range(rng.randint(1, 600)))
    yield "big and small", [rng.choice((-1, 1)) * (1 + rng.random()) * 2.0**60 if rng.random() < 0.3
                            else rng.gauss(0, 1) * 2.0 ** rng.randint(-20, 20) for _ in range(rng.randint(1, 200))]


def test_proven_sums_equal_the_sequential_sum() -> None:
    rng = random.Random(7)
    proven = fallback = 0
    for _ in range(400):
        for name, terms in _families(rng):
            peak = max(abs(x) for x in terms)
            value = proven_sum(terms, bound_exponent(peak))
            if value is None:
                fallback += 1
                continue
            proven += 1
            assert _bits(value) == _bits(neumaier(terms)), (name, terms)
    assert fallback <= proven // 100


def test_sums_neumaier_does_not_round_correctly_are_never_misproven() -> None:
    # A power of two 2^e, then odd multiples of 2^(e - 53) (each addition
    # a tie or a rounding of the running sum) and tiny terms that the
    # correction sum drops: Neumaier then misses the correctly rounded sum.
    rng = random.Random(11)
    not_rounded = 0
    for _ in range(3000):
        e = rng.randint(20, 80)
        terms = [2.0**e]
        terms += [float((1 + 2 * rng.randint(0, 3)) * 2.0 ** (e - 53 - rng.randint(0, 2)))
                  for _ in range(rng.randint(1, 20))]
        terms += [rng.choice((-1.0, 1.0)) * 2.0 ** (e - 58 - rng.randint(0, 60)) for _ in range(rng.randint(0, 3))]
        exact = float(sum(Fraction(x) for x in terms))
        sequential = neumaier(terms)
        not_rounded += _bits(exact) != _bits(sequential)
        value = proven_sum(terms, bound_exponent(max(abs(x) for x in terms)))
        if value is not None:
            assert _bits(value) == _bits(sequential)
    assert not_rounded > 0
