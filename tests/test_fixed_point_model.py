"""The arithmetic of the fixed-point product form (QS_FIXED_POINT) restated
in exact Python integers, on the CPU: the scale choice never lets a row sum
overflow 64 bits, and every row sum stays within the documented bound
2^(2b - 61) max|x sqrt(stab)| of the exact value (b = ceil(log2(longest
row))).  The device kernels are compared with the oracle in
test_gpu_fixed_point.py; this pins the error model those tolerances rest on."""
import math
import struct
from fractions import Fraction

import numpy as np


def bits(v):
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def sqrt_exp(st):
    """ceil(log2(sqrt(st))): sqrt(st) <= 2^c."""
    lg = 0 if st == 1 else (st - 1).bit_length()
    return (lg + 1) >> 1


def bound_bits(v, st):
    """|v| times 2^c added in the exponent field: a bound of |v sqrt(st)|."""
    return (bits(v) & 0x7FFFFFFFFFFFFFFF) + (sqrt_exp(st) << 52)


def shift(maxbits, len_bits):
    e = maxbits >> 52
    return 62 - (max(e, 1) - 1022) - len_bits


def round_scaled(v, K):
    """round(v 2^K), ties to even."""
    return round(Fraction(v) * Fraction(2) ** K)   # Python's round: half to even


def test_scale_choice_and_error_bound():
    rng = np.random.default_rng(20261203)
    for trial in range(60):
        n = int(rng.integers(50, 400))
        stab = rng.choice([1, 2, 4, 8, 16, 32, 64, 128, 3, 6, 12, 24], size=n)
        scale = 2.0 ** int(rng.integers(-300, 300))
        x = rng.standard_normal(n) * scale
        if trial % 7 == 0:
            x[rng.integers(0, n, size=n // 3)] *= 1e-12     # a wide dynamic range
        xs = [float(np.float64(x[j]) * np.sqrt(np.float64(stab[j]))) for j in range(n)]  # the FP64 product x sqrt(stab)
        maxbits = max(bound_bits(float(x[j]), int(stab[j])) for j in range(n))
        assert maxbits < 0x7FF0000000000000
        rows, longest = [], 1
        for _ in range(40):
            ln = int(rng.integers(1, 70))
            longest = max(longest, ln)
            rows.append((rng.integers(0, n, size=ln), rng.integers(0, 2, size=ln)))
        b = (longest - 1).bit_length()
        K = shift(maxbits, b)
        q = [round_scaled(v, K) for v in xs]
        mx = max(abs(v) for v in xs)
        assert all(abs(v) <= 2 ** (62 - b) for v in q)
        for cols, signs in rows:
            total = sum(-q[c] if s else q[c] for c, s in zip(cols, signs))
            assert abs(total) < 2 ** 63                   # the int64 sum cannot overflow
            exact = sum(-Fraction(xs[c]) if s else Fraction(xs[c]) for c, s in zip(cols, signs))
            err = abs(Fraction(total) / Fraction(2) ** K - exact)
            assert err <= Fraction(mx) * Fraction(2) ** (2 * b - 61), (trial, float(err), mx)


def test_bound_is_within_a_factor_of_two_per_element():
    for st in range(1, 513):
        c = sqrt_exp(st)
        assert math.sqrt(st) <= 2 ** c < 2 * math.sqrt(st) + 1e-12
    for v in (1.0, -3.5, 1e-300, 5e-324, 1.7e308 / 64):
        for st in (1, 2, 3, 4, 512):
            b = bound_bits(v, st)
            assert b < 0x7FF0000000000000
            val = struct.unpack("<d", struct.pack("<Q", b))[0]
            assert val >= abs(v) * math.sqrt(st) * (1 - 1e-15) or abs(v) < 1e-307
