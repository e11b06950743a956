"""The arithmetic of the executor's tensor-core FP64 updates (ttg_gb300/csrc/emu_f64.cuh), restated
with Python integers and checked against exact rationals (CPU):
  * splitting: row scale 2^e (|x| < 2^e), F = round(x 2^(55-e)) as seven balanced base-256 digits,
    each of at most 8 significant bits (exact in bf16);
  * products: group sums acc_g = sum_{i+j=g} sum_k a_i b_j for g <= 6 stay below 2^24 in magnitude
    for k = 128 (exact in the tensor cores' FP32 accumulation);
  * composition: X = H 2^32 + L in 64 bits (X 2^-8 when |H| >= 2^30), rounded once to FP64 and
    scaled by a power of two;
  * subtraction from C: one FMA with 2^sE, or with two clamped normal powers of two where 2^sE is
    not normal, rounded once for |sE| <= 2044 and the right limit beyond.
The emulated dot product must be at least as accurate as a plain FP64 loop over the same inputs."""
import math
import struct
from fractions import Fraction

import numpy as np
import pytest


def _bits(x):
    return struct.unpack("<q", struct.pack("<d", x))[0]


def split_row(row):
    mex = max(((_bits(v) >> 52) & 0x7FF) for v in row)
    e = mex - 1022
    digits = []
    for v in row:
        b = _bits(v)
        ex = (b >> 52) & 0x7FF
        F = 0
        if ex > 0 and mex > 0:
            mant = (b & ((1 << 52) - 1)) | (1 << 52)
            sh = ex - 1020 - e
            assert sh <= 2
            f = mant << sh if sh >= 0 else ((mant + (1 << (-sh - 1))) >> (-sh) if sh > -60 else 0)
            F = -f if b < 0 else f
        d = [0] * 7
        for i in range(6, 0, -1):
            d[i] = ((F + 128) & 255) - 128
            F = (F - d[i]) >> 8
        d[0] = F
        assert all(-128 <= x <= 128 for x in d)
        digits.append(d)
    return e, digits


def compose(acc, E):
    """X 2^E as the executor forms it: X = sum_g acc_g 2^(8(6-g)) in 64 bits (as X 2^-s when the
    high groups are large), rounded to FP64 (to nearest even), then scaled by 2^(s + E)."""
    H = (acc[0] << 16) + (acc[1] << 8) + acc[2]
    L = (acc[3] << 24) + (acc[4] << 16) + (acc[5] << 8) + acc[6]
    s = 8 if abs(H) >= 2 ** 30 else 0
    X = (H << (32 - s)) + (L >> s)  # >> floors, as the arithmetic shift does
    assert abs(X) < 2 ** 63
    return math.ldexp(float(X), E + s)  # float(int) rounds to nearest even


def emulated_dot(a, b):
    ea, da = split_row(a)
    eb, db = split_row(b)
    acc = []
    for g in range(7):
        t = sum(da[k][i] * db[k][g - i] for i in range(g + 1) for k in range(len(a)))
        assert abs(t) < 2 ** 24, "group sum not exact in FP32"
        acc.append(t)
    return compose(acc, ea + eb - 62)


@pytest.mark.parametrize("seed", range(6))
def test_emulated_dot_is_at_least_fp64_accurate(seed):
    rng = np.random.default_rng(seed)
    worst_emu = worst_fp64 = 0.0
    for trial in range(40):
        scale = 10.0 ** rng.uniform(-3, 3, size=2)
        a = rng.uniform(-1, 1, 128) * scale[0]
        b = rng.uniform(-1, 1, 128) * scale[1]
        if trial % 4 == 0:  # no cancellation: the largest group sums
            a, b = np.abs(a), np.abs(b)
        if trial % 7 == 0:  # entries far below the row maximum
            a[rng.integers(0, 128, 20)] *= 1e-9
        exact = sum(Fraction(x) * Fraction(y) for x, y in zip(a, b))
        den = Fraction(float(np.max(np.abs(a)) * np.max(np.abs(b))))
        worst_emu = max(worst_emu, float(abs(Fraction(emulated_dot(a, b)) - exact) / den))
        s = 0.0
        for x, y in zip(a, b):
            s = s + x * y
        worst_fp64 = max(worst_fp64, float(abs(Fraction(s) - exact) / den))
    assert worst_emu <= 4e-15
    assert worst_emu <= worst_fp64


def test_extreme_digits_stay_exact():
    """All-equal rows of the largest magnitude: every digit at its bound, group sums at their maximum."""
    a = np.full(128, np.nextafter(1.0, 0.0))
    exact = sum(Fraction(x) * Fraction(x) for x in a)
    got = emulated_dot(a, a)
    assert abs(Fraction(got) - exact) <= exact * Fraction(2.0 ** -52)


def test_zero_and_subnormal_rows():
    assert emulated_dot(np.zeros(128), np.ones(128)) == 0.0
    tiny = np.full(128, 5e-324)
    assert emulated_dot(tiny, np.ones(128)) == 0.0  # subnormal rows carry no digits


def _round(q):
    """A rational rounded to FP64 (to nearest even; float(Fraction) rounds correctly)."""
    try:
        return float(q)
    except OverflowError:
        return math.inf if q > 0 else -math.inf


def _sub_scaled(c, X, sE):
    """c - X 2^sE as the executor forms it (emu_f64.cuh): X rounded to FP64, then one FMA with
    2^sE, or, when 2^sE is not a normal FP64 number, with 2^a 2^b (a = sE / 2 truncated, both
    clamped to the normal exponents) after the exact product X 2^a."""
    x = float(X)
    if -1022 <= sE <= 1023:
        return _round(Fraction(c) - Fraction(x) * Fraction(2) ** sE)
    a = min(max(int(sE / 2), -1022), 1023)
    b = min(max(sE - a, -1022), 1023)
    p = x * 2.0 ** a if a >= 0 else x / 2.0 ** -a  # exact: |x| >= 1 and a >= -1022
    assert math.isinf(p) or Fraction(p) == Fraction(x) * Fraction(2) ** a
    if math.isinf(p):
        return -p if c == c else c
    return _round(Fraction(c) - Fraction(p) * Fraction(2) ** b)


@pytest.mark.parametrize("sE", [-2150, -2044, -1600, -1100, -1075, -1074, -1060, -1023, -1022, -500, 0,
                                900, 1023, 1024, 1500, 2046, 2200])
def test_scaled_subtraction_rounds_once(sE):
    """c - X 2^sE: the value rounded once from the exact c - fl(X) 2^sE wherever |sE| <= 2044
    (subnormal and overflowing results included), and the right limit beyond."""
    rng = np.random.default_rng(sE & 0xffff)
    for _ in range(200):
        X = int(rng.integers(1, 2 ** 62)) * int(rng.choice([-1, 1]))
        x = float(X)
        for c in (0.0, 1.5, -3.25e-300, 7e-310, 2.0 ** -1074, 1e300):
            got = _sub_scaled(c, X, sE)
            if abs(sE) <= 2044:
                assert got == _round(Fraction(c) - Fraction(x) * Fraction(2) ** sE)
            elif sE < 0:  # X 2^sE below half the smallest subnormal: c itself
                assert got == c
            else:
                assert math.isinf(got) and (got < 0) == (X > 0)
