"""CPU check of the integer rounding behind the double-float split (ttg_gb300/csrc/refine.cu,
split_f64): for every FP64 value a whose biased exponent e is in [950, 1149],
    hi = sign | ((e - 896) << 23 | top 23 mantissa bits) + round-up bit   (nearest, ties to even)
    lo = fl32(r) * 2^(e - 1075),  r = +-(low 29 bits, minus 2^29 when rounded up)
equals the FP64 conversions hi = fl32(a), lo = fl32(a - hi) bit for bit. The device code is checked
against the same conversions on the GPU (test_gpu_mixed.py::test_split_f64_bitwise); this test
sweeps the whole exponent range of the integer path, its two edges and the rounding ties in numpy.
"""
import numpy as np


def split_bits(a):
    b = a.view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    t = ((b >> np.uint64(29)) & np.uint64(0x7FFFFF)).astype(np.int64)
    rem = (b & np.uint64(0x1FFFFFFF)).astype(np.int64)
    up = (rem > (1 << 28)) | ((rem == (1 << 28)) & ((t & 1) == 1))
    sgn = (b >> np.uint64(63)).astype(np.int64)
    mag = (((e - 896) << 23) | t) + up.astype(np.int64)
    hi = ((sgn << 31) | mag).astype(np.uint32).view(np.float32)
    r = np.where(up, rem - (1 << 29), rem)
    r = np.where(sgn == 1, -r, r)
    scale = ((e - 948) << 23).astype(np.uint32).view(np.float32)
    lo = r.astype(np.float32) * scale  # int -> float32 rounds to nearest even, the scaling is exact
    return e, hi, lo


def test_integer_split_matches_fp64_conversions():
    rng = np.random.default_rng(11)
    n = 1 << 21
    e = rng.integers(950, 1150, n, dtype=np.int64)
    e[:4] = [950, 950, 1149, 1149]
    m = rng.integers(0, 1 << 52, n, dtype=np.int64)
    m[: n // 8] = (m[: n // 8] & ~((1 << 29) - 1)) | (1 << 28)  # ties of the hi rounding
    m[n // 8: n // 4] |= (1 << 29) - 1                           # carries into the exponent
    s = rng.integers(0, 2, n, dtype=np.int64)
    bits = (s << 63) | (e << 52) | m
    a = bits.astype(np.uint64).view(np.float64)
    ee, hi, lo = split_bits(a)
    assert ((ee >= 950) & (ee <= 1149)).all()
    h_ref = a.astype(np.float32)
    l_ref = (a - h_ref.astype(np.float64)).astype(np.float32)
    assert np.array_equal(hi.view(np.uint32), h_ref.view(np.uint32))
    assert np.array_equal(lo.view(np.uint32), l_ref.view(np.uint32))
    # hi + lo carries 48 significant bits of a
    err = np.abs((hi.astype(np.float64) + lo.astype(np.float64)) - a) / np.abs(a)
    assert err.max() <= 2.0 ** -47
