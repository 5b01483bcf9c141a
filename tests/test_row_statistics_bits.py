"""The row statistics' bit arithmetic (stats_rows in split_gemm.cu): for a double x with high word
hi (sign cleared) and a running exponent base, hi * 8 - (base - 127) * 2^23 read as an FP32 is
|x| 2^(1023 - base) with 20 of the 52 mantissa bits, for every exponent field above base - 127: an
underestimate by less than 2^-20 relative, which the plan's 2^-10 allowance on the sums of squares
covers.  The largest high word flags Inf/NaN (exponent field 0x7ff) and gives the frexp exponent of
the largest |x| whenever it is a normal number."""
import math

import numpy as np


def _hi(x):
    return (np.asarray(x, dtype=np.float64).view(np.uint64) >> np.uint64(32)).astype(np.uint64) & np.uint64(0x7FFFFFFF)


def test_fp32_value_from_the_high_word():
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, 200000) * np.exp2(rng.integers(-1000, 1000, 200000))
    hi = _hi(x)
    ea = (hi >> np.uint64(20)).astype(np.int64)
    for base in (127, 300, 1023, 1500, 2046):
        sel = (ea > base - 127) & (ea <= base)
        cbias = np.uint64(((base - 127) << 23) & 0xFFFFFFFF)
        bits = (hi[sel] * np.uint64(8) - cbias) & np.uint64(0xFFFFFFFF)
        f = bits.astype(np.uint32).view(np.float32).astype(np.float64)
        ref = np.abs(x[sel]) * np.exp2(1023.0 - base)
        assert np.all(f <= ref) and np.all(f > 0)
        assert np.max((ref - f) / ref) < 2.0 ** -20


def test_largest_high_word_gives_the_exponent_and_the_nonfinite_flag():
    rng = np.random.default_rng(4)
    for _ in range(200):
        row = rng.uniform(-1, 1, 64) * np.exp2(rng.integers(-1020, 1020))
        m = int(np.max(_hi(row)))
        top = float(np.max(np.abs(row)))
        if m >> 20:  # normal maximum: the frexp exponent follows from the high word alone
            trunc = np.uint64(m << 32).view(np.float64)
            assert math.frexp(float(trunc))[1] == math.frexp(top)[1]
        assert m < 0x7FF00000
    row[5] = np.inf
    assert int(np.max(_hi(row))) >= 0x7FF00000
    row[5] = np.nan
    assert int(np.max(_hi(row))) >= 0x7FF00000
