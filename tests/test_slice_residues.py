"""The residue form's slicing arithmetic (slice_emit in split_gemm.cu, CRT mode): the scaled integer
U < 2^56 goes in as four signed 14-bit FP32 chunks w0..w3, and the residue modulo p is
x = w3 k3 + w2 k2 + w1 k1 + w0 (k_j the symmetric residue of 2^(14 j) mod p) followed by
x - p rint(x inv) with inv = 1/p rounded to FP32.  The constants in the source are checked, every
intermediate stays an integer below 2^24 (exact in FP32), and for every x the chunks can produce
next to a half multiple of p (where the FP32 quotient estimate is closest to picking the wrong
multiple) the residue is the symmetric one, |r| <= 128: the bound the tensor-core products'
exactness rests on.  The estimate is evaluated exactly: fmaf(x, inv, 1.5 * 2^23) rounds x * inv
once, to the nearest integer (ties to even) for |x * inv| < 2^22."""
import os
import re
import struct

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "blaze_gb300", "csrc", "split_gemm.cu")


def _floats(body):
    out = []
    for tok in re.findall(r"[-+]?0x[0-9a-fA-F.]+p[-+]?\d+f|[-+]?\d+\.?\d*f", body):
        t = tok[:-1]
        out.append(float.fromhex(t) if "x" in t else float(t))
    return out


def _constants():
    src = open(SRC).read()
    mods = [int(v) for v in re.search(r"c_mod\[MAX_MODULI\] = \{([^}]*)\}", src).group(1).split(",")]
    modf = _floats(re.search(r"c_modf\[MAX_MODULI\] = \{([^}]*)\}", src).group(1))
    inv = _floats(re.search(r"c_modf_inv\[MAX_MODULI\] = \{([^}]*)\}", src).group(1))
    k14_body = re.search(r"c_mod_k14\[3\]\[MAX_MODULI\] = \{(.*?)\};", src, re.S).group(1)
    rows = [_floats(r) for r in re.findall(r"\{([^{}]*)\}", k14_body)]
    return mods, modf, inv, rows


def _f32(x):
    return struct.unpack("<f", struct.pack("<f", x))[0]


def test_slicing_constants_match_the_moduli():
    mods, modf, inv, k14 = _constants()
    assert len(mods) == len(modf) == len(inv) == 15 and len(k14) == 3
    for t, p in enumerate(mods):
        assert modf[t] == float(p)
        assert inv[t] == _f32(1.0 / p)
        for j in range(3):
            k = int(k14[j][t])
            assert k == k14[j][t] and abs(k) <= p // 2
            assert (k - pow(2, 14 * (j + 1), p)) % p == 0


@pytest.mark.parametrize("t", list(range(15)))
def test_residue_is_the_symmetric_one_next_to_every_half_multiple(t):
    mods, modf, inv, k14 = _constants()
    p = mods[t]
    ks = [int(k14[j][t]) for j in range(3)]
    cmax = (1 << 14) - 1
    X = cmax * (1 + sum(abs(k) for k in ks))  # largest |x| the chunks reach
    assert X < 1 << 23  # every partial sum of the chain is an integer exact in FP32
    m, e = np.frexp(np.float64(inv[t]))  # inv = m 2^e, m in [0.5, 1)
    mant = int(m * (1 << 24))            # inv = mant 2^(e - 24), mant < 2^24
    shift = 24 - int(e)
    assert float(mant) * 2.0 ** (-shift) == inv[t]
    # x next to (kq + 1/2) p for every kq in range, both sides
    kq = np.arange(-(X // p) - 1, X // p + 1, dtype=np.int64)
    offs = [p // 2 - 1, p // 2, p // 2 + 1, (p + 1) // 2]
    x = np.unique(np.concatenate([kq * p + o for o in offs]))
    x = x[np.abs(x) <= X]
    assert np.all(np.abs(x) * inv[t] < 2.0 ** 22)
    # q = round_half_even(x * mant / 2^shift), exactly in integers
    num = x * mant
    half = np.int64(1) << (shift - 1)
    fl = np.floor_divide(num, np.int64(1) << shift)
    rem = num - fl * (np.int64(1) << shift)
    up = (rem > half) | ((rem == half) & (fl % 2 == 1))
    q = fl + up.astype(np.int64)
    r = x - p * q
    assert np.all(np.abs(r) <= 128), (p, int(np.max(np.abs(r))))
    assert np.all((r - x) % p == 0)
