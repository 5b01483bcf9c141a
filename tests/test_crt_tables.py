"""The residue (CRT) reconstruction constants: crt_tables.h is what crt_tables.py generates, and for
every modulus count N = 2..15 the reconstruction the device runs (crt_cols in split_gemm.cu: super
residues u_s = (c_p A_s + c_q B_s) mod P_s, W = sum_s u_s P/P_s in integers, the multiple of P to
remove picked by an FP32 estimate of sum_s u_s / P_s) returns every integer T with
|T| < P / 2.125 (the range the residue plan guarantees) from its residues, including both ends of
that range.  The FP32 estimate is replayed with one rounding per multiply-add, as the device's fmaf
rounds."""
import importlib.util
import os
import random
import struct
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GEN = os.path.join(ROOT, "blaze_gb300", "csrc", "crt_tables.py")
HDR = os.path.join(ROOT, "blaze_gb300", "csrc", "crt_tables.h")


def _gen():
    spec = importlib.util.spec_from_file_location("crt_tables_gen", GEN)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _f32(x):
    """x (a Fraction) rounded to the nearest FP32, ties to even."""
    c = np.float32(float(x))
    best = None
    for cand in (np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf))):
        d = abs(Fraction(float(cand)) - x)
        even = (struct.unpack("<I", struct.pack("<f", float(cand)))[0] & 1) == 0
        if best is None or d < best[0] or (d == best[0] and even):
            best = (d, cand)
    return Fraction(float(best[1]))


def _reconstruct(t, residues):
    """The device's reconstruction of one output from its residues in [0, p)."""
    P = t["P"]
    fq = -_f32(Fraction(t["fbias"]))
    W = 0
    for s in t["sups"]:
        cp = residues[s["ia"]]
        cq = residues[s["ib"]] if s["ib"] >= 0 else 0
        u = (cp * s["A"] + cq * s["B"]) % s["Ps"]
        # fmaf(float(2^23 + u), finv, fq): 2^23 + u is exact in FP32 (u < 2^16)
        fq = _f32(Fraction((1 << 23) + u) * _f32(Fraction(1, s["Ps"])) + fq)
        W += u * (P // s["Ps"])
    q = int(round(fq))  # the device adds 1.5 * 2^23 and reads the integer back: round to nearest
    return W - q * P


def test_header_is_what_the_generator_writes(tmp_path):
    out = tmp_path / "crt_tables.h"
    _gen().emit(str(out))
    with open(HDR) as f:
        assert out.read_text() == f.read()


def test_moduli_are_pairwise_coprime_and_residues_fit_bf16():
    g = _gen()
    from math import gcd
    mods = g.MODULI
    assert all(2 <= p <= 257 for p in mods)
    for i in range(len(mods)):
        for j in range(i + 1, len(mods)):
            assert gcd(mods[i], mods[j]) == 1, (mods[i], mods[j])


@pytest.mark.parametrize("n", list(range(2, 16)))
def test_reconstruction_returns_every_integer_of_the_plans_range(n):
    g = _gen()
    t = g.table(n)
    P = t["P"]
    lim = int(Fraction(P) / Fraction(2125, 1000))  # |T| < P / 2.125
    rng = random.Random(1000 + n)
    cases = [0, 1, -1, lim - 1, -(lim - 1), lim // 2, -(lim // 3)]
    cases += [rng.randrange(-lim + 1, lim) for _ in range(300)]
    mods = g.MODULI[:n]
    for T in cases:
        res = [T % p for p in mods]  # the tensor-core epilogue leaves residues in [0, p)
        assert _reconstruct(t, res) == T, (n, T)
    # the signed result fits the limbs the device uses
    assert (lim.bit_length() + 1) <= 32 * t["limbs"]
