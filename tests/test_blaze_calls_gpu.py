"""Replay, through the real library on a GB300, every CBLAS call Blaze made in BLAS mode
(tests/golden/blaze_calls.txt, recorded from Blaze itself by tests/golden/record_blaze_calls.py):
same order, transposition flags, sizes, leading dimensions, alpha and beta, on seeded inputs,
checked against the oracle's restatement of Blaze's default kernel with Blaze's relaxed
equality (1e-8), for every arithmetic form that claims FP64 accuracy."""
import os

import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O
from helpers import blaze_equal, stored_dims

pytestmark = pytest.mark.gpu
CALLS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blaze_calls.txt")


def load_calls():
    out = []
    for ln in open(CALLS).read().splitlines():
        f = ln.split()
        out.append(dict(order=int(f[1]), ta=int(f[2]), tb=int(f[3]), m=int(f[4]), n=int(f[5]), k=int(f[6]),
                        alpha=float(f[7]), lda=int(f[8]), ldb=int(f[9]), beta=float(f[10]), ldc=int(f[11])))
    return out


@pytest.mark.parametrize("method", [G.METHOD_AUTO, G.METHOD_NATIVE, G.METHOD_SPLIT])
def test_replay_blaze_calls(method):
    prev = G.lib().gb300_set_default_method(method)
    try:
        for i, c in enumerate(load_calls()):
            ra, _ = stored_dims(c["order"], c["ta"], c["m"], c["k"])
            rb, _ = stored_dims(c["order"], c["tb"], c["k"], c["n"])
            rc, _ = stored_dims(c["order"], O.NO_TRANS, c["m"], c["n"])
            A = O.uniform(ra * c["lda"], 100 + i)
            B = O.uniform(rb * c["ldb"], 200 + i)
            C = O.uniform(rc * c["ldc"], 300 + i)
            R = C.copy()
            O.gemm(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A, c["lda"], B, c["ldb"],
                   c["beta"], R, c["ldc"], kernel="default")
            G.cblas_dgemm(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A, c["lda"], B, c["ldb"],
                          c["beta"], C, c["ldc"])
            assert blaze_equal(R, C, 1e-8).all(), c
    finally:
        G.lib().gb300_set_default_method(prev)
