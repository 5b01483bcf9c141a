"""Seeded batched-product workloads: M, N, K log-uniform integers in [lo, hi] (round(exp(U[ln lo,
ln hi]))), uniform [-1,1] entries, operands packed in one device buffer per operand."""
from __future__ import annotations

import numpy as np

import oracle as O
from helpers import stored_dims


def sizes(count: int, seed: int, lo: int = 4, hi: int = 256) -> np.ndarray:
    u = O.uniform(3 * count, seed, np.log(lo), np.log(hi))
    return np.clip(np.rint(np.exp(u)).astype(np.int64), lo, hi).reshape(count, 3)


def host_batch(count: int, seed: int, dtype=np.float64, layouts: bool = False, alphabeta: bool = False,
               lo: int = 4, hi: int = 256):
    """The problem dicts (offsets into one buffer per operand) and the host operands of a batch."""
    mnk = sizes(count, seed, lo, hi)
    rng = np.random.default_rng(seed)
    specs, hostA, hostB, hostC = [], [], [], []
    offA = offB = offC = 0
    for q in range(count):
        m, n, k = (int(x) for x in mnk[q])
        if layouts:
            order = O.ROW_MAJOR if rng.integers(2) == 0 else O.COL_MAJOR
            ta = O.NO_TRANS if rng.integers(2) == 0 else O.TRANS
            tb = O.NO_TRANS if rng.integers(2) == 0 else O.TRANS
        else:
            order, ta, tb = O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS
        ra, ca = stored_dims(order, ta, m, k)
        rb, cb = stored_dims(order, tb, k, n)
        rc, cc = stored_dims(order, O.NO_TRANS, m, n)
        alpha, beta = (1.0, 0.0) if not alphabeta else ((1.5, 0.0), (1.0, 1.0), (-0.5, 2.0))[q % 3]
        specs.append(dict(order=order, transA=ta, transB=tb, m=m, n=n, k=k, alpha=alpha, beta=beta,
                          offA=offA, lda=ca, offB=offB, ldb=cb, offC=offC, ldc=cc, ra=ra, rb=rb, rc=rc))
        offA += ra * ca; offB += rb * cb; offC += rc * cc
    A = O.uniform(offA, seed + 1, dtype=dtype)
    B = O.uniform(offB, seed + 2, dtype=dtype)
    C = O.uniform(offC, seed + 3, dtype=dtype)
    return specs, A, B, C


def build(torch, count: int, seed: int, dtype=np.float64, layouts: bool = False, alphabeta: bool = False,
          lo: int = 4, hi: int = 256):
    """Host operands, device copies and the problem dicts for a batch."""
    specs, A, B, C = host_batch(count, seed, dtype, layouts, alphabeta, lo, hi)
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    dC = torch.from_numpy(C).cuda()
    esz = 8 if dtype == np.float64 else 4
    for sp in specs:
        sp["A"] = dA.data_ptr() + sp["offA"] * esz
        sp["B"] = dB.data_ptr() + sp["offB"] * esz
        sp["C"] = dC.data_ptr() + sp["offC"] * esz
    del tdt
    return specs, A, B, C, dA, dB, dC


def reference(specs, A, B, C0, kernel="default"):
    """The same batch through the oracle's restatement of Blaze's default (or small) kernel."""
    R = C0.copy()
    for sp in specs:
        a = A[sp["offA"]: sp["offA"] + sp["ra"] * sp["lda"]]
        b = B[sp["offB"]: sp["offB"] + sp["rb"] * sp["ldb"]]
        c = R[sp["offC"]: sp["offC"] + sp["rc"] * sp["ldc"]]
        O.gemm(sp["order"], sp["transA"], sp["transB"], sp["m"], sp["n"], sp["k"], sp["alpha"], a, sp["lda"], b,
               sp["ldb"], sp["beta"], c, sp["ldc"], kernel=kernel)
    return R
