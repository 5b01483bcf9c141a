"""Generate the golden fixtures of the neighbouring BLAS routines (gemv, trmv, complex gemm, trmm,
trsm, axpy and the dot products, real and complex) from Blaze itself.

Run in a container that has the reference headers (Blaze is header-only):

    make -C oracle ref                         # builds oracle/_ref/libblazeref.so from the headers
    python tests/golden/make_golden_next.py    # writes tests/golden/next_golden.npz

Each case is evaluated by Blaze's default (non-BLAS) kernels on blaze::CustomMatrix /
CustomVector views (oracle/blaze_ref.cpp): y = alpha*op(A)*x + beta*y for gemv; complex
C = alpha*op(A)*op(B) + beta*C with op in {N, T, conjugate-transpose} for zgemm; B = alpha*op(A)*B or
alpha*B*op(A) with A triangular (upper/lower, unit/non-unit diagonal) for trmm; x = op(A)*x with A
triangular for trmv (Blaze's LowerMatrix / UpperMatrix / Uni* adaptors).  Inputs are not
stored: they are regenerated from their seeds by the oracle's MT19937 generator (checksums kept).
"""
from __future__ import annotations

import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "next_golden.npz")
CONJ = 113


def zvals(count, seed):
    re = O.uniform(max(count, 1), seed)[:count]
    im = O.uniform(max(count, 1), seed + 7919)[:count]
    return re + 1j * im


def gemv_cases():
    out, seed = [], 5000
    sizes = [(0, 5), (5, 0), (1, 1), (7, 13), (64, 37), (130, 257)]
    ab = [(1.0, 0.0), (2.5, 1.0), (-1.0, -0.5)]
    for i, (m, n) in enumerate(sizes):
        for j, (order, ta) in enumerate(itertools.product((O.ROW_MAJOR, O.COL_MAJOR), (O.NO_TRANS, O.TRANS))):
            al, be = ab[(i + j) % 3]
            out.append((order, ta, m, n, al, be, (i + j) % 2, seed))
            seed += 3
    return out


def zgemm_cases():
    out, seed = [], 7000
    sizes = [(3, 4, 5), (37, 16, 63), (64, 64, 64), (130, 40, 90)]
    ops = (O.NO_TRANS, O.TRANS, CONJ)
    ab = [(1 + 0j, 0j), (0.5 - 1j, 0j), (1 + 0j, 1 + 0j), (-0.25 + 2j, 0.5 - 0.5j)]
    for i, (m, n, k) in enumerate(sizes):
        for j, (order, ta, tb) in enumerate(itertools.product((O.ROW_MAJOR, O.COL_MAJOR), ops, ops)):
            if (i + j) % 2:  # half of the 18 layouts per size
                continue
            al, be = ab[(i + j) % 4]
            out.append((order, ta, tb, m, n, k, al, be, j % 2, seed))
            seed += 3
    return out


def trmm_cases():
    out, seed = [], 9000
    sizes = [(5, 7), (37, 16), (130, 36)]
    combos = list(itertools.product((O.ROW_MAJOR, O.COL_MAJOR), (141, 142), (121, 122), (O.NO_TRANS, O.TRANS), (131, 132)))
    for i, (m, n) in enumerate(sizes):
        for j, (order, side, uplo, ta, diag) in enumerate(combos):
            if (i + j) % 2:
                continue
            al = (1.0, -0.75, 2.0)[(i + j) % 3]
            out.append((order, side, uplo, ta, diag, m, n, al, j % 2, seed))
            seed += 2
    return out


def zgemv_cases():
    out, seed = [], 11000
    sizes = [(1, 1), (7, 13), (64, 37), (130, 257)]
    ab = [(1 + 0j, 0j), (0.5 - 1j, 0j), (1 + 0j, 1 + 0j), (-0.25 + 2j, 0.5 - 0.5j)]
    for i, (m, n) in enumerate(sizes):
        for j, (order, ta) in enumerate(itertools.product((O.ROW_MAJOR, O.COL_MAJOR), (O.NO_TRANS, O.TRANS, CONJ))):
            al, be = ab[(i + j) % 4]
            out.append((order, ta, m, n, al, be, (i + j) % 2, seed))
            seed += 3
    return out


def trmv_cases():
    out, seed = [], 13000
    for cplx in (0, 1):
        ops = (O.NO_TRANS, O.TRANS, CONJ) if cplx else (O.NO_TRANS, O.TRANS)
        combos = list(itertools.product((O.ROW_MAJOR, O.COL_MAJOR), (121, 122), ops, (131, 132)))
        for i, n in enumerate((1, 7, 64, 130)):
            for j, (order, uplo, ta, diag) in enumerate(combos):
                if n > 1 and (i + j) % 2:
                    continue
                out.append((cplx, order, uplo, ta, diag, n, j % 2, seed))
                seed += 2
    return out


def ztrmm_cases():
    out, seed = [], 15000
    sizes = [(5, 7), (37, 16), (130, 36)]
    combos = list(itertools.product((O.ROW_MAJOR, O.COL_MAJOR), (141, 142), (121, 122), (O.NO_TRANS, O.TRANS, CONJ),
                                    (131, 132)))
    for i, (m, n) in enumerate(sizes):
        for j, (order, side, uplo, ta, diag) in enumerate(combos):
            if (i + j) % 3:
                continue
            al = (1 + 0j, -0.75 + 0.5j, 2j)[(i + j) % 3]
            out.append((order, side, uplo, ta, diag, m, n, al, j % 2, seed))
            seed += 2
    return out


def dot_cases():
    out, seed = [], 17000
    for cplx in (0, 1):
        for conj in ((0, 1) if cplx else (0,)):
            for n in (1, 3, 7, 100, 1000, 4097):
                out.append((cplx, conj, n, seed))
                seed += 2
    return out


def axpy_cases():
    out, seed = [], 18000
    for cplx in (0, 1):
        alphas = (0.5 - 1.25j, -2 + 0j, 1j) if cplx else (1.5, -0.75, 3.0)
        for i, n in enumerate((1, 7, 257, 1000)):
            out.append((cplx, n, alphas[i % 3], seed))
            seed += 2
    return out


def trsm_cases():
    """blazetest's BLAS operation test solves 3 x 3 triangular systems with one and with several
    right-hand sides on either side (OperationTest.h:255-715); here also triangles of a few hundred
    rows (few right-hand sides keep the fixture small)."""
    out, seed = [], 19000
    sizes = [(3, 1), (1, 3), (3, 3), (37, 16), (130, 8), (300, 6), (6, 300)]
    for cplx in (0, 1):
        ops = (O.NO_TRANS, O.TRANS, CONJ) if cplx else (O.NO_TRANS, O.TRANS)
        combos = list(itertools.product((O.ROW_MAJOR, O.COL_MAJOR), (141, 142), (121, 122), ops, (131, 132)))
        alphas = (1 + 0j, 0.5j, -2 + 0j) if cplx else (1.0, -0.5, 2.0)
        for i, (m, n) in enumerate(sizes):
            for j, (order, side, uplo, ta, diag) in enumerate(combos):
                keep = 1 if max(m, n) <= 3 else (4 if max(m, n) < 200 else 8)
                if (i + j) % keep:
                    continue
                out.append((cplx, order, side, uplo, ta, diag, m, n, alphas[(i + j) % 3], j % 2, seed))
                seed += 2
    return out


def trsm_operands(cplx, ka, lda, m, n, order, pad, seed):
    """The triangle's stored square and the solution X0 in the storage of B (ldb = columns + pad)."""
    rb, cb = stored(order, O.NO_TRANS, m, n)
    ldb = cb + pad
    A, X0 = O.triangular_operands(bool(cplx), ka, lda, rb, ldb, seed)
    return A, X0, ldb


def stored(order, trans, rows, cols):
    t = trans != O.NO_TRANS
    r, c = (cols, rows) if t else (rows, cols)
    return (r, c) if order == O.ROW_MAJOR else (c, r)


def main():
    arrays = {}
    for q, (order, ta, m, n, al, be, pad, seed) in enumerate(gemv_cases()):
        r, c = stored(order, O.NO_TRANS, m, n)  # A is m x n in CBLAS order
        lda = max(c, 1) + pad
        A = O.uniform(max(r * lda, 1), seed)
        xl, yl = (m, n) if ta != O.NO_TRANS else (n, m)
        x = O.uniform(max(xl, 1), seed + 1)[:xl]
        y = O.uniform(max(yl, 1), seed + 2)[:yl]
        O.ref_gemv(order, ta, m, n, al, A, lda, x, be, y)
        arrays[f"gemv{q}_meta"] = np.array([order, ta, m, n, lda, seed], dtype=np.int64)
        arrays[f"gemv{q}_ab"] = np.array([al, be])
        arrays[f"gemv{q}_y"] = y
    for q, (order, ta, tb, m, n, k, al, be, pad, seed) in enumerate(zgemm_cases()):
        ra, ca = stored(order, ta, m, k)
        rb, cb = stored(order, tb, k, n)
        rc, cc = stored(order, O.NO_TRANS, m, n)
        lda, ldb, ldc = ca + pad, cb + pad, cc + pad
        A = zvals(ra * lda, seed)
        B = zvals(rb * ldb, seed + 1)
        C = zvals(rc * ldc, seed + 2)
        O.ref_zgemm(order, ta, tb, m, n, k, al, A, lda, B, ldb, be, C, ldc)
        arrays[f"zgemm{q}_meta"] = np.array([order, ta, tb, m, n, k, lda, ldb, ldc, seed], dtype=np.int64)
        arrays[f"zgemm{q}_ab"] = np.array([al, be])
        arrays[f"zgemm{q}_C"] = C
    for q, (order, side, uplo, ta, diag, m, n, al, pad, seed) in enumerate(trmm_cases()):
        ka = m if side == 141 else n
        lda = ka + pad
        rb, cb = stored(order, O.NO_TRANS, m, n)
        ldb = cb + pad
        A = O.uniform(ka * lda, seed)
        B = O.uniform(rb * ldb, seed + 1)
        O.ref_trmm(order, side, uplo, ta, diag, m, n, al, A, lda, B, ldb)
        arrays[f"trmm{q}_meta"] = np.array([order, side, uplo, ta, diag, m, n, lda, ldb, seed], dtype=np.int64)
        arrays[f"trmm{q}_alpha"] = np.array([al])
        arrays[f"trmm{q}_B"] = B
    for q, (order, ta, m, n, al, be, pad, seed) in enumerate(zgemv_cases()):
        r, c = stored(order, O.NO_TRANS, m, n)
        lda = c + pad
        A = zvals(r * lda, seed)
        xl, yl = (m, n) if ta != O.NO_TRANS else (n, m)
        x = zvals(xl, seed + 1)
        y = zvals(yl, seed + 2)
        O.ref_zgemv(order, ta, m, n, al, A, lda, x, be, y)
        arrays[f"zgemv{q}_meta"] = np.array([order, ta, m, n, lda, seed], dtype=np.int64)
        arrays[f"zgemv{q}_ab"] = np.array([al, be])
        arrays[f"zgemv{q}_y"] = y
    for q, (cplx, order, uplo, ta, diag, n, pad, seed) in enumerate(trmv_cases()):
        lda = n + pad
        A = zvals(n * lda, seed) if cplx else O.uniform(n * lda, seed)
        x = zvals(n, seed + 1) if cplx else O.uniform(n, seed + 1).copy()
        O.ref_trmv(order, uplo, ta, diag, n, A, lda, x)
        arrays[f"trmv{q}_meta"] = np.array([cplx, order, uplo, ta, diag, n, lda, seed], dtype=np.int64)
        arrays[f"trmv{q}_x"] = x
    for q, (order, side, uplo, ta, diag, m, n, al, pad, seed) in enumerate(ztrmm_cases()):
        ka = m if side == 141 else n
        lda = ka + pad
        rb, cb = stored(order, O.NO_TRANS, m, n)
        ldb = cb + pad
        A = zvals(ka * lda, seed)
        B = zvals(rb * ldb, seed + 1)
        O.ref_ztrmm(order, side, uplo, ta, diag, m, n, al, A, lda, B, ldb)
        arrays[f"ztrmm{q}_meta"] = np.array([order, side, uplo, ta, diag, m, n, lda, ldb, seed], dtype=np.int64)
        arrays[f"ztrmm{q}_alpha"] = np.array([al])
        arrays[f"ztrmm{q}_B"] = B
    for q, (cplx, conj, n, seed) in enumerate(dot_cases()):
        x = zvals(n, seed) if cplx else O.uniform(n, seed).copy()
        y = zvals(n, seed + 1) if cplx else O.uniform(n, seed + 1).copy()
        arrays[f"dot{q}_meta"] = np.array([cplx, conj, n, seed], dtype=np.int64)
        arrays[f"dot{q}_r"] = np.array([O.ref_dot(x, y, conj=bool(conj))])
    for q, (cplx, n, al, seed) in enumerate(axpy_cases()):
        x = zvals(n, seed) if cplx else O.uniform(n, seed).copy()
        y = zvals(n, seed + 1) if cplx else O.uniform(n, seed + 1).copy()
        O.ref_axpy(al, x, y)
        arrays[f"axpy{q}_meta"] = np.array([cplx, n, seed], dtype=np.int64)
        arrays[f"axpy{q}_alpha"] = np.array([al])
        arrays[f"axpy{q}_y"] = y
    # trsm: Blaze forms B = op(A) X0 (left) or X0 op(A) (right) with its own kernels (the trmm
    # evaluation above, alpha = 1); solving with alpha (a power of two, so alpha X0 is exact) must
    # give back alpha X0
    for q, (cplx, order, side, uplo, ta, diag, m, n, al, pad, seed) in enumerate(trsm_cases()):
        ka = m if side == 141 else n
        lda = ka + pad
        A, X0, ldb = trsm_operands(cplx, ka, lda, m, n, order, pad, seed)
        B = X0.copy()
        if cplx:
            O.ref_ztrmm(order, side, uplo, ta, diag, m, n, 1 + 0j, A, lda, B, ldb)
        else:
            O.ref_trmm(order, side, uplo, ta, diag, m, n, 1.0, A, lda, B, ldb)
        arrays[f"trsm{q}_meta"] = np.array([cplx, order, side, uplo, ta, diag, m, n, lda, ldb, pad, seed],
                                           dtype=np.int64)
        arrays[f"trsm{q}_alpha"] = np.array([al])
        arrays[f"trsm{q}_B"] = B
    np.savez_compressed(OUT, **arrays)
    print(OUT, len(arrays), "arrays,", os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
