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


# ---- products Blaze's kernel selection keeps on the CPU, sent to ?gemm by include/gb300_blaze.h
# (tests/golden/blaze_gated_calls.txt, recorded from Blaze with the header)
GATED_CALLS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blaze_gated_calls.txt")


@pytest.mark.parametrize("method", [G.METHOD_AUTO, G.METHOD_NATIVE, G.METHOD_SPLIT])
def test_replay_intercepted_blaze_calls(method):
    lines = open(GATED_CALLS).read().splitlines()
    assert len(lines) == 14
    prev = G.lib().gb300_set_default_method(method)
    try:
        for i, ln in enumerate(lines):
            f = ln.split()
            c = dict(order=int(f[1]), ta=int(f[2]), tb=int(f[3]), m=int(f[4]), n=int(f[5]), k=int(f[6]),
                     alpha=float(f[7]), lda=int(f[8]), ldb=int(f[9]), beta=float(f[10]), ldc=int(f[11]))
            dt = np.float32 if f[0] == "sgemm" else np.float64
            ra, _ = stored_dims(c["order"], c["ta"], c["m"], c["k"])
            rb, _ = stored_dims(c["order"], c["tb"], c["k"], c["n"])
            rc, _ = stored_dims(c["order"], O.NO_TRANS, c["m"], c["n"])
            A = O.uniform(ra * c["lda"], 700 + i, dtype=dt)
            B = O.uniform(rb * c["ldb"], 800 + i, dtype=dt)
            C = O.uniform(rc * c["ldc"], 900 + i, dtype=dt)
            R = C.copy()
            O.gemm(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A, c["lda"], B, c["ldb"],
                   c["beta"], R, c["ldc"], kernel="default")
            call = G.cblas_sgemm if dt == np.float32 else G.cblas_dgemm
            call(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A, c["lda"], B, c["ldb"],
                 c["beta"], C, c["ldc"])
            if dt == np.float64:
                assert blaze_equal(R, C, 1e-8).all(), c
            else:
                scale = max(1.0, float(np.max(np.abs(R))))
                assert float(np.max(np.abs(C.astype(np.float64) - R.astype(np.float64)))) <= \
                    c["k"] * 2.0 ** -22 * scale + 1e-6, c
    finally:
        G.lib().gb300_set_default_method(prev)


# ---- the reference's own operation test (blazetest dmatdmatmult/MDaMDa.cpp in BLAS and debug mode) ---
BLAZETEST_CALLS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blazetest_mdamda_calls.txt")


@pytest.mark.parametrize("method", [G.METHOD_AUTO, G.METHOD_NATIVE, G.METHOD_SPLIT])
def test_replay_blazetest_operation_test_calls(method):
    lines = open(BLAZETEST_CALLS).read().splitlines()
    assert len(lines) == 288
    prev = G.lib().gb300_set_default_method(method)
    try:
        for i, ln in enumerate(lines):
            f = ln.split()
            c = dict(order=int(f[1]), ta=int(f[2]), tb=int(f[3]), m=int(f[4]), n=int(f[5]), k=int(f[6]),
                     alpha=float(f[7]), lda=int(f[8]), ldb=int(f[9]), beta=float(f[10]), ldc=int(f[11]))
            ra, _ = stored_dims(c["order"], c["ta"], c["m"], c["k"])
            rb, _ = stored_dims(c["order"], c["tb"], c["k"], c["n"])
            rc, _ = stored_dims(c["order"], O.NO_TRANS, c["m"], c["n"])
            A = O.uniform(max(ra * c["lda"], 1), 1100 + i)
            B = O.uniform(max(rb * c["ldb"], 1), 1200 + i)
            C = O.uniform(max(rc * c["ldc"], 1), 1300 + i)
            R = C.copy()
            O.gemm(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A, c["lda"], B, c["ldb"],
                   c["beta"], R, c["ldc"], kernel="default")
            G.cblas_dgemm(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A, c["lda"], B,
                          c["ldb"], c["beta"], C, c["ldc"])
            assert blaze_equal(R, C, 1e-8).all(), c
    finally:
        G.lib().gb300_set_default_method(prev)


# ---- Blaze's OpenMP evaluation (BLAZE_BLAS_IS_PARALLEL=0): concurrent tile calls inside the operands
SMP_CALLS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blaze_smp_calls.txt")


def test_replay_openmp_tile_calls_concurrently():
    """Each product's tile calls, as Blaze's OpenMP layer made them (offset pointers inside the
    whole matrices, their leading dimensions), issued at once from as many host threads; the
    assembled C against the same calls through the oracle's restatement of Blaze's kernel."""
    import threading

    products, cur = [], None
    for ln in open(SMP_CALLS).read().splitlines():
        f = ln.split()
        if f[0] == "product":
            cur = []
            products.append(cur)
            continue
        cur.append(dict(order=int(f[1]), ta=int(f[2]), tb=int(f[3]), m=int(f[4]), n=int(f[5]), k=int(f[6]),
                        alpha=float(f[7]), lda=int(f[8]), ldb=int(f[9]), beta=float(f[10]), ldc=int(f[11]),
                        offA=int(f[12]), offB=int(f[13]), offC=int(f[14])))
    assert len(products) == 5 and all(len(p) == 4 for p in products)
    for q, tiles in enumerate(products):
        def extent(c, which):
            if which == "A":
                r, _ = stored_dims(c["order"], c["ta"], c["m"], c["k"])
                return c["offA"] + r * c["lda"]
            if which == "B":
                r, _ = stored_dims(c["order"], c["tb"], c["k"], c["n"])
                return c["offB"] + r * c["ldb"]
            r, _ = stored_dims(c["order"], O.NO_TRANS, c["m"], c["n"])
            return c["offC"] + r * c["ldc"]
        A = O.uniform(max(extent(c, "A") for c in tiles), 1400 + q)
        B = O.uniform(max(extent(c, "B") for c in tiles), 1500 + q)
        C = O.uniform(max(extent(c, "C") for c in tiles), 1600 + q)
        R = C.copy()
        for c in tiles:
            O.gemm(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A[c["offA"]:], c["lda"],
                   B[c["offB"]:], c["ldb"], c["beta"], R[c["offC"]:], c["ldc"], kernel="default")
        errors = []
        start = threading.Barrier(len(tiles))

        def tile_call(c):
            try:
                start.wait()
                G.cblas_dgemm(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"],
                              A.ctypes.data + 8 * c["offA"], c["lda"], B.ctypes.data + 8 * c["offB"], c["ldb"],
                              c["beta"], C.ctypes.data + 8 * c["offC"], c["ldc"])
            except Exception as e:  # noqa: BLE001
                errors.append(e)

        threads = [threading.Thread(target=tile_call, args=(c,)) for c in tiles]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert not errors, errors
        assert blaze_equal(R, C, 1e-8).all(), q


# ---- the routines next to ?gemm, as Blaze's expressions call them (tests/golden/blaze_next_calls.txt)
NEXT_CALLS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blaze_next_calls.txt")


def _scalar(tok):
    if "," in tok:
        re_, im_ = tok.split(",")
        return complex(float(re_), float(im_))
    return float(tok)


def _mat(X, order, rows, cols, ld):
    """The rows x cols matrix stored in X (CBLAS order, leading dimension ld), as a numpy view."""
    s = X.itemsize
    if order == O.ROW_MAJOR:
        return np.lib.stride_tricks.as_strided(X, (rows, cols), (ld * s, s))
    return np.lib.stride_tricks.as_strided(X, (rows, cols), (s, ld * s))


def _op(M, t):
    return M if t == 111 else (M.T if t == 112 else M.conj().T)


def _tri(M, uplo, diag):
    T = np.tril(M) if uplo == 122 else np.triu(M)
    if diag == 132:
        np.fill_diagonal(T, 1.0)
    return T


def _vals(count, seed, kind):
    if kind == "z":
        return O.uniform(count, seed) + 1j * O.uniform(count, seed + 7919)
    v = O.uniform(count, seed)
    return v.astype(np.float32) if kind == "s" else v


def test_replay_blaze_neighbouring_calls():
    lines = open(NEXT_CALLS).read().splitlines()
    assert len(lines) == 21
    for q, ln in enumerate(lines):
        f = ln.split()
        name, kind = f[0], f[0][0]
        eps = 2.0 ** -24 if kind == "s" else 2.0 ** -53
        if name.endswith("gemv"):
            order, ta, m, n = (int(v) for v in f[1:5])
            al, lda, incx, be, incy = _scalar(f[5]), int(f[6]), int(f[7]), _scalar(f[8]), int(f[9])
            rows = m if order == O.ROW_MAJOR else n
            A = _vals(rows * lda, 400 + q, kind)
            xl, yl = (m, n) if ta != 111 else (n, m)
            x = _vals(xl * abs(incx), 500 + q, kind)
            y = _vals(yl * abs(incy), 600 + q, kind)
            ref = al * (_op(_mat(A, order, m, n, lda), ta).astype(np.complex128 if kind == "z" else np.float64)
                        @ x[::incx]) + be * y[::incy]
            if kind == "z":
                G.cblas_zgemv(order, ta, m, n, al, A, lda, x, incx, be, y, incy)
            else:
                G.cblas_gemv(order, ta, m, n, al, A, lda, x, incx, be, y, incy, dtype=kind)
            got = y[::incy]
            k = xl
        elif name.endswith("trmv"):
            order, uplo, ta, diag, n, lda, incx = (int(v) for v in f[1:8])
            A = _vals(n * lda, 400 + q, kind)
            x = _vals(n * abs(incx), 500 + q, kind)
            ref = _op(_tri(np.array(_mat(A, order, n, n, lda)), uplo, diag), ta) @ x[::incx]
            G.cblas_trmv(order, uplo, ta, diag, n, A, lda, x, incx, dtype=kind)
            got = x[::incx]
            k = n
        elif name == "dgemm":  # a real product Blaze's lowered area threshold sent to BLAS
            order, ta, tb, m, n, k = (int(v) for v in f[1:7])
            al, lda, ldb, be, ldc = float(f[7]), int(f[8]), int(f[9]), float(f[10]), int(f[11])
            A = _vals(m * lda, 400 + q, kind)
            B = _vals(k * ldb, 500 + q, kind)
            C = _vals(m * ldc, 600 + q, kind)
            ref = al * (np.array(_mat(A, order, m, k, lda)) @ np.array(_mat(B, order, k, n, ldb))) + \
                be * np.array(_mat(C, order, m, n, ldc))
            G.cblas_dgemm(order, ta, tb, m, n, k, al, A, lda, B, ldb, be, C, ldc)
            got = np.array(_mat(C, order, m, n, ldc))
        elif name.endswith("gemm"):
            order, ta, tb, m, n, k = (int(v) for v in f[1:7])
            al, lda, ldb, be, ldc = _scalar(f[7]), int(f[8]), int(f[9]), _scalar(f[10]), int(f[11])
            ra = (k if ta != 111 else m) if order == O.ROW_MAJOR else (m if ta != 111 else k)
            rb = (n if tb != 111 else k) if order == O.ROW_MAJOR else (k if tb != 111 else n)
            rc = m if order == O.ROW_MAJOR else n
            A = _vals(ra * lda, 400 + q, kind)
            B = _vals(rb * ldb, 500 + q, kind)
            C = _vals(rc * ldc, 600 + q, kind)
            sa = (k, m) if ta != 111 else (m, k)
            sb = (n, k) if tb != 111 else (k, n)
            ref = al * (_op(_mat(A, order, *sa, lda), ta) @ _op(_mat(B, order, *sb, ldb), tb)) + \
                be * np.array(_mat(C, order, m, n, ldc))
            G.cblas_zgemm(order, ta, tb, m, n, k, al, A, lda, B, ldb, be, C, ldc)
            got = np.array(_mat(C, order, m, n, ldc))
        elif "dot" in name:  # ddot, zdotu_sub, zdotc_sub
            n, incx, incy = (int(v) for v in f[1:4])
            x = _vals(n * abs(incx), 500 + q, kind)
            y = _vals(n * abs(incy), 600 + q, kind)
            xs = x[::incx].conj() if "dotc" in name else x[::incx]
            ref = np.array([np.sum(xs * y[::incy])])
            got = np.array([G.cblas_dot(n, x, incx, y, incy, dtype=kind, conj="dotc" in name)])
            k = n
        elif name.endswith("axpy"):
            n, al, incx, incy = int(f[1]), _scalar(f[2]), int(f[3]), int(f[4])
            x = _vals(n * abs(incx), 500 + q, kind)
            y = _vals(n * abs(incy), 600 + q, kind)
            ref = al * x[::incx] + y[::incy]
            G.cblas_axpy(n, al, x, incx, y, incy, dtype=kind)
            got = y[::incy]
            k = 1
        elif name.endswith("trsm"):
            order, side, uplo, ta, diag, m, n = (int(v) for v in f[1:8])
            al, lda, ldb = _scalar(f[8]), int(f[9]), int(f[10])
            ka = m if side == 141 else n
            rb = m if order == O.ROW_MAJOR else n
            A, B = O.triangular_operands(kind == "z", ka, lda, rb, ldb, 700 + q)
            want = B.copy()
            O.trsm(order, side, uplo, ta, diag, m, n, al, A, lda, want, ldb)
            G.cblas_trsm(order, side, uplo, ta, diag, m, n, al, A, lda, B, ldb, dtype=kind)
            ref, got = np.array(_mat(want, order, m, n, ldb)), np.array(_mat(B, order, m, n, ldb))
            k = ka
        else:  # trmm
            assert name.endswith("trmm"), ln
            order, side, uplo, ta, diag, m, n = (int(v) for v in f[1:8])
            al, lda, ldb = _scalar(f[8]), int(f[9]), int(f[10])
            ka = m if side == 141 else n
            A = _vals(ka * lda, 400 + q, kind)
            rb = m if order == O.ROW_MAJOR else n
            B = _vals(rb * ldb, 500 + q, kind)
            T = _op(_tri(np.array(_mat(A, order, ka, ka, lda)), uplo, diag), ta)
            B0 = np.array(_mat(B, order, m, n, ldb))
            ref = al * (T @ B0 if side == 141 else B0 @ T)
            if kind == "z":
                G.cblas_ztrmm(order, side, uplo, ta, diag, m, n, al, A, lda, B, ldb)
            else:
                G.cblas_trmm(order, side, uplo, ta, diag, m, n, al, A, lda, B, ldb, dtype=kind)
            got = np.array(_mat(B, order, m, n, ldb))
            k = ka
        scale = max(float(np.max(np.abs(ref))), 1.0)
        assert float(np.max(np.abs(got - ref))) <= 4 * k * eps * scale * 8, (q, ln)
