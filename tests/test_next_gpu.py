"""The BLAS routines next to ?gemm on Blaze's seam (cblas_?gemv, cblas_zgemm / cblas_cgemm,
cblas_?trmm) on a GB300, through the C-ABI:

- every case of tests/golden/next_golden.npz (Blaze's own results) within Blaze's relaxed equality;
- larger shapes against numpy, with the FP64-accurate normwise bound for the complex and triangular
  products (their real products run in the split form by default);
- device-resident operands used in place, negative vector strides, alpha = 0 / beta = 0 rules."""
import os

import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O
from helpers import blaze_equal

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "next_golden.npz")
ACC = 1e-8  # Blaze's relaxed accuracy for double
CONJ = 113


@pytest.fixture(scope="module")
def golden():
    z = np.load(GOLDEN)
    return {k: z[k] for k in z.files}


def zvals(count, seed):
    re = O.uniform(max(count, 1), seed)[:count]
    im = O.uniform(max(count, 1), seed + 7919)[:count]
    return re + 1j * im


def stored(order, trans, rows, cols):
    t = trans != O.NO_TRANS
    r, c = (cols, rows) if t else (rows, cols)
    return (r, c) if order == O.ROW_MAJOR else (c, r)


def cases(golden, prefix):
    return sorted({int(k[len(prefix):].split("_")[0]) for k in golden if k.startswith(prefix) and k.endswith("_meta")})


def test_gemv_matches_blaze(golden):
    for q in cases(golden, "gemv"):
        order, ta, m, n, lda, seed = (int(v) for v in golden[f"gemv{q}_meta"])
        if m == 0 or n == 0:
            # Blaze settles empty matrices itself (y = beta*y, or reset) before its BLAS kernel
            # (DMatDVecMultExpr.h:414-420, TDVecDMatMultExpr.h:416-423); CBLAS returns at once
            continue
        al, be = golden[f"gemv{q}_ab"]
        r, c = stored(order, O.NO_TRANS, m, n)
        A = O.uniform(max(r * lda, 1), seed)
        xl, yl = (m, n) if ta != O.NO_TRANS else (n, m)
        x = O.uniform(max(xl, 1), seed + 1)[:xl].copy()
        y = O.uniform(max(yl, 1), seed + 2)[:yl].copy()
        G.cblas_gemv(order, ta, m, n, float(al), A, lda, x, 1, float(be), y, 1)
        ok = blaze_equal(golden[f"gemv{q}_y"], y, ACC)
        assert ok.all(), (q, order, ta, m, n, np.max(np.abs(y - golden[f"gemv{q}_y"])))


def test_zgemm_matches_blaze(golden):
    for q in cases(golden, "zgemm"):
        order, ta, tb, m, n, k, lda, ldb, ldc, seed = (int(v) for v in golden[f"zgemm{q}_meta"])
        al, be = golden[f"zgemm{q}_ab"]
        ra, _ = stored(order, ta, m, k)
        rb, _ = stored(order, tb, k, n)
        rc, _ = stored(order, O.NO_TRANS, m, n)
        A = zvals(ra * lda, seed)
        B = zvals(rb * ldb, seed + 1)
        C = zvals(rc * ldc, seed + 2)
        G.cblas_zgemm(order, ta, tb, m, n, k, complex(al), A, lda, B, ldb, complex(be), C, ldc)
        ref = golden[f"zgemm{q}_C"]
        ok = blaze_equal(ref.real, C.real, ACC) & blaze_equal(ref.imag, C.imag, ACC)
        assert ok.all(), (q, order, ta, tb, m, n, k, np.max(np.abs(C - ref)))


def test_trmm_matches_blaze(golden):
    for q in cases(golden, "trmm"):
        order, side, uplo, ta, diag, m, n, lda, ldb, seed = (int(v) for v in golden[f"trmm{q}_meta"])
        al = float(golden[f"trmm{q}_alpha"][0])
        ka = m if side == 141 else n
        rb, _ = stored(order, O.NO_TRANS, m, n)
        A = O.uniform(ka * lda, seed)
        B = O.uniform(rb * ldb, seed + 1)
        G.cblas_trmm(order, side, uplo, ta, diag, m, n, al, A, lda, B, ldb)
        ok = blaze_equal(golden[f"trmm{q}_B"], B, ACC)
        assert ok.all(), (q, order, side, uplo, ta, diag, m, n, np.max(np.abs(B - golden[f"trmm{q}_B"])))


@pytest.mark.parametrize("order,ta", [(101, 111), (101, 112), (102, 111), (102, 112)])
def test_gemv_large_strided_and_device(order, ta):
    m, n = 3000, 2200
    A = O.uniform(m * n, 11).reshape(m, n) if order == 101 else O.uniform(m * n, 11).reshape(n, m)
    Al = A if order == 101 else A.T  # logical m x n
    opA = Al.T if ta != 111 else Al
    xl, yl = opA.shape[1], opA.shape[0]
    x = O.uniform(2 * xl, 12)
    y = O.uniform(3 * yl, 13)
    y0 = y.copy()
    lda = n if order == 101 else m
    # x with stride -2, y with stride 3
    G.cblas_gemv(order, ta, m, n, 1.5, A.ravel(), lda, x, -2, -0.5, y, 3)
    xv = x[(xl - 1) * 2::-2][:xl]  # element j of x sits at x[(xl - 1 - j) * 2] for stride -2
    ref = 1.5 * (opA @ xv) - 0.5 * y0[::3][:yl]
    assert np.allclose(y[::3][:yl], ref, rtol=1e-12, atol=1e-11)
    untouched = np.ones(3 * yl, bool)
    untouched[::3][:yl] = False
    assert np.array_equal(y[untouched], y0[untouched])
    # device-resident operands, beta = 0 ignores y's contents
    torch = pytest.importorskip("torch")
    dA = torch.from_numpy(A.ravel().copy()).cuda()
    dx = torch.from_numpy(xv.copy()).cuda()
    dy = torch.full((yl,), float("nan"), dtype=torch.float64, device="cuda")
    G.cblas_gemv(order, ta, m, n, 2.0, dA, lda, dx, 1, 0.0, dy, 1)
    assert np.allclose(dy.cpu().numpy(), 2.0 * (opA @ xv), rtol=1e-12, atol=1e-11)


@pytest.mark.parametrize("ta,tb", [(111, 111), (CONJ, 112), (112, CONJ)])
def test_zgemm_large_meets_the_fp64_bound(ta, tb):
    m, n, k = 600, 520, 700
    A = zvals(m * k, 21).reshape(m, k) if ta == 111 else zvals(m * k, 21).reshape(k, m)
    B = zvals(k * n, 22).reshape(k, n) if tb == 111 else zvals(k * n, 22).reshape(n, k)
    C = zvals(m * n, 23).reshape(m, n)
    C0 = C.copy()
    al, be = 0.75 - 0.5j, 0.25 + 1j
    G.cblas_zgemm(101, ta, tb, m, n, k, al, A.ravel(), A.shape[1], B.ravel(), B.shape[1], be, C.ravel(), n)
    op = {111: lambda X: X, 112: lambda X: X.T, CONJ: lambda X: X.conj().T}
    ref = al * (op[ta](A) @ op[tb](B)) + be * C0
    err = np.linalg.norm(C - ref) / (abs(al) * np.linalg.norm(A) * np.linalg.norm(B))
    assert err <= 4 * k * 2.0 ** -53, err


def test_cgemm_single_precision():
    m, n, k = 130, 70, 90
    A = zvals(m * k, 31).astype(np.complex64)
    B = zvals(k * n, 32).astype(np.complex64)
    C = np.zeros(m * n, np.complex64)
    G.cblas_zgemm(101, 111, 111, m, n, k, 1.0 + 0j, A, k, B, n, 0j, C, n, single=True)
    ref = A.reshape(m, k).astype(np.complex128) @ B.reshape(k, n).astype(np.complex128)
    err = np.linalg.norm(C.reshape(m, n) - ref) / (np.linalg.norm(A) * np.linalg.norm(B))
    assert err <= 4 * k * 2.0 ** -24, err


@pytest.mark.parametrize("side,uplo,ta,diag", [(141, 122, 111, 131), (142, 121, 112, 132), (141, 121, 112, 131)])
def test_trmm_large_in_place_and_device(side, uplo, ta, diag):
    m, n = 900, 700
    ka = m if side == 141 else n
    A = O.uniform(ka * ka, 41).reshape(ka, ka)
    B = O.uniform(m * n, 42).reshape(m, n)
    T = np.tril(A) if uplo == 122 else np.triu(A)
    if diag == 132:
        np.fill_diagonal(T, 1.0)
    opT = T.T if ta != 111 else T
    ref = 0.5 * (opT @ B if side == 141 else B @ opT)
    Bh = B.ravel().copy()
    G.cblas_trmm(101, side, uplo, ta, diag, m, n, 0.5, A.ravel(), ka, Bh, n)
    err = np.linalg.norm(Bh.reshape(m, n) - ref) / (0.5 * np.linalg.norm(T) * np.linalg.norm(B))
    assert err <= 4 * ka * 2.0 ** -53, err
    torch = pytest.importorskip("torch")
    dA = torch.from_numpy(A.ravel().copy()).cuda()
    dB = torch.from_numpy(B.ravel().copy()).cuda()
    G.cblas_trmm(101, side, uplo, ta, diag, m, n, 0.5, dA, ka, dB, n)
    assert np.allclose(dB.cpu().numpy(), Bh, rtol=1e-13, atol=1e-13)


def test_alpha_zero_reads_no_inputs():
    # alpha == 0: A and x / B are not read (NaN there must not leak), y / C scaled by beta
    m, n = 40, 30
    A = np.full(m * n, np.nan)
    x = np.full(n, np.nan)
    y = O.uniform(m, 51).copy()
    y0 = y.copy()
    G.cblas_gemv(101, 111, m, n, 0.0, A, n, x, 1, 2.0, y, 1)
    assert np.allclose(y, 2.0 * y0)
    Bt = O.uniform(m * n, 52).copy()
    G.cblas_trmm(101, 141, 122, 111, 131, m, n, 0.0, np.full(m * m, np.nan), m, Bt, n)
    assert np.array_equal(Bt, np.zeros(m * n))


# ---- complex gemv, trmv (real and complex), complex trmm ----------------------------------------
def test_zgemv_matches_blaze(golden):
    for q in cases(golden, "zgemv"):
        order, ta, m, n, lda, seed = (int(v) for v in golden[f"zgemv{q}_meta"])
        al, be = golden[f"zgemv{q}_ab"]
        r, _ = stored(order, O.NO_TRANS, m, n)
        A = zvals(r * lda, seed)
        xl, yl = (m, n) if ta != O.NO_TRANS else (n, m)
        x = zvals(xl, seed + 1)
        y = zvals(yl, seed + 2)
        G.cblas_zgemv(order, ta, m, n, complex(al), A, lda, x, 1, complex(be), y, 1)
        ref = golden[f"zgemv{q}_y"]
        ok = blaze_equal(ref.real, y.real, ACC) & blaze_equal(ref.imag, y.imag, ACC)
        assert ok.all(), (q, order, ta, m, n, np.max(np.abs(y - ref)))


def test_trmv_matches_blaze(golden):
    for q in cases(golden, "trmv"):
        cplx, order, uplo, ta, diag, n, lda, seed = (int(v) for v in golden[f"trmv{q}_meta"])
        A = zvals(n * lda, seed) if cplx else O.uniform(n * lda, seed)
        x = zvals(n, seed + 1) if cplx else O.uniform(n, seed + 1).copy()
        G.cblas_trmv(order, uplo, ta, diag, n, A, lda, x, 1, dtype="z" if cplx else "d")
        ref = golden[f"trmv{q}_x"]
        ok = blaze_equal(ref.real, x.real, ACC) & blaze_equal(np.imag(ref), np.imag(x), ACC)
        assert ok.all(), (q, cplx, order, uplo, ta, diag, n, np.max(np.abs(x - ref)))


def test_ztrmm_matches_blaze(golden):
    for q in cases(golden, "ztrmm"):
        order, side, uplo, ta, diag, m, n, lda, ldb, seed = (int(v) for v in golden[f"ztrmm{q}_meta"])
        al = complex(golden[f"ztrmm{q}_alpha"][0])
        ka = m if side == 141 else n
        rb, _ = stored(order, O.NO_TRANS, m, n)
        A = zvals(ka * lda, seed)
        B = zvals(rb * ldb, seed + 1)
        G.cblas_ztrmm(order, side, uplo, ta, diag, m, n, al, A, lda, B, ldb)
        ref = golden[f"ztrmm{q}_B"]
        ok = blaze_equal(ref.real, B.real, ACC) & blaze_equal(ref.imag, B.imag, ACC)
        assert ok.all(), (q, order, side, uplo, ta, diag, m, n, np.max(np.abs(B - ref)))


def _op(M, t):
    return M if t == 111 else (M.T if t == 112 else M.conj().T)


@pytest.mark.parametrize("order,ta", [(101, 111), (101, CONJ), (102, 112), (102, CONJ)])
def test_zgemv_large_strided_device_and_misaligned(order, ta):
    torch = pytest.importorskip("torch")
    m, n = 2100, 1700
    S = zvals(m * n, 61)
    Al = S.reshape(m, n) if order == 101 else S.reshape(n, m).T  # logical m x n
    opA = _op(Al, ta)
    xl, yl = opA.shape[1], opA.shape[0]
    x = zvals(2 * xl, 62)
    y = zvals(3 * yl, 63)
    y0 = y.copy()
    lda = n if order == 101 else m
    al, be = 0.5 - 1.5j, 0.25 + 0.5j
    G.cblas_zgemv(order, ta, m, n, al, S, lda, x, -2, be, y, 3)
    xv = x[(xl - 1) * 2::-2][:xl]
    ref = al * (opA @ xv) + be * y0[::3][:yl]
    assert np.allclose(y[::3][:yl], ref, rtol=1e-12, atol=1e-11)
    untouched = np.ones(3 * yl, bool)
    untouched[::3][:yl] = False
    assert np.array_equal(y[untouched], y0[untouched])
    # device operands; A and y start 8 bytes past a 16-byte boundary (copied before the kernel reads
    # them as 16-byte pairs), beta = 0 ignores y's contents
    dA = torch.from_numpy(np.concatenate([[0.0], S.view(np.float64)])).cuda()
    dx = torch.from_numpy(xv.copy()).cuda()
    dy = torch.full((2 * yl + 1,), float("nan"), dtype=torch.float64, device="cuda")
    G.cblas_zgemv(order, ta, m, n, 2.0 + 0j, dA.data_ptr() + 8, lda, dx, 1, 0j, dy.data_ptr() + 8, 1)
    got = dy.cpu().numpy()[1:].view(np.complex128)
    assert np.allclose(got, 2.0 * (opA @ xv), rtol=1e-12, atol=1e-11)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("order,uplo,ta,diag", [(101, 122, 111, 131), (101, 121, 112, 132), (102, 122, 112, 131),
                                                (102, 121, 111, 132), (101, 122, CONJ, 131)])
def test_trmv_large_strided_and_device(cplx, order, uplo, ta, diag):
    if ta == CONJ and not cplx:
        ta = 112
    torch = pytest.importorskip("torch")
    n = 3001
    S = zvals(n * n, 71) if cplx else O.uniform(n * n, 71)
    Al = S.reshape(n, n) if order == 101 else S.reshape(n, n).T
    T = np.tril(Al) if uplo == 122 else np.triu(Al)
    if diag == 132:
        np.fill_diagonal(T, 1.0)
    x = zvals(2 * n, 72) if cplx else O.uniform(2 * n, 72).copy()
    x0 = x.copy()
    xv = x0[(n - 1) * 2::-2][:n]
    G.cblas_trmv(order, uplo, ta, diag, n, S, n, x, -2, dtype="z" if cplx else "d")
    ref = _op(T, ta) @ xv
    got = x[(n - 1) * 2::-2][:n]
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-11)
    gaps = np.ones(2 * n, bool)
    gaps[(n - 1) * 2::-2] = False
    assert np.array_equal(x[gaps], x0[gaps])
    # device-resident operands, unit stride
    dS = torch.from_numpy(S.copy()).cuda()
    dx = torch.from_numpy(xv.copy()).cuda()
    G.cblas_trmv(order, uplo, ta, diag, n, dS, n, dx, 1, dtype="z" if cplx else "d")
    assert np.allclose(dx.cpu().numpy(), ref, rtol=1e-12, atol=1e-11)


@pytest.mark.parametrize("side,uplo,ta,diag", [(141, 122, 111, 131), (142, 121, CONJ, 132), (141, 121, 112, 131)])
def test_ztrmm_large_in_place_and_device(side, uplo, ta, diag):
    torch = pytest.importorskip("torch")
    m, n = 700, 520
    ka = m if side == 141 else n
    A = zvals(ka * ka, 81).reshape(ka, ka)
    B = zvals(m * n, 82).reshape(m, n)
    T = np.tril(A) if uplo == 122 else np.triu(A)
    if diag == 132:
        np.fill_diagonal(T, 1.0)
    al = 0.5 - 0.25j
    ref = al * (_op(T, ta) @ B if side == 141 else B @ _op(T, ta))
    Bh = B.ravel().copy()
    G.cblas_ztrmm(101, side, uplo, ta, diag, m, n, al, A.ravel(), ka, Bh, n)
    err = np.linalg.norm(Bh.reshape(m, n) - ref) / (abs(al) * np.linalg.norm(T) * np.linalg.norm(B))
    assert err <= 4 * ka * 2.0 ** -53, err
    dA = torch.from_numpy(A.ravel().copy()).cuda()
    dB = torch.from_numpy(B.ravel().copy()).cuda()
    G.cblas_ztrmm(101, side, uplo, ta, diag, m, n, al, dA, ka, dB, n)
    assert np.allclose(dB.cpu().numpy(), Bh, rtol=1e-13, atol=1e-13)


def test_single_precision_complex_gemv_trmv_trmm():
    m, n = 300, 200
    A = zvals(m * n, 91).astype(np.complex64)
    x = zvals(n, 92).astype(np.complex64)
    y = np.zeros(m, np.complex64)
    G.cblas_zgemv(101, 111, m, n, 1.0 + 0j, A, n, x, 1, 0j, y, 1, single=True)
    ref = A.reshape(m, n).astype(np.complex128) @ x.astype(np.complex128)
    assert np.linalg.norm(y - ref) / (np.linalg.norm(A) * np.linalg.norm(x)) <= 4 * n * 2.0 ** -24
    Tn = zvals(n * n, 93).astype(np.complex64)
    xt = zvals(n, 94).astype(np.complex64)
    xr = np.tril(Tn.reshape(n, n)).astype(np.complex128) @ xt.astype(np.complex128)
    G.cblas_trmv(101, 122, 111, 131, n, Tn, n, xt, 1, dtype="c")
    assert np.linalg.norm(xt - xr) / (np.linalg.norm(Tn) * np.linalg.norm(xr)) <= 4 * n * 2.0 ** -24
    xs = O.uniform(n, 95).astype(np.float32)
    Ts = O.uniform(n * n, 96).astype(np.float32)
    xsr = np.triu(Ts.reshape(n, n)).astype(np.float64).T @ xs.astype(np.float64)
    G.cblas_trmv(101, 121, 112, 131, n, Ts, n, xs, 1, dtype="s")
    assert np.allclose(xs, xsr, rtol=1e-4, atol=1e-4)
    B = zvals(n * 64, 97).astype(np.complex64)
    Br = np.triu(Tn.reshape(n, n)).astype(np.complex128) @ B.reshape(n, 64).astype(np.complex128)
    G.cblas_ztrmm(101, 141, 121, 111, 131, n, 64, 1.0 + 0j, Tn, n, B, 64, single=True)
    assert np.linalg.norm(B.reshape(n, 64) - Br) / (np.linalg.norm(Tn) * np.linalg.norm(B)) <= 4 * n * 2.0 ** -24


def test_complex_alpha_zero_reads_no_inputs():
    m, n = 40, 30
    y = zvals(m, 98)
    y0 = y.copy()
    nan = np.full(m * n, np.nan + 1j * np.nan)
    G.cblas_zgemv(101, 111, m, n, 0j, nan, n, np.full(n, np.nan + 0j), 1, 2.0 - 1j, y, 1)
    assert np.allclose(y, (2.0 - 1j) * y0)
    B = zvals(m * n, 99)
    G.cblas_ztrmm(101, 141, 122, 111, 131, m, n, 0j, np.full(m * m, np.nan + 0j), m, B, n)
    assert np.array_equal(B, np.zeros(m * n, np.complex128))
