"""The golden fixtures of the neighbouring routines (Blaze's own results, tests/golden/next_golden.npz),
pinned on the CPU: each case's inputs are regenerated from their seeds and the product recomputed
with numpy in the CBLAS meaning of the arguments (storage order, transposition, conjugate
transpose, triangle and unit diagonal).  This fixes what the fixtures mean before the GPU tests
compare the library against them."""
import os

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "next_golden.npz")
CONJ = 113


@pytest.fixture(scope="module")
def golden():
    z = np.load(GOLDEN)
    return {k: z[k] for k in z.files}


def zvals(count, seed):
    re = O.uniform(max(count, 1), seed)[:count]
    im = O.uniform(max(count, 1), seed + 7919)[:count]
    return re + 1j * im


def cases(golden, prefix):
    return sorted({int(k[len(prefix):].split("_")[0]) for k in golden if k.startswith(prefix) and k.endswith("_meta")})


def mat(X, order, rows, cols, ld):
    """The rows x cols matrix stored in X (CBLAS order, leading dimension ld)."""
    if order == O.ROW_MAJOR:
        return np.array([X[i * ld:i * ld + cols] for i in range(rows)]).reshape(rows, cols)
    return np.array([X[j * ld:j * ld + rows] for j in range(cols)]).reshape(cols, rows).T


def op(M, trans):
    return M if trans == O.NO_TRANS else (M.T if trans == O.TRANS else M.conj().T)


def tri(M, uplo, diag):
    T = np.tril(M) if uplo == 122 else np.triu(M)
    if diag == 132:
        np.fill_diagonal(T, 1.0)
    return T


def close(a, b):
    return np.max(np.abs(a - b), initial=0.0) <= 1e-12 * max(1.0, np.max(np.abs(b), initial=0.0))


def test_zgemv_fixtures(golden):
    for q in cases(golden, "zgemv"):
        order, ta, m, n, lda, seed = (int(v) for v in golden[f"zgemv{q}_meta"])
        al, be = golden[f"zgemv{q}_ab"]
        r = m if order == O.ROW_MAJOR else n
        A = mat(zvals(r * lda, seed), order, m, n, lda)
        xl, yl = (m, n) if ta != O.NO_TRANS else (n, m)
        x, y = zvals(xl, seed + 1), zvals(yl, seed + 2)
        assert close(golden[f"zgemv{q}_y"], al * (op(A, ta) @ x) + be * y), q


def test_trmv_fixtures(golden):
    for q in cases(golden, "trmv"):
        cplx, order, uplo, ta, diag, n, lda, seed = (int(v) for v in golden[f"trmv{q}_meta"])
        A = zvals(n * lda, seed) if cplx else O.uniform(n * lda, seed)
        x = zvals(n, seed + 1) if cplx else O.uniform(n, seed + 1)
        T = tri(mat(A, order, n, n, lda), uplo, diag)
        assert close(golden[f"trmv{q}_x"], op(T, ta) @ x), q


def test_ztrmm_fixtures(golden):
    for q in cases(golden, "ztrmm"):
        order, side, uplo, ta, diag, m, n, lda, ldb, seed = (int(v) for v in golden[f"ztrmm{q}_meta"])
        al = complex(golden[f"ztrmm{q}_alpha"][0])
        ka = m if side == 141 else n
        rb = m if order == O.ROW_MAJOR else n
        T = tri(mat(zvals(ka * lda, seed), order, ka, ka, lda), uplo, diag)
        B0 = zvals(rb * ldb, seed + 1)
        Bm = mat(B0, order, m, n, ldb)
        ref = al * (op(T, ta) @ Bm if side == 141 else Bm @ op(T, ta))
        got = mat(golden[f"ztrmm{q}_B"], order, m, n, ldb)
        assert close(got, ref), q
        # the elements between the rows (the pitch padding) are untouched
        keep = np.ones(B0.size, bool)
        for i in range(m if order == O.ROW_MAJOR else n):
            keep[i * ldb:i * ldb + (n if order == O.ROW_MAJOR else m)] = False
        assert np.array_equal(golden[f"ztrmm{q}_B"][keep], B0[keep]), q


def test_dot_fixtures(golden):
    """Blaze's x * y and conj(x) * y against the definition (products summed in double)."""
    for q in cases(golden, "dot"):
        cplx, conj, n, seed = (int(v) for v in golden[f"dot{q}_meta"])
        x = zvals(n, seed) if cplx else O.uniform(n, seed)
        y = zvals(n, seed + 1) if cplx else O.uniform(n, seed + 1)
        want = np.sum((x.conj() if conj else x) * y)
        got = golden[f"dot{q}_r"][0]
        assert abs(got - want) <= 1e-13 * max(1.0, float(np.sum(np.abs(x) * np.abs(y)))), q


def test_axpy_fixtures(golden):
    for q in cases(golden, "axpy"):
        cplx, n, seed = (int(v) for v in golden[f"axpy{q}_meta"])
        al = golden[f"axpy{q}_alpha"][0]
        x = zvals(n, seed) if cplx else O.uniform(n, seed)
        y = zvals(n, seed + 1) if cplx else O.uniform(n, seed + 1)
        assert close(golden[f"axpy{q}_y"], al * x + y), q


def trsm_case(golden, q):
    cplx, order, side, uplo, ta, diag, m, n, lda, ldb, pad, seed = (int(v) for v in golden[f"trsm{q}_meta"])
    al = golden[f"trsm{q}_alpha"][0]
    ka = m if side == 141 else n
    rb = m if order == O.ROW_MAJOR else n
    A, X0 = O.triangular_operands(bool(cplx), ka, lda, rb, ldb, seed)
    if not cplx:
        al = float(al.real)
    return (cplx, order, side, uplo, ta, diag, m, n, lda, ldb), al, A, X0


def test_trsm_fixtures_pin_the_substitution(golden):
    """Blaze formed B = op(A) X0 (or X0 op(A)) with its own kernels; the oracle's substitution
    (orc_trsm_left) solving op(A) X = alpha B gives back alpha X0 within Blaze's relaxed equality,
    the check blazetest's BLAS operation test makes (OperationTest.h:286: A * x == b)."""
    from helpers import blaze_equal
    assert len(cases(golden, "trsm")) >= 250
    for q in cases(golden, "trsm"):
        (cplx, order, side, uplo, ta, diag, m, n, lda, ldb), al, A, X0 = trsm_case(golden, q)
        B = golden[f"trsm{q}_B"].copy()
        O.trsm(order, side, uplo, ta, diag, m, n, al, A, lda, B, ldb)
        assert blaze_equal(B, trsm_expected(order, m, n, ldb, al, X0), 1e-8).all(), q


def trsm_expected(order, m, n, ldb, al, X0):
    """alpha X0 on B's m x n elements, the padding between rows (or columns) as stored."""
    E = X0.copy()
    ii, jj = np.arange(m)[:, None], np.arange(n)[None, :]
    pos = (ii * ldb + jj) if order == O.ROW_MAJOR else (jj * ldb + ii)
    E[pos] = al * E[pos]
    return E
