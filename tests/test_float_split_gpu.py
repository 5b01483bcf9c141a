"""Float products (cblas_sgemm / gb300_sgemm_ex) through the FP64-accurate machinery: operands
widened to double, the residue form run at the float target k 2^-24, the result rounded once to
float; the reported bound adds 2^-24 for that rounding.  Checked against an FP64 reference of the
float inputs, for storage orders, transposes, ragged shapes, alpha / beta with C read, host and
device operands; the other forms requested for float run as asked; small products stay native."""
import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def stored(order, trans, rows, cols):
    t = trans != O.NO_TRANS
    r, c = (cols, rows) if t else (rows, cols)
    return (r, c) if order == O.ROW_MAJOR else (c, r)


def logical(X, order, trans, rows, cols, ld):
    r, c = stored(order, trans, rows, cols)
    M = X[: r * ld].reshape(r, ld)[:, :c].astype(np.float64)
    M = M if order == O.ROW_MAJOR else M.T  # the CBLAS matrix as stored
    return M.T if trans != O.NO_TRANS else M


@pytest.mark.parametrize("order,ta,tb,m,n,k", [(101, 111, 111, 1024, 1024, 1024), (101, 112, 111, 517, 389, 701),
                                               (102, 111, 112, 640, 900, 333), (102, 112, 112, 300, 260, 1500)])
@pytest.mark.parametrize("where", ["host", "device"])
def test_float_auto_is_fp32_accurate(order, ta, tb, m, n, k, where):
    ra, ca = stored(order, ta, m, k)
    rb, cb = stored(order, tb, k, n)
    rc, cc = stored(order, O.NO_TRANS, m, n)
    lda, ldb, ldc = ca + 3, cb + 1, cc + 2
    A = O.uniform(ra * lda, 301).astype(np.float32)
    B = O.uniform(rb * ldb, 302).astype(np.float32)
    C = O.uniform(rc * ldc, 303).astype(np.float32)
    alpha, beta = 0.75, -1.25
    ref = alpha * (logical(A, order, ta, m, k, lda) @ logical(B, order, tb, k, n, ldb)) + \
        beta * logical(C, order, O.NO_TRANS, m, n, ldc)
    if where == "device":
        dA, dB, dC = (torch.from_numpy(X).cuda() for X in (A, B, C.copy()))
        o = G.sgemm_ex(order, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, G.opts(method="auto"))
        out = dC.cpu().numpy()
    else:
        out = C.copy()
        o = G.sgemm_ex(order, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, out, ldc, G.opts(method="auto"))
    assert o.method_used == G.METHOD_SPLIT_CRT
    assert 0 < o.error_bound <= k * 2.0 ** -24 + 2.0 ** -24
    got = logical(out, order, O.NO_TRANS, m, n, ldc)
    nA = np.linalg.norm(logical(A, order, ta, m, k, lda))
    nB = np.linalg.norm(logical(B, order, tb, k, n, ldb))
    # the bound is relative to |alpha| ||A|| ||B||; beta C is added in double and rounded once
    nC = np.linalg.norm(logical(C, order, O.NO_TRANS, m, n, ldc))
    err = np.linalg.norm(got - ref) / (abs(alpha) * nA * nB + abs(beta) * nC)
    assert err <= o.error_bound, (err, o.error_bound)
    # the gap in C's pitch is left as it was
    full = out.reshape(rc, ldc)
    assert np.array_equal(full[:, cc:], C.reshape(rc, ldc)[:, cc:])


def test_float_forms_run_as_asked_and_small_stays_native():
    m = n = k = 512
    A = O.uniform(m * k, 311).astype(np.float32)
    B = O.uniform(k * n, 312).astype(np.float32)
    ref = A.reshape(m, k).astype(np.float64) @ B.reshape(k, n).astype(np.float64)
    scale = np.linalg.norm(A) * np.linalg.norm(B)
    for method, used in (("bf16x3", G.METHOD_BF16X3), ("bf16", G.METHOD_BF16), ("native", G.METHOD_NATIVE),
                         ("split_crt", G.METHOD_SPLIT_CRT)):
        C = np.zeros(m * n, np.float32)
        o = G.sgemm_ex(101, 111, 111, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method=method))
        assert o.method_used == used, method
        err = np.linalg.norm(C.reshape(m, n) - ref) / scale
        assert err <= o.error_bound, (method, err, o.error_bound)
    # a small product under auto: the native FFMA kernel
    C = np.zeros(64 * 64, np.float32)
    o = G.sgemm_ex(101, 111, 111, 64, 64, 64, 1.0, A[:4096], 64, B[:4096], 64, 0.0, C, 64, G.opts(method="auto"))
    assert o.method_used == G.METHOD_NATIVE
