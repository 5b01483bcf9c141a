"""FP64-accurate products of host operands, page-locked or pageable, in blocks (row panels of A x
column blocks of B, copies overlapped with the computation): the result, the reported bound and the
method against the compensated FP64 oracle and against the same product of device-resident operands,
for plain and transposed operands, alpha/beta with C read back in, ragged last blocks and exact
integer products; a product of a single panel takes the staged path."""
import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O
from helpers import normwise

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def pinned(x):
    return torch.from_numpy(np.ascontiguousarray(x)).pin_memory()


def run(order, ta, tb, m, n, k, A, lda, B, ldb, C, ldc, alpha, beta, method="auto", memory="pinned"):
    if memory == "pinned":
        hA, hB, hC = pinned(A), pinned(B), pinned(C)
    else:  # plain numpy arrays: pageable memory, as Blaze's matrices are
        hA, hB, hC = np.ascontiguousarray(A), np.ascontiguousarray(B), np.ascontiguousarray(C).copy()
    before = G.launch_count()
    o = G.dgemm_ex(order, ta, tb, m, n, k, alpha, hA, lda, hB, ldb, beta, hC, ldc, G.opts(method=method))
    out = hC.numpy() if memory == "pinned" else hC
    return o, out, G.launch_count() - before


def device_run(order, ta, tb, m, n, k, A, lda, B, ldb, C, ldc, alpha, beta, method="auto"):
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    dC = torch.from_numpy(C.copy()).cuda()
    o = G.dgemm_ex(order, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, G.opts(method=method))
    return o, dC.cpu().numpy()


@pytest.mark.parametrize("memory", ["pinned", "pageable"])
@pytest.mark.parametrize("ta,tb,n", [(O.NO_TRANS, O.NO_TRANS, 520), (O.TRANS, O.NO_TRANS, 520),
                                     (O.NO_TRANS, O.TRANS, 4400), (O.TRANS, O.TRANS, 4400),
                                     (O.NO_TRANS, O.NO_TRANS, 6500), (O.TRANS, O.NO_TRANS, 8800)])
def test_panels_match_the_device_path_and_the_bound(ta, tb, n, memory):
    # three panels: 2048, 2048, 512 rows; two column blocks: n = 4400 2304 + 2096, n = 6500
    # 3328 + 3172, n = 8800 4608 + 4192
    m, k = 4608, 900
    alpha, beta = 1.25, -0.5
    lda = (m if ta == O.TRANS else k) + 3
    ldb = (k if tb == O.TRANS else n) + 1
    A = O.uniform((k if ta == O.TRANS else m) * lda, 71)
    B = O.uniform((n if tb == O.TRANS else k) * ldb, 72)
    C = O.uniform(m * n, 73)
    o, out, launches = run(O.ROW_MAJOR, ta, tb, m, n, k, A, lda, B, ldb, C.copy(), n, alpha, beta, memory=memory)
    assert o.method_used == G.METHOD_SPLIT_CRT
    assert launches >= 4 * 3 + 3 * 3  # per panel: statistics, scaling, slicing; per block: three more
    od, ref_dev = device_run(O.ROW_MAJOR, ta, tb, m, n, k, A, lda, B, ldb, C, n, alpha, beta)
    P = O.product_rows_dot2(O.ROW_MAJOR, ta, tb, m, n, k, A, lda, B, ldb)
    nA = O.fro_norm_op(O.ROW_MAJOR, ta, m, k, A, lda)
    nB = O.fro_norm_op(O.ROW_MAJOR, tb, k, n, B, ldb)
    res = (out.reshape(m, n) - beta * C.reshape(m, n)) / alpha
    err = normwise(res, P, nA, nB)
    assert 0 < o.error_bound <= k * 2.0 ** -53
    assert err <= o.error_bound, (err, o.error_bound)
    # the device path rounds A with one exponent for all rows; both meet their bounds, so they agree
    # to the sum of the two
    diff = normwise(out.reshape(m, n), ref_dev.reshape(m, n), nA * abs(alpha), nB)
    assert diff <= o.error_bound + od.error_bound


def test_panels_are_exact_on_integer_products():
    m, n, k = 4352, 256, 3000
    A = O.integers(m * k, 81, -1000, 1000)
    B = O.integers(k * n, 82, -1000, 1000)
    C = np.zeros(m * n)
    o, out, launches = run(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, A, k, B, n, C, n, 1.0, 0.0)
    assert o.method_used == G.METHOD_SPLIT_CRT and launches >= 4 * 2 + 3 * 2
    exact = A.astype(np.int64).reshape(m, k) @ B.astype(np.int64).reshape(k, n)
    assert np.array_equal(out.reshape(m, n), exact.astype(np.float64))


def test_pageable_column_major_with_beta_a_pitched_c_and_a_single_panel():
    # column-major: the logical row-major product is C^T = B^T A^T, so the panels run over n
    m, n, k = 700, 4400, 640
    A = O.uniform(m * k, 91)  # column-major m x k, lda = m
    B = O.uniform(k * n, 92)  # column-major k x n, ldb = k
    C = O.uniform(m * n, 93)  # column-major m x n, ldc = m
    o, out, launches = run(O.COL_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, A, m, B, k, C.copy(), m, 2.0, 0.5,
                           memory="pageable")
    assert o.method_used == G.METHOD_SPLIT_CRT and launches >= 4 * 3 + 3 * 3
    ref = 2.0 * (A.reshape(k, m).T @ B.reshape(n, k).T) + 0.5 * C.reshape(n, m).T
    got = out.reshape(n, m).T
    scale = 2.0 * np.linalg.norm(A) * np.linalg.norm(B)
    assert np.linalg.norm(got - ref) / scale <= 2 * k * 2.0 ** -53
    # pageable C with a pitch above n: C goes back per block through pitched copies, the gap between
    # the rows is left as it was
    m2, n2, k2, ldc2 = 4608, 4400, 300, 4405
    A2 = O.uniform(m2 * k2, 95)
    B2 = O.uniform(k2 * n2, 96)
    C2 = np.full(m2 * ldc2, 7.0)
    o2, out2, launches2 = run(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m2, n2, k2, A2, k2, B2, n2, C2, ldc2, 1.0, 0.0,
                              memory="pageable")
    assert o2.method_used == G.METHOD_SPLIT_CRT and launches2 >= 4 * 3 + 3 * 6
    got2 = out2.reshape(m2, ldc2)
    assert np.all(got2[:, n2:] == 7.0)
    ref2 = A2.reshape(m2, k2) @ B2.reshape(k2, n2)
    assert np.linalg.norm(got2[:, :n2] - ref2) / (np.linalg.norm(A2) * np.linalg.norm(B2)) <= 2 * k2 * 2.0 ** -53
    # one panel (m < 4096 rows in the logical form): the staged path, same accuracy contract
    m1 = 2000
    A1 = O.uniform(m1 * k, 94)
    C1 = np.zeros(m1 * 256)
    o1, out1, launches1 = run(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m1, 256, k, A1, k, B[:k * 256], 256, C1, 256,
                              1.0, 0.0, memory="pageable")
    assert launches1 < 4 * 2 + 3 * 2
    P = O.product_rows_dot2(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m1, 256, k, A1, k, B[:k * 256], 256)
    err = normwise(out1.reshape(m1, 256), P, O.fro_norm_op(O.ROW_MAJOR, O.NO_TRANS, m1, k, A1, k),
                   O.fro_norm_op(O.ROW_MAJOR, O.NO_TRANS, k, 256, B[:k * 256], 256))
    assert err <= o1.error_bound
