"""FP64-accurate products of page-locked host operands in blocks (row panels of A x column blocks of
B, copies overlapped with the computation): the result, the reported bound and the method against the
compensated FP64 oracle and against the same product of device-resident operands, for plain and
transposed operands, alpha/beta with C read back in, ragged last blocks and exact integer products."""
import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O
from helpers import normwise

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def pinned(x):
    return torch.from_numpy(np.ascontiguousarray(x)).pin_memory()


def run(order, ta, tb, m, n, k, A, lda, B, ldb, C, ldc, alpha, beta, method="auto"):
    hA, hB, hC = pinned(A), pinned(B), pinned(C)
    before = G.launch_count()
    o = G.dgemm_ex(order, ta, tb, m, n, k, alpha, hA, lda, hB, ldb, beta, hC, ldc, G.opts(method=method))
    return o, hC.numpy(), G.launch_count() - before


def device_run(order, ta, tb, m, n, k, A, lda, B, ldb, C, ldc, alpha, beta, method="auto"):
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    dC = torch.from_numpy(C.copy()).cuda()
    o = G.dgemm_ex(order, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, G.opts(method=method))
    return o, dC.cpu().numpy()


@pytest.mark.parametrize("ta,tb,n", [(O.NO_TRANS, O.NO_TRANS, 520), (O.TRANS, O.NO_TRANS, 520),
                                     (O.NO_TRANS, O.TRANS, 4400), (O.TRANS, O.TRANS, 4400)])
def test_panels_match_the_device_path_and_the_bound(ta, tb, n):
    m, k = 4608, 900  # three panels: 2048, 2048, 512 rows; n = 4400: two column blocks, 2304 + 2096
    alpha, beta = 1.25, -0.5
    lda = (m if ta == O.TRANS else k) + 3
    ldb = (k if tb == O.TRANS else n) + 1
    A = O.uniform((k if ta == O.TRANS else m) * lda, 71)
    B = O.uniform((n if tb == O.TRANS else k) * ldb, 72)
    C = O.uniform(m * n, 73)
    o, out, launches = run(O.ROW_MAJOR, ta, tb, m, n, k, A, lda, B, ldb, C.copy(), n, alpha, beta)
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


def test_pageable_host_operands_take_the_staged_path():
    m, n, k = 4608, 256, 512
    A = O.uniform(m * k, 91)
    B = O.uniform(k * n, 92)
    C = np.zeros(m * n)
    before = G.launch_count()
    o = G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method="auto"))
    assert G.launch_count() - before < 4 * 2 + 3 * 2
    P = O.product_rows_dot2(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, A, k, B, n)
    err = normwise(C.reshape(m, n), P, O.fro_norm_op(O.ROW_MAJOR, O.NO_TRANS, m, k, A, k),
                   O.fro_norm_op(O.ROW_MAJOR, O.NO_TRANS, k, n, B, n))
    assert err <= o.error_bound
