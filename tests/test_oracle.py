"""The CPU oracle, pinned: generator known answers, the Blaze restatement against Blaze's own
output (golden fixtures), and the compensated reference against exact integer products."""
import numpy as np
import pytest

import oracle as O
from helpers import BLAZE_ACC, blaze_equal, golden_inputs, load_golden, logical_C


def test_mt19937_known_answer():
    # The C++ standard ([rand.predef]) requires the 10000th output of mt19937 seeded with 5489
    # to be 4123659995.
    assert int(O.mt19937_raw(5489, 10000)[-1]) == 4123659995


def test_uniform_matches_numpy_legacy_stream():
    rs = np.random.RandomState(12345)
    assert np.array_equal(O.uniform(1000, 12345, 0.0, 1.0), rs.random_sample(1000))


def test_spread_distribution_shape():
    x = O.spread(20000, 3)
    e = np.floor(np.log2(np.abs(x)))
    assert e.min() == -20 and e.max() == 20
    assert 0.45 < np.mean(x > 0) < 0.55


def test_golden_inputs_reproduce():
    for c in load_golden()[::17]:
        A, B, C0 = golden_inputs(c)
        assert np.isclose(np.sum(A, dtype=np.float64), c["sumA"], rtol=0, atol=1e-9 * max(1, A.size))
        assert np.isclose(np.sum(B, dtype=np.float64), c["sumB"], rtol=0, atol=1e-9 * max(1, B.size))
        assert np.isclose(np.sum(C0, dtype=np.float64), c["sumC0"], rtol=0, atol=1e-9 * max(1, C0.size))


@pytest.mark.parametrize("kernel", ["blocked", "default", "small"])
def test_port_matches_blaze_golden(kernel):
    """The C restatement reproduces Blaze's results (Blaze's relaxed equality for double,
    a float-rounding bound for float) on every golden case."""
    for c in load_golden():
        A, B, C = golden_inputs(c)
        O.gemm(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A, c["lda"], B, c["ldb"],
               c["beta"], C, c["ldc"], kernel=kernel)
        L = logical_C(c, C)
        R = logical_C(c, c["C_ref"])
        if c["dtype"] == np.float64:
            assert blaze_equal(R, L, 1e-12).all(), c
        else:
            assert np.max(np.abs(L - R), initial=0.0) <= 1e-5 * max(1, c["k"]), c


def test_port_matches_blaze_directly():
    if O.build_ref() is None:
        pytest.skip("reference headers are not present in this container")
    rng = np.random.default_rng(0)
    for _ in range(10):
        m, n, k = (int(v) for v in rng.integers(1, 90, 3))
        for order in (O.ROW_MAJOR, O.COL_MAJOR):
            A = O.uniform(m * k, 1); B = O.uniform(k * n, 2)
            ld = n if order == O.ROW_MAJOR else m
            C1 = np.zeros(m * n); C2 = np.zeros(m * n)
            lda = k if order == O.ROW_MAJOR else m
            ldb = n if order == O.ROW_MAJOR else k
            O.gemm(order, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, lda, B, ldb, 0.0, C1, ld)
            O.ref_gemm(order, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, lda, B, ldb, 0.0, C2, ld)
            assert blaze_equal(C2, C1, 1e-12).all()


def test_dot2_is_exact_on_integer_products():
    m, n, k = 17, 23, 300
    A = O.integers(m * k, 5, -1000, 1000)
    B = O.integers(k * n, 6, -1000, 1000)
    exact = A.astype(np.int64).reshape(m, k) @ B.astype(np.int64).reshape(k, n)
    P = O.product_rows_dot2(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, A, k, B, n)
    assert np.array_equal(P, exact.astype(np.float64))


def test_dot2_beats_plain_on_cancellation():
    # sum of x_i*y_i with heavy cancellation: plain summation loses everything, Dot2 keeps it
    k = 1001
    x = np.empty(k); y = np.ones(k)
    x[0:1000:2] = 1e16; x[1:1000:2] = -1e16; x[1000] = 1.0
    P = O.product_rows_dot2(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, 1, 1, k, x, k, y, 1)
    assert P[0, 0] == 1.0


def test_fro_norm_and_layouts():
    m, k = 13, 7
    A = O.uniform(m * k, 9)
    ref = float(np.sqrt(np.sum(A * A)))
    for order in (O.ROW_MAJOR, O.COL_MAJOR):
        for t in (O.NO_TRANS, O.TRANS):
            rows, cols = (m, k) if (order == O.ROW_MAJOR) == (t == O.NO_TRANS) else (k, m)
            # logical dims for this (order, trans) that store as the same buffer
            if order == O.ROW_MAJOR:
                lr, lc, ld = (m, k, k) if t == O.NO_TRANS else (k, m, k)
            else:
                lr, lc, ld = (k, m, k) if t == O.NO_TRANS else (m, k, k)
            assert abs(O.fro_norm_op(order, t, lr, lc, A, ld) - ref) <= 1e-14 * ref
            L = O.logical(order, t, lr, lc, A, ld)
            assert abs(float(np.sqrt(np.sum(L * L))) - ref) <= 1e-13 * ref
            del rows, cols


def test_small_kernel_sums_like_the_default_kernel():
    """Blaze's small kernel and its default kernel add each element's products in the same k
    order; their restatements agree bit for bit on every storage order and ragged shape."""
    rng = np.random.default_rng(7)
    for dt in (np.float64, np.float32):
        for _ in range(40):
            m, n, k = (int(v) for v in rng.integers(1, 140, 3))
            order = O.ROW_MAJOR if rng.integers(2) else O.COL_MAJOR
            ta = O.TRANS if rng.integers(2) else O.NO_TRANS
            tb = O.TRANS if rng.integers(2) else O.NO_TRANS
            lda = (k if ta == O.NO_TRANS else m) if order == O.ROW_MAJOR else (m if ta == O.NO_TRANS else k)
            ldb = (n if tb == O.NO_TRANS else k) if order == O.ROW_MAJOR else (k if tb == O.NO_TRANS else n)
            ldc = n if order == O.ROW_MAJOR else m
            A = O.uniform(m * k, 11, dtype=dt); B = O.uniform(k * n, 12, dtype=dt); C0 = O.uniform(m * n, 13, dtype=dt)
            alpha, beta = (1.0, 0.0) if rng.integers(2) else (-0.5, 1.5)
            C1, C2 = C0.copy(), C0.copy()
            O.gemm(order, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C1, ldc, kernel="small")
            O.gemm(order, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C2, ldc, kernel="default")
            assert np.array_equal(C1, C2), (m, n, k, order, ta, tb)


def test_small_kernel_batch_equals_the_single_products():
    import batched
    for dt in (np.float64, np.float32):
        specs, A, B, C0 = batched.host_batch(300, 21, dtype=dt, layouts=True, alphabeta=True)
        desc, ab = O.batch_descriptor(specs)
        C1 = O.gemm_batch_small(desc, ab, A, B, C0.copy(), nthreads=4)
        C2 = batched.reference(specs, A, B, C0, kernel="small")
        assert np.array_equal(C1, C2)
