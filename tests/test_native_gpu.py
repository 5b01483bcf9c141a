"""Native FP64/FP32 kernel through the C-ABI on a GB300: parity with Blaze's own results and
with the compensated FP64 oracle, CBLAS semantics (alpha/beta, storage orders, leading
dimensions, beta == 0 not reading C), device-resident operands, concurrency and failure reporting."""
import threading

import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O
from helpers import check_result, golden_inputs, load_golden, normwise, stored_dims

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    L = G.lib()
    G.device_info()  # raises if no device
    return L


def run_cblas(c, A, B, C, method=None):
    f = G.cblas_dgemm if c["dtype"] == np.float64 else G.cblas_sgemm
    if method is None:
        f(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A, c["lda"], B, c["ldb"], c["beta"], C,
          c["ldc"])
    else:
        fx = G.dgemm_ex if c["dtype"] == np.float64 else G.sgemm_ex
        fx(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A, c["lda"], B, c["ldb"], c["beta"], C,
           c["ldc"], G.opts(method=method))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_golden_cases_native(dtype):
    """Every golden case (Blaze's own outputs), through cblas_?gemm with the native kernel."""
    prev = G.lib().gb300_set_default_method(G.METHOD_NATIVE)
    try:
        n_run = 0
        for c in load_golden():
            if c["dtype"] != dtype:
                continue
            A, B, C = golden_inputs(c)
            C0 = C.copy()
            run_cblas(c, A, B, C)
            check_result(c, C, c["C_ref"], C0)
            n_run += 1
        assert n_run > 0
    finally:
        G.lib().gb300_set_default_method(prev)


def _layouts():
    return [(o, a, b) for o in (O.ROW_MAJOR, O.COL_MAJOR) for a in (O.NO_TRANS, O.TRANS) for b in (O.NO_TRANS, O.TRANS)]


@pytest.mark.parametrize("order,ta,tb", _layouts())
def test_larger_shapes_normwise_vs_dot2(order, ta, tb):
    """1000-ish shapes crossing tile edges: normwise error against the compensated oracle stays
    within the FP64 bound k*2^-53 (and elementwise within Blaze's relaxed 1e-8)."""
    m, n, k = 517, 389, 1031
    ra, ca = stored_dims(order, ta, m, k)
    rb, cb = stored_dims(order, tb, k, n)
    rc, cc = stored_dims(order, O.NO_TRANS, m, n)
    lda, ldb, ldc = ca + 4, cb + 2, cc + 6
    A = O.uniform(ra * lda, 11); B = O.uniform(rb * ldb, 12); C = O.uniform(rc * ldc, 13)
    alpha, beta = 1.5, -0.5
    C0 = C.copy()
    G.dgemm_ex(order, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, G.opts(method="native"))
    P = O.product_rows_dot2(order, ta, tb, m, n, k, A, lda, B, ldb)
    Cl0 = O.logical(order, O.NO_TRANS, m, n, C0, ldc)
    ref = alpha * P + beta * Cl0
    out = O.logical(order, O.NO_TRANS, m, n, C, ldc)
    nA = O.fro_norm_op(order, ta, m, k, A, lda); nB = O.fro_norm_op(order, tb, k, n, B, ldb)
    err = normwise(out - beta * Cl0, ref - beta * Cl0, nA, nB) / abs(alpha)
    assert err <= k * 2.0 ** -53, err
    assert np.all(np.abs(out - ref) <= np.maximum(1e-8, 1e-8 * np.abs(ref)))


@pytest.mark.parametrize("m,n,k", [(4096, 64, 4096), (128, 256, 20000), (100, 3, 9000)])
def test_split_k_shapes(m, n, k):
    """Skinny shapes that use split-k (fixed-order reduction): normwise within k*2^-53."""
    A = O.uniform(m * k, 21); B = O.uniform(k * n, 22); C = np.empty(m * n)
    G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method="native"))
    rows = np.arange(0, m, max(1, m // 64))
    P = O.product_rows_dot2(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, A, k, B, n, rows=rows)
    got = C.reshape(m, n)[rows]
    nA = O.fro_norm_op(O.ROW_MAJOR, O.NO_TRANS, m, k, A, k) * np.sqrt(len(rows) / m)
    nB = O.fro_norm_op(O.ROW_MAJOR, O.NO_TRANS, k, n, B, n)
    assert normwise(got, P, nA, nB) <= k * 2.0 ** -53


def test_beta_zero_does_not_read_c():
    m = n = k = 200
    A = O.uniform(m * k, 1); B = O.uniform(k * n, 2)
    C = np.full(m * n, np.nan)
    G.cblas_dgemm(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n)
    assert np.isfinite(C).all()


def test_alpha_zero_and_k_zero_scale_c():
    m, n = 70, 90
    C = O.uniform(m * n, 3); C0 = C.copy()
    A = O.uniform(m * 5, 4); B = O.uniform(5 * n, 5)
    G.cblas_dgemm(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, 5, 0.0, A, 5, B, n, 2.0, C, n)
    assert np.array_equal(C, 2.0 * C0)
    G.cblas_dgemm(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, 0, 1.0, A, 1, B, n, 0.0, C, n)
    assert np.all(C == 0.0)


def test_odd_leading_dimensions_and_offsets():
    """Unaligned bases and odd leading dimensions (unpadded CustomMatrix) go through realignment."""
    m, n, k = 131, 77, 65
    buf = O.uniform(1 + m * (k + 1), 7)
    A = buf[1:]  # 8-byte aligned only
    B = O.uniform(k * (n + 1), 8)
    C = np.zeros(m * (n + 3))
    G.cblas_dgemm(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k + 1, B, n + 1, 0.0, C, n + 3)
    ref = O.logical(O.ROW_MAJOR, O.NO_TRANS, m, k, np.ascontiguousarray(A), k + 1) @ \
        O.logical(O.ROW_MAJOR, O.NO_TRANS, k, n, B, n + 1)
    got = O.logical(O.ROW_MAJOR, O.NO_TRANS, m, n, C, n + 3)
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-12)


def test_device_resident_operands_and_stream():
    torch = pytest.importorskip("torch")
    m, n, k = 640, 384, 512
    A = O.uniform(m * k, 31); B = O.uniform(k * n, 32)
    dA = torch.from_numpy(A).cuda(); dB = torch.from_numpy(B).cuda()
    dC = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    before = G.launch_count()
    o = G.opts(method="native", residency=G.PTR_DEVICE, stream=s.cuda_stream, synchronous=False)
    G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, dA, k, dB, n, 0.0, dC, n, o)
    torch.cuda.synchronize()
    assert G.launch_count() > before
    ref = A.reshape(m, k) @ B.reshape(k, n)
    assert np.allclose(dC.cpu().numpy().reshape(m, n), ref, rtol=1e-12, atol=1e-12)


def test_concurrent_callers_are_serialized_correctly():
    """Blaze's SMP layer may call cblas_dgemm from several threads at once."""
    m = n = k = 300
    A = [O.uniform(m * k, 40 + i) for i in range(6)]
    B = [O.uniform(k * n, 50 + i) for i in range(6)]
    C = [np.zeros(m * n) for _ in range(6)]
    errs = []

    def work(i):
        try:
            for _ in range(3):
                G.cblas_dgemm(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A[i], k, B[i], n, 0.0, C[i], n)
        except Exception as e:  # noqa: BLE001
            errs.append(e)

    th = [threading.Thread(target=work, args=(i,)) for i in range(6)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs
    for i in range(6):
        assert np.allclose(C[i].reshape(m, n), A[i].reshape(m, k) @ B[i].reshape(k, n), rtol=1e-12, atol=1e-12)


def test_stalled_pipeline_reports_timeout_and_context_survives():
    """A launch whose TMA producer never arrives ends by its bounded waits with
    GB300_ERR_DEVICE_TIMEOUT; the next call on the same context is correct."""
    m = n = k = 256
    A = O.uniform(m * k, 61); B = O.uniform(k * n, 62); C = np.zeros(m * n)
    G.lib().gb300_debug_inject_stall(1, 20_000_000)
    with pytest.raises(G.Gb300Error) as ei:
        G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method="native"))
    assert ei.value.status == G.ERR_DEVICE_TIMEOUT
    G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method="native"))
    assert np.allclose(C.reshape(m, n), A.reshape(m, k) @ B.reshape(k, n), rtol=1e-12, atol=1e-12)


def test_sgemm_larger_normwise():
    m, n, k = 300, 520, 700
    A = O.uniform(m * k, 71, dtype=np.float32); B = O.uniform(k * n, 72, dtype=np.float32)
    C = np.zeros(m * n, dtype=np.float32)
    G.cblas_sgemm(O.ROW_MAJOR, O.NO_TRANS, O.TRANS, m, n, k, 1.0, A, k, B, k, 0.0, C, n)
    ref = A.astype(np.float64).reshape(m, k) @ B.astype(np.float64).reshape(n, k).T
    err = normwise(C.reshape(m, n), ref, float(np.linalg.norm(A.astype(np.float64))), float(np.linalg.norm(B.astype(np.float64))))
    assert err <= k * 2.0 ** -24


@pytest.mark.parametrize("ta", [O.NO_TRANS, O.TRANS])
@pytest.mark.parametrize("tb", [O.NO_TRANS, O.TRANS])
@pytest.mark.parametrize("m,n,k", [(300, 520, 700), (520, 60, 900), (50, 530, 800)])
def test_sgemm_native_every_layout_and_tile(ta, tb, m, n, k):
    """The float kernel reads its shared-memory tiles with 128-bit loads in a layout-dependent
    way (k, row or column chunks); every transposition and the three tile shapes (C with at most
    64 columns, at most 64 rows, or neither) against an FP64 product."""
    A = O.uniform(m * k, 81, dtype=np.float32)
    B = O.uniform(k * n, 82, dtype=np.float32)
    C = np.full(m * n, np.nan, dtype=np.float32)
    lda = m if ta == O.TRANS else k
    ldb = k if tb == O.TRANS else n
    G.sgemm_ex(O.ROW_MAJOR, ta, tb, m, n, k, 1.0, A, lda, B, ldb, 0.0, C, n, G.opts(method="native"))
    opA = A.astype(np.float64).reshape(k, m).T if ta == O.TRANS else A.astype(np.float64).reshape(m, k)
    opB = B.astype(np.float64).reshape(n, k).T if tb == O.TRANS else B.astype(np.float64).reshape(k, n)
    ref = opA @ opB
    err = normwise(C.reshape(m, n), ref, float(np.linalg.norm(A.astype(np.float64))),
                   float(np.linalg.norm(B.astype(np.float64))))
    assert err <= k * 2.0 ** -24, err
    assert np.max(np.abs(C.reshape(m, n) - ref)) <= k * 2.0 ** -22
