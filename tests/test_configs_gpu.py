"""Parity at the benchmark configurations, on a GB300, through the C-ABI.

1. Plain FP64 C = A*B, M = N = K = 1024, row-major, uniform [-1,1] from a seeded mt19937: the
   native and the FP64-accurate forms against the oracle's restatement of Blaze's blocked kernel
   (``mmm``, blaze/math/dense/MMM.h:105-600; pinned to Blaze itself by tests/test_oracle.py) within
   Blaze's relaxed equality (blaze/math/shims/Equal.h:214-223, 1e-8), and normwise against the
   compensated (Dot2) oracle within k*2^-53.  The drop-in call (cblas_dgemm on host memory) too.
2. M = N = K in {4096, 8192, 16384}, row-major x row-major and row-major x column-major
   (DMatTDMatMultExpr.h:13222, CBLAS NoTrans x Trans), uniform and exponent-spread inputs:
   normwise error on sampled rows against Dot2 within the reported a-priori bound and within
   k*2^-53; the native kernel at 4096 and 8192; the digit form with 3..8 slices, BF16x3 and BF16
   within their stated bounds at 4096.
3. The full batch of 10,000 uneven products (M, N, K log-uniform in [4, 256]), FP64 and FP32,
   through one captured grouped plan, every product against the oracle's restatement of Blaze's
   default kernel (DMatDMatMultExpr.h:590-681).
4. (M,K,N) = (65536,256,256), (256,65536,256), (4096,4096,64) with a column-major A
   (TDMatTDMatMultExpr.h:559-566 and TDMatDMatMultExpr.h:540-548), native and FP64-accurate,
   every element against the oracle's blocked kernel (Blaze's relaxed equality) and normwise
   against Dot2.

Large results are checked on sampled rows so that each case needs a few seconds of CPU time."""
from __future__ import annotations

import os

import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O
from batched import build, reference
from helpers import BLAZE_ACC, blaze_equal, stored_dims

pytestmark = pytest.mark.gpu

U53 = 2.0 ** -53
NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    G.lib()
    G.device_info()
    return t


def operands(order, ta, tb, m, n, k, dist, seed):
    ra, ca = stored_dims(order, ta, m, k)
    rb, cb = stored_dims(order, tb, k, n)
    gen = O.uniform if dist == "uniform" else O.spread
    return gen(ra * ca, seed), ca, gen(rb * cb, seed + 1), cb


def sample_rows(m, count):
    return np.unique(np.linspace(0, m - 1, min(m, count)).astype(np.int64))


def sampled_error(order, ta, tb, m, n, k, A, lda, B, ldb, rows, C_rows):
    """Normwise error ||C - C_ref||_F / (||A||_F ||B||_F) estimated from the sampled rows of
    op(A)op(B) (logical row-major rows of C), scaled by sqrt(m / rows)."""
    P = O.product_rows_dot2(order, ta, tb, m, n, k, A, lda, B, ldb, rows=rows, nthreads=NT)
    d = np.asarray(C_rows, np.float64) - P
    nA, nB = float(np.linalg.norm(A)), float(np.linalg.norm(B))
    return float(np.sqrt(np.sum(d * d) * m / len(rows))) / (nA * nB)


def logical_rows(order, m, n, C, ldc, rows):
    """Rows `rows` of the logical m x n result stored in C (numpy or a device tensor)."""
    if order == O.ROW_MAJOR:
        if hasattr(C, "cpu"):
            return C.view(m, ldc)[rows][:, :n].cpu().numpy()
        return C.reshape(m, ldc)[rows][:, :n]
    if hasattr(C, "cpu"):
        return C.view(n, ldc)[:, rows].cpu().numpy().T
    return C.reshape(n, ldc)[:, rows].T


def device_product(torch, order, ta, tb, m, n, k, dA, lda, dB, ldb, method, slices=0):
    ldc = n if order == O.ROW_MAJOR else m
    dC = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    o = G.dgemm_ex(order, ta, tb, m, n, k, 1.0, dA, lda, dB, ldb, 0.0, dC, ldc,
                   G.opts(method=method, slices=slices, residency=G.PTR_DEVICE))
    torch.cuda.synchronize()
    return dC, ldc, o


# ---- configuration 1 -------------------------------------------------------------------------
def test_config1_1024_against_blazes_blocked_kernel(torch):
    m = n = k = 1024
    A, lda, B, ldb = operands(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, "uniform", 42)
    R = np.zeros(m * n)
    O.gemm(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, lda, B, ldb, 0.0, R, n, kernel="blocked",
           nthreads=NT)
    rows = sample_rows(m, 64)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    for method in ("native", "split"):
        dC, ldc, o = device_product(torch, O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, dA, lda, dB, ldb, method)
        C = dC.cpu().numpy()
        ok = blaze_equal(R, C, BLAZE_ACC[np.float64])
        assert ok.all(), (method, int(np.count_nonzero(~ok)))
        err = sampled_error(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, A, lda, B, ldb, rows,
                            C.reshape(m, n)[rows])
        assert err <= k * U53, (method, err)
        if method == "split":
            assert err <= o.error_bound <= k * U53, (err, o.error_bound)
    # the drop-in call on host memory (what Blaze's BLAS mode issues for C = A * B)
    C = np.zeros(m * n)
    G.cblas_dgemm(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, lda, B, ldb, 0.0, C, n)
    assert blaze_equal(R, C, BLAZE_ACC[np.float64]).all()


# ---- configuration 2 -------------------------------------------------------------------------
SQUARE = [(s, dist, lay) for s in (4096, 8192, 16384) for dist in ("uniform", "spread") for lay in ("rr", "rc")]
_SQUARE_CACHE: dict = {}


def square_operands(torch, size, dist):
    """Host and device operands of one size and distribution, shared by both layouts (the
    row x column-major case reads the same storage as an n x k row-major B)."""
    key = (size, dist)
    if key not in _SQUARE_CACHE:
        _SQUARE_CACHE.clear()
        torch.cuda.empty_cache()
        gen = O.uniform if dist == "uniform" else O.spread
        A, B = gen(size * size, 7 + size), gen(size * size, 8 + size)
        _SQUARE_CACHE[key] = (A, B, torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda())
    return _SQUARE_CACHE[key]


@pytest.mark.parametrize("size,dist,layout", SQUARE)
def test_config2_square_fp64_accurate(torch, size, dist, layout):
    m = n = k = size
    tb = O.NO_TRANS if layout == "rr" else O.TRANS
    A, B, dA, dB = square_operands(torch, size, dist)
    lda = ldb = size
    rows = sample_rows(m, 8 if size >= 16384 else 16)
    methods = ["split"] + (["native"] if size <= 8192 else [])
    for method in methods:
        dC, ldc, o = device_product(torch, O.ROW_MAJOR, O.NO_TRANS, tb, m, n, k, dA, lda, dB, ldb, method)
        err = sampled_error(O.ROW_MAJOR, O.NO_TRANS, tb, m, n, k, A, lda, B, ldb, rows,
                            logical_rows(O.ROW_MAJOR, m, n, dC, ldc, rows))
        assert err <= k * U53, (method, err)
        if method == "split":
            assert o.method_used == G.METHOD_SPLIT_CRT
            assert err <= o.error_bound <= k * U53, (err, o.error_bound)
        del dC
    if size == 16384 and layout == "rc":
        _SQUARE_CACHE.clear()
        torch.cuda.empty_cache()


@pytest.mark.parametrize("dist", ["uniform", "spread"])
def test_config2_slice_counts_and_bf16_forms_at_4096(torch, dist):
    """The digit (Ozaki scheme I) form with 3..8 BF16 slices, BF16x3 and BF16, each within the
    bound it reports; more slices never raise the error by more than rounding noise."""
    m = n = k = 4096
    A, lda, B, ldb = operands(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, dist, 99)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    rows = sample_rows(m, 8)
    errs = {}
    for slices in range(3, 9):
        dC, ldc, o = device_product(torch, O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, dA, lda, dB, ldb,
                                    G.METHOD_SPLIT, slices)
        assert o.slices_used == slices
        err = sampled_error(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, A, lda, B, ldb, rows,
                            logical_rows(O.ROW_MAJOR, m, n, dC, ldc, rows))
        assert err <= o.error_bound, (slices, err, o.error_bound)
        errs[slices] = err
    for s in range(3, 8):
        assert errs[s + 1] <= max(errs[s], 1e-15), errs
    for method, stated in (("bf16x3", 3 * 2.0 ** -16 + k * 2.0 ** -24), ("bf16", 2 * 2.0 ** -8 + k * 2.0 ** -24)):
        dC, ldc, o = device_product(torch, O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, dA, lda, dB, ldb, method)
        assert o.method_used == G.METHODS[method]
        err = sampled_error(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, A, lda, B, ldb, rows,
                            logical_rows(O.ROW_MAJOR, m, n, dC, ldc, rows))
        assert err <= o.error_bound <= stated * 1.0001, (method, err, o.error_bound, stated)


# ---- configuration 3 -------------------------------------------------------------------------
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_config3_full_batch_through_the_graph_plan(torch, dtype):
    specs, A, B, C0, dA, dB, dC = build(torch, 10000, seed=2024, dtype=dtype)
    plan = G.GroupedPlan(G.problems(specs), 8 if dtype == np.float64 else 4)
    plan.run()
    G.synchronize()
    got = dC.cpu().numpy()
    plan.close()
    ref = reference(specs, A, B, C0)
    bad = []
    for q, sp in enumerate(specs):
        sl = slice(sp["offC"], sp["offC"] + sp["rc"] * sp["ldc"])
        if dtype == np.float64:
            ok = blaze_equal(ref[sl], got[sl], BLAZE_ACC[np.float64]).all()
        else:
            err = np.max(np.abs(got[sl].astype(np.float64) - ref[sl].astype(np.float64)), initial=0.0)
            ok = err <= max(sp["k"], 1) * 2.0 ** -21 * 4
        if not ok:
            bad.append(q)
    assert not bad, f"{len(bad)} of {len(specs)} products differ, first {specs[bad[0]]}"


# ---- configuration 4 -------------------------------------------------------------------------
RECT = [(65536, 256, 256), (256, 65536, 256), (4096, 4096, 64)]


@pytest.mark.parametrize("m,k,n", RECT)
@pytest.mark.parametrize("layout", ["tdmat_tdmat", "tdmat_dmat"])
def test_config4_rectangular_column_major_a(torch, m, k, n, layout):
    # tdmat_tdmat: A, B and C column-major; tdmat_dmat: A column-major, B and C row-major
    order, ta = (O.COL_MAJOR, O.NO_TRANS) if layout == "tdmat_tdmat" else (O.ROW_MAJOR, O.TRANS)
    tb = O.NO_TRANS
    A, lda, B, ldb = operands(order, ta, tb, m, n, k, "uniform", 5 + m + n)
    ldc = n if order == O.ROW_MAJOR else m
    R = np.zeros(m * n)
    O.gemm(order, ta, tb, m, n, k, 1.0, A, lda, B, ldb, 0.0, R, ldc, kernel="blocked", nthreads=NT)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    rows = sample_rows(m, 16)
    for method in ("native", "split"):
        dC, _, o = device_product(torch, order, ta, tb, m, n, k, dA, lda, dB, ldb, method)
        C = dC.cpu().numpy()
        ok = blaze_equal(R, C, BLAZE_ACC[np.float64])
        assert ok.all(), (method, int(np.count_nonzero(~ok)))
        err = sampled_error(order, ta, tb, m, n, k, A, lda, B, ldb, rows, logical_rows(order, m, n, C, ldc, rows))
        assert err <= k * U53, (method, err)
        if method == "split":
            assert err <= o.error_bound <= k * U53, (err, o.error_bound)
