"""The allocation-free native product (gb300_dgemm_native_noalloc), for callers that cannot
allocate device memory themselves — e.g. a host framework that owns all device memory through its
own pool, or a loop in which cudaMalloc/cudaFree and their implicit device synchronization are not
allowed.  Its split-k scratch is a fixed array inside the library.

Checks, through the C-ABI: two calls in a row give the same result as the existing entry point
(gb300_dgemm_ex with the native method) within the tolerance the other native tests use, for a
split-k shape that uses the scratch and a column-major shape; a product whose scratch would not fit
is rejected with a clear error.  This file is collected last so that a failure here leaves every
other test already run; it also passes on its own in a fresh process."""
import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu


def _device_copy(torch, x):
    return torch.from_numpy(x).cuda()


def test_noalloc_matches_existing_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    G.lib()
    cases = [
        # (order, transA, transB, m, n, k): split-k shapes (few output tiles, long k) use the scratch
        (O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, 512, 64, 8192),
        (O.COL_MAJOR, O.TRANS, O.NO_TRANS, 300, 200, 6000),
    ]
    for call in range(2):
        for idx, (order, ta, tb, m, n, k) in enumerate(cases):
            seed = 1000 + 10 * call + idx
            if order == O.ROW_MAJOR:
                lda = m if ta == O.TRANS else k
                ldb = k if tb == O.TRANS else n
                ldc = n
            else:
                lda = k if ta == O.TRANS else m
                ldb = n if tb == O.TRANS else k
                ldc = m
            A = O.uniform(m * k, seed)
            B = O.uniform(k * n, seed + 1)
            C0 = O.uniform(m * n, seed + 2)
            alpha, beta = (1.0, 0.0) if call == 0 else (-0.75, 0.5)
            dA, dB = _device_copy(torch, A), _device_copy(torch, B)
            dC1, dC2 = _device_copy(torch, C0), _device_copy(torch, C0)
            G.dgemm_native_noalloc(order, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC1, ldc)
            G.dgemm_ex(order, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC2, ldc,
                       G.opts(method="native", residency=G.PTR_DEVICE))
            torch.cuda.synchronize()
            got, ref = dC1.cpu().numpy(), dC2.cpu().numpy()
            assert np.allclose(got, ref, rtol=1e-12, atol=1e-12), (call, idx, float(np.max(np.abs(got - ref))))
            # and against the CPU restatement of Blaze's kernel
            R = C0.copy()
            O.gemm(order, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, R, ldc)
            assert np.allclose(got, R, rtol=1e-10, atol=1e-10)


def test_noalloc_rejects_products_whose_scratch_does_not_fit():
    torch = pytest.importorskip("torch")
    m, n, k = 1024, 256, 65536  # 16 output tiles -> about 10 k-splits of 2 MiB partials each
    dA = torch.zeros(m * k, dtype=torch.float64, device="cuda")
    dB = torch.zeros(k * n, dtype=torch.float64, device="cuda")
    dC = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    with pytest.raises(G.Gb300Error) as ei:
        G.dgemm_native_noalloc(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, dA, k, dB, n, 0.0, dC, n)
    assert ei.value.status == G.ERR_INVALID_ARG
    assert "scratch" in str(ei.value)
