"""The allocation-free native product (gb300_dgemm_native_noalloc), for callers that cannot
allocate device memory themselves — e.g. a host framework that owns all device memory through its
own pool, or a loop in which cudaMalloc/cudaFree and their implicit device synchronization are not
allowed.  Its split-k scratch is a fixed array inside the library.

Checks, through the C-ABI: two calls in a row give the same result as the existing entry point
(gb300_dgemm_ex with the native method) within the tolerance the other native tests use, for a
split-k shape that uses the scratch and a column-major shape; the second round of calls changes
neither the library's own buffers, nor torch's allocations, nor the device's free memory; a
product whose scratch would not fit is rejected with a clear error and leaves C as it was; a
device-side wait that runs out (the stall-injection hook) is reported as a timeout and the next
call is correct.  This file is collected last so that a failure here leaves every other test
already run; it also passes on its own in a fresh process."""
import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu

CASES = [
    # (order, transA, transB, m, n, k): split-k shapes (few output tiles, long k) use the scratch
    (O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, 512, 64, 8192),
    (O.COL_MAJOR, O.TRANS, O.NO_TRANS, 300, 200, 6000),
]


def _lds(order, ta, tb, m, n, k):
    if order == O.ROW_MAJOR:
        return (m if ta == O.TRANS else k), (k if tb == O.TRANS else n), n
    return (k if ta == O.TRANS else m), (n if tb == O.TRANS else k), m


def _memory_state(torch):
    torch.cuda.synchronize()
    _, free, _ = G.device_info()
    return G.pool_bytes(), torch.cuda.memory_allocated(), free


def test_noalloc_matches_existing_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    G.lib()
    # every operand of both rounds exists before the first call, so that nothing but the calls
    # themselves runs between the memory readings
    ops = []
    for call in range(2):
        for idx, (order, ta, tb, m, n, k) in enumerate(CASES):
            seed = 1000 + 10 * call + idx
            A = O.uniform(m * k, seed)
            B = O.uniform(k * n, seed + 1)
            C0 = O.uniform(m * n, seed + 2)
            dev = [torch.from_numpy(x).cuda() for x in (A, B, C0, C0)]
            ops.append((call, idx, A, B, C0, dev))
    before = None
    for call, idx, A, B, C0, (dA, dB, dC1, dC2) in ops:
        order, ta, tb, m, n, k = CASES[idx]
        lda, ldb, ldc = _lds(order, ta, tb, m, n, k)
        alpha, beta = (1.0, 0.0) if call == 0 else (-0.75, 0.5)
        if call == 1 and idx == 0:
            before = _memory_state(torch)
        G.dgemm_native_noalloc(order, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC1, ldc)
        if call == 1:
            # the second round allocates nothing anywhere
            assert _memory_state(torch) == before, (idx, before, _memory_state(torch))
        G.dgemm_ex(order, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC2, ldc,
                   G.opts(method="native", residency=G.PTR_DEVICE))
        torch.cuda.synchronize()
        got, ref = dC1.cpu().numpy(), dC2.cpu().numpy()
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-12), (call, idx, float(np.max(np.abs(got - ref))))
        # and against the CPU restatement of Blaze's kernel
        R = C0.copy()
        O.gemm(order, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, R, ldc)
        assert np.allclose(got, R, rtol=1e-10, atol=1e-10)
        if call == 1:
            before = _memory_state(torch)  # dgemm_ex may grow its own pool; the next call may not


def test_noalloc_rejects_products_whose_scratch_does_not_fit():
    torch = pytest.importorskip("torch")
    m, n, k = 1024, 256, 65536  # 16 output tiles -> about 10 k-splits of 2 MiB partials each
    dA = torch.zeros(m * k, dtype=torch.float64, device="cuda")
    dB = torch.zeros(k * n, dtype=torch.float64, device="cuda")
    C0 = O.uniform(m * n, 77)
    dC = torch.from_numpy(C0).cuda()
    with pytest.raises(G.Gb300Error) as ei:
        G.dgemm_native_noalloc(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, dA, k, dB, n, 0.0, dC, n)
    assert ei.value.status == G.ERR_INVALID_ARG
    assert "scratch" in str(ei.value)
    torch.cuda.synchronize()
    assert np.array_equal(dC.cpu().numpy(), C0), "a rejected product modified C"


def test_noalloc_reports_a_device_wait_that_ran_out_and_recovers():
    torch = pytest.importorskip("torch")
    order, ta, tb, m, n, k = CASES[0]
    lda, ldb, ldc = _lds(order, ta, tb, m, n, k)
    A = O.uniform(m * k, 91)
    B = O.uniform(k * n, 92)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dC = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    # the next native launch issues no copies, so its bounded waits run out after 20 ms
    G.lib().gb300_debug_inject_stall(1, 20_000_000)
    with pytest.raises(G.Gb300Error) as ei:
        G.dgemm_native_noalloc(order, ta, tb, m, n, k, 1.0, dA, lda, dB, ldb, 0.0, dC, ldc)
    assert ei.value.status == G.ERR_DEVICE_TIMEOUT
    # the status word in the shared array is cleared by the next call, which is correct
    G.dgemm_native_noalloc(order, ta, tb, m, n, k, 1.0, dA, lda, dB, ldb, 0.0, dC, ldc)
    torch.cuda.synchronize()
    R = np.zeros(m * n)
    O.gemm(order, ta, tb, m, n, k, 1.0, A, lda, B, ldb, 0.0, R, ldc)
    assert np.allclose(dC.cpu().numpy(), R, rtol=1e-10, atol=1e-10)
