"""Calls from several host threads at once (Blaze's SMP layer calls BLAS concurrently on sub-tiles
when BLAZE_BLAS_IS_PARALLEL=0) across every path that shares library state: the overlapped host
block pipeline (its copy streams and events), the staged path, device-resident operands and the
neighbouring routines (gemv, complex gemm, trmm); and the ILP64 entry points (`_64`, 64-bit
integers, selected by BLAZE_BLAS_IS_64BIT) computing the same results as the 32-bit ones."""
import ctypes as ct
import threading

import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def zvals(count, seed):
    return O.uniform(count, seed) + 1j * O.uniform(count, seed + 7919)


def test_threads_mixing_every_path():
    m, n, k = 4608, 512, 384        # four row panels: the host block pipeline
    ms, ns, ks = 300, 200, 100      # one panel: the staged path
    jobs = []
    for t in range(8):
        kind = ("pipeline_pinned", "pipeline_pageable", "staged", "device", "gemv", "zgemm", "trmm", "staged")[t]
        jobs.append((t, kind))
    results, errs = {}, []

    def work(t, kind):
        try:
            for rep in range(2):
                seed = 1000 + 10 * t + rep
                if kind.startswith("pipeline"):
                    A = O.uniform(m * k, seed)
                    B = O.uniform(k * n, seed + 1)
                    if kind == "pipeline_pinned":
                        hA, hB = torch.from_numpy(A).pin_memory(), torch.from_numpy(B).pin_memory()
                        hC = torch.zeros(m * n, dtype=torch.float64).pin_memory()
                        G.cblas_dgemm(101, 111, 111, m, n, k, 1.0, hA, k, hB, n, 0.0, hC, n)
                        C = hC.numpy()
                    else:
                        C = np.zeros(m * n)
                        G.cblas_dgemm(101, 111, 111, m, n, k, 1.0, A, k, B, n, 0.0, C, n)
                    ref = A.reshape(m, k) @ B.reshape(k, n)
                    results[(t, rep)] = np.linalg.norm(C.reshape(m, n) - ref) / (np.linalg.norm(A) * np.linalg.norm(B))
                elif kind in ("staged", "device"):
                    A = O.uniform(ms * ks, seed)
                    B = O.uniform(ks * ns, seed + 1)
                    ref = A.reshape(ms, ks) @ B.reshape(ks, ns)
                    if kind == "device":
                        dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
                        dC = torch.zeros(ms * ns, dtype=torch.float64, device="cuda")
                        G.cblas_dgemm(101, 111, 111, ms, ns, ks, 1.0, dA, ks, dB, ns, 0.0, dC, ns)
                        C = dC.cpu().numpy()
                    else:
                        C = np.zeros(ms * ns)
                        G.cblas_dgemm(101, 111, 111, ms, ns, ks, 1.0, A, ks, B, ns, 0.0, C, ns)
                    results[(t, rep)] = np.linalg.norm(C.reshape(ms, ns) - ref) / (np.linalg.norm(A) * np.linalg.norm(B))
                elif kind == "gemv":
                    A = O.uniform(ms * ns, seed)
                    x = O.uniform(ns, seed + 1)
                    y = np.zeros(ms)
                    G.cblas_gemv(101, 111, ms, ns, 1.0, A, ns, x, 1, 0.0, y, 1)
                    ref = A.reshape(ms, ns) @ x
                    results[(t, rep)] = np.max(np.abs(y - ref)) / np.max(np.abs(ref))
                elif kind == "zgemm":
                    A = zvals(ms * ks, seed)
                    B = zvals(ks * ns, seed + 1)
                    C = np.zeros(ms * ns, np.complex128)
                    G.cblas_zgemm(101, 111, 111, ms, ns, ks, 1.0 + 0j, A, ks, B, ns, 0j, C, ns)
                    ref = A.reshape(ms, ks) @ B.reshape(ks, ns)
                    results[(t, rep)] = np.linalg.norm(C.reshape(ms, ns) - ref) / (np.linalg.norm(A) * np.linalg.norm(B))
                else:  # trmm
                    A = O.uniform(ms * ms, seed)
                    B = O.uniform(ms * ns, seed + 1)
                    Bh = B.copy()
                    G.cblas_trmm(101, 141, 122, 111, 131, ms, ns, 1.0, A, ms, Bh, ns)
                    ref = np.tril(A.reshape(ms, ms)) @ B.reshape(ms, ns)
                    results[(t, rep)] = np.linalg.norm(Bh.reshape(ms, ns) - ref) / (
                        np.linalg.norm(np.tril(A.reshape(ms, ms))) * np.linalg.norm(B))
        except Exception as e:  # noqa: BLE001
            errs.append((kind, e))

    th = [threading.Thread(target=work, args=j) for j in jobs]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert not errs, errs
    assert len(results) == 16
    for key, err in results.items():
        assert err <= 4 * 4608 * 2.0 ** -53, (key, err)


def test_ilp64_entry_points_compute():
    L = G.lib()
    I64, D, VP = ct.c_int64, ct.c_double, ct.c_void_p
    L.cblas_dgemm_64.argtypes = [ct.c_int, ct.c_int, ct.c_int, I64, I64, I64, D, VP, I64, VP, I64, D, VP, I64]
    L.cblas_dgemv_64.argtypes = [ct.c_int, ct.c_int, I64, I64, D, VP, I64, VP, I64, D, VP, I64]
    L.cblas_ztrmm_64.argtypes = [ct.c_int] * 5 + [I64, I64, VP, VP, I64, VP, I64]
    L.cblas_dtrmv_64.argtypes = [ct.c_int] * 4 + [I64, VP, I64, VP, I64]
    m, n, k = 130, 70, 90
    A = O.uniform(m * k, 1); B = O.uniform(k * n, 2)
    C32 = np.zeros(m * n); C64 = np.zeros(m * n)
    G.cblas_dgemm(101, 111, 111, m, n, k, 1.0, A, k, B, n, 0.0, C32, n)
    L.gb300_clear_error()
    L.cblas_dgemm_64(101, 111, 111, m, n, k, 1.0, A.ctypes.data, k, B.ctypes.data, n, 0.0, C64.ctypes.data, n)
    assert G.last_error()[0] == G.OK
    assert np.array_equal(C32, C64)
    x = O.uniform(k, 3); y = np.zeros(m)
    L.cblas_dgemv_64(101, 111, m, k, 1.0, A.ctypes.data, k, x.ctypes.data, 1, 0.0, y.ctypes.data, 1)
    assert G.last_error()[0] == G.OK
    assert np.allclose(y, A.reshape(m, k) @ x, rtol=1e-12, atol=1e-12)
    T = zvals(m * m, 4); Bz = zvals(m * n, 5); Bz0 = Bz.copy()
    al = np.array([0.5 - 0.25j])
    L.cblas_ztrmm_64(101, 141, 121, 113, 132, m, n, al.ctypes.data, T.ctypes.data, m, Bz.ctypes.data, n)
    assert G.last_error()[0] == G.OK
    Tu = np.triu(T.reshape(m, m))
    np.fill_diagonal(Tu, 1.0)
    ref = al[0] * (Tu.conj().T @ Bz0.reshape(m, n))
    assert np.linalg.norm(Bz.reshape(m, n) - ref) / (abs(al[0]) * np.linalg.norm(Tu) * np.linalg.norm(Bz0)) <= 4 * m * 2.0 ** -53
    xv = O.uniform(m, 6); xv0 = xv.copy()
    Am = O.uniform(m * m, 7)
    L.cblas_dtrmv_64(102, 122, 112, 131, m, Am.ctypes.data, m, xv.ctypes.data, 1)
    assert G.last_error()[0] == G.OK
    Acm = Am.reshape(m, m).T  # column-major m x m
    assert np.allclose(xv, np.tril(Acm).T @ xv0, rtol=1e-12, atol=1e-12)
    # argument checks work the same on the 64-bit entry points
    L.cblas_dgemm_64(101, 111, 111, -1, n, k, 1.0, A.ctypes.data, k, B.ctypes.data, n, 0.0, C64.ctypes.data, n)
    assert G.last_error()[0] == G.ERR_INVALID_ARG
