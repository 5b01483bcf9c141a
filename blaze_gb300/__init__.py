"""blaze_gb300 — GB300 (sm_103a) backend for Blaze's dense matrix multiplication.

The product is the C-ABI shared library ``libgb300blas.so`` (headers in ``include/``): a drop-in
CBLAS ``cblas_dgemm``/``cblas_sgemm`` for Blaze's BLAS mode plus the extended ``gb300_*`` API.
This module is a thin ctypes binding over that library, used by the tests and the benchmark the
way Blaze's own blazetest/blazemark programs use ``blaze::gemm``.  There is no CPU path here: if
the library is missing, importing the binding raises.
"""
from __future__ import annotations

import ctypes as ct
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgb300blas.so")

# CBLAS enums (standard ABI values)
RowMajor, ColMajor = 101, 102
NoTrans, Trans, ConjTrans = 111, 112, 113

# gb300_status
OK, ERR_INVALID_ARG, ERR_CUDA, ERR_NO_MEMORY, ERR_DEVICE_TIMEOUT, ERR_NOT_SUPPORTED, ERR_NO_DEVICE, ERR_ADMISSION = range(8)
# gb300_method
METHOD_AUTO, METHOD_NATIVE, METHOD_SPLIT, METHOD_BF16X3, METHOD_BF16, METHOD_SPLIT_CRT = range(6)
METHODS = {"auto": METHOD_AUTO, "native": METHOD_NATIVE, "split": METHOD_SPLIT, "bf16x3": METHOD_BF16X3,
           "bf16": METHOD_BF16, "split_crt": METHOD_SPLIT_CRT}
# gb300_residency
PTR_DETECT, PTR_DEVICE, PTR_HOST = range(3)


class GemmOpts(ct.Structure):
    _fields_ = [
        ("method", ct.c_int),
        ("slices", ct.c_int),
        ("target_error", ct.c_double),
        ("residency", ct.c_int),
        ("stream", ct.c_void_p),
        ("synchronous", ct.c_int),
        ("method_used", ct.c_int),
        ("slices_used", ct.c_int),
        ("error_bound", ct.c_double),
    ]


class GemmProblem(ct.Structure):
    _fields_ = [
        ("order", ct.c_int), ("transA", ct.c_int), ("transB", ct.c_int),
        ("m", ct.c_int64), ("n", ct.c_int64), ("k", ct.c_int64),
        ("alpha", ct.c_double), ("beta", ct.c_double),
        ("A", ct.c_void_p), ("lda", ct.c_int64),
        ("B", ct.c_void_p), ("ldb", ct.c_int64),
        ("C", ct.c_void_p), ("ldc", ct.c_int64),
    ]


class ServerConfig(ct.Structure):
    _fields_ = [("memory_budget_bytes", ct.c_int64), ("slots", ct.c_int), ("reserve_sms", ct.c_int),
                ("aging_ms", ct.c_double), ("large_threshold", ct.c_int64), ("batch_threshold", ct.c_int64),
                ("batch_max", ct.c_int), ("large_slots", ct.c_int)]


class ServeRequest(ct.Structure):
    _fields_ = [
        ("order", ct.c_int), ("transA", ct.c_int), ("transB", ct.c_int),
        ("m", ct.c_int64), ("n", ct.c_int64), ("k", ct.c_int64),
        ("alpha", ct.c_double), ("beta", ct.c_double),
        ("A", ct.c_void_p), ("lda", ct.c_int64),
        ("B", ct.c_void_p), ("ldb", ct.c_int64),
        ("C", ct.c_void_p), ("ldc", ct.c_int64),
        ("accuracy", ct.c_int), ("target_error", ct.c_double),
    ]


class ServeResult(ct.Structure):
    _fields_ = [("status", ct.c_int), ("method_used", ct.c_int), ("slices", ct.c_int),
                ("error_bound", ct.c_double), ("queue_ms", ct.c_double), ("run_ms", ct.c_double),
                ("latency_ms", ct.c_double)]


class ServerStats(ct.Structure):
    _fields_ = [("submitted", ct.c_int64), ("completed", ct.c_int64), ("rejected", ct.c_int64),
                ("failed", ct.c_int64), ("queued", ct.c_int64),
                ("p50_ms", ct.c_double), ("p99_ms", ct.c_double), ("mean_ms", ct.c_double), ("max_ms", ct.c_double),
                ("wall_s", ct.c_double), ("tflops", ct.c_double),
                ("bytes_in_use", ct.c_int64), ("peak_bytes", ct.c_int64), ("budget_bytes", ct.c_int64),
                ("class_completed", ct.c_int64 * 3), ("class_p50_ms", ct.c_double * 3),
                ("class_p99_ms", ct.c_double * 3), ("grouped_launches", ct.c_int64),
                ("grouped_mean_batch", ct.c_double)]


class Gb300Error(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


_lib = None


def build(force: bool = False) -> str:
    from . import nvcc_build
    return nvcc_build.build(force=force)


def lib() -> ct.CDLL:
    """Load libgb300blas.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run `python -m blaze_gb300.nvcc_build` (needs nvcc)")
    L = ct.CDLL(LIB_PATH)
    I32, I64, D, F, VP = ct.c_int32, ct.c_int64, ct.c_double, ct.c_float, ct.c_void_p
    L.cblas_dgemm.argtypes = [ct.c_int, ct.c_int, ct.c_int, I32, I32, I32, D, VP, I32, VP, I32, D, VP, I32]
    L.cblas_dgemm.restype = None
    L.cblas_sgemm.argtypes = [ct.c_int, ct.c_int, ct.c_int, I32, I32, I32, F, VP, I32, VP, I32, F, VP, I32]
    L.cblas_sgemm.restype = None
    L.cblas_dgemm_64.argtypes = [ct.c_int, ct.c_int, ct.c_int, I64, I64, I64, D, VP, I64, VP, I64, D, VP, I64]
    L.cblas_dgemm_64.restype = None
    L.cblas_sgemm_64.argtypes = [ct.c_int, ct.c_int, ct.c_int, I64, I64, I64, F, VP, I64, VP, I64, F, VP, I64]
    L.cblas_sgemm_64.restype = None
    for nm, T in (("cblas_dgemv", D), ("cblas_sgemv", F)):
        getattr(L, nm).argtypes = [ct.c_int, ct.c_int, I32, I32, T, VP, I32, VP, I32, T, VP, I32]
        getattr(L, nm).restype = None
    for nm in ("cblas_zgemm", "cblas_cgemm"):
        getattr(L, nm).argtypes = [ct.c_int, ct.c_int, ct.c_int, I32, I32, I32, VP, VP, I32, VP, I32, VP, VP, I32]
        getattr(L, nm).restype = None
    for nm, T in (("cblas_dtrmm", D), ("cblas_strmm", F)):
        getattr(L, nm).argtypes = [ct.c_int] * 5 + [I32, I32, T, VP, I32, VP, I32]
        getattr(L, nm).restype = None
    for nm in ("cblas_zgemv", "cblas_cgemv"):
        getattr(L, nm).argtypes = [ct.c_int, ct.c_int, I32, I32, VP, VP, I32, VP, I32, VP, VP, I32]
        getattr(L, nm).restype = None
    for nm in ("cblas_ztrmm", "cblas_ctrmm"):
        getattr(L, nm).argtypes = [ct.c_int] * 5 + [I32, I32, VP, VP, I32, VP, I32]
        getattr(L, nm).restype = None
    for nm in ("cblas_strmv", "cblas_dtrmv", "cblas_ctrmv", "cblas_ztrmv"):
        getattr(L, nm).argtypes = [ct.c_int] * 4 + [I32, VP, I32, VP, I32]
        getattr(L, nm).restype = None
    for nm, T in (("cblas_dtrsm", D), ("cblas_strsm", F)):
        getattr(L, nm).argtypes = [ct.c_int] * 5 + [I32, I32, T, VP, I32, VP, I32]
        getattr(L, nm).restype = None
    for nm in ("cblas_ztrsm", "cblas_ctrsm"):
        getattr(L, nm).argtypes = [ct.c_int] * 5 + [I32, I32, VP, VP, I32, VP, I32]
        getattr(L, nm).restype = None
    for nm, T in (("cblas_daxpy", D), ("cblas_saxpy", F)):
        getattr(L, nm).argtypes = [I32, T, VP, I32, VP, I32]
        getattr(L, nm).restype = None
    for nm in ("cblas_zaxpy", "cblas_caxpy"):
        getattr(L, nm).argtypes = [I32, VP, VP, I32, VP, I32]
        getattr(L, nm).restype = None
    L.cblas_ddot.argtypes = [I32, VP, I32, VP, I32]
    L.cblas_ddot.restype = D
    L.cblas_sdot.argtypes = [I32, VP, I32, VP, I32]
    L.cblas_sdot.restype = F
    for nm in ("cblas_zdotu_sub", "cblas_zdotc_sub", "cblas_cdotu_sub", "cblas_cdotc_sub",
               "cblas_zdotu", "cblas_zdotc", "cblas_cdotu", "cblas_cdotc"):
        getattr(L, nm).argtypes = [I32, VP, I32, VP, I32, VP]
        getattr(L, nm).restype = None
    L.gb300_dgemm_ex.argtypes = [ct.c_int, ct.c_int, ct.c_int, I64, I64, I64, D, VP, I64, VP, I64, D, VP, I64,
                                 ct.POINTER(GemmOpts)]
    L.gb300_dgemm_ex.restype = ct.c_int
    L.gb300_sgemm_ex.argtypes = [ct.c_int, ct.c_int, ct.c_int, I64, I64, I64, F, VP, I64, VP, I64, F, VP, I64,
                                 ct.POINTER(GemmOpts)]
    L.gb300_sgemm_ex.restype = ct.c_int
    L.gb300_gemm_opts_init.argtypes = [ct.POINTER(GemmOpts)]
    L.gb300_gemm_opts_init.restype = None
    L.gb300_last_error.restype = ct.c_int
    L.gb300_last_error_message.restype = ct.c_char_p
    L.gb300_clear_error.restype = None
    L.gb300_set_default_method.argtypes = [ct.c_int]
    L.gb300_set_default_method.restype = ct.c_int
    L.gb300_device_info.argtypes = [ct.POINTER(ct.c_int), ct.POINTER(I64), ct.POINTER(I64)]
    L.gb300_device_info.restype = ct.c_int
    L.gb300_launch_count.restype = I64
    L.gb300_pool_bytes.restype = I64
    L.gb300_measure_fp64_peak.argtypes = [ct.POINTER(ct.c_double)]
    L.gb300_measure_fp64_peak.restype = ct.c_int
    L.gb300_measure_fp32_peak.argtypes = [ct.POINTER(ct.c_double)]
    L.gb300_measure_fp32_peak.restype = ct.c_int
    L.gb300_synchronize.restype = ct.c_int
    L.gb300_dgemm_native_noalloc.argtypes = [ct.c_int, ct.c_int, ct.c_int, I64, I64, I64, D, VP, I64, VP, I64, D,
                                             VP, I64, VP]
    L.gb300_dgemm_native_noalloc.restype = ct.c_int
    PP = ct.POINTER(GemmProblem)
    L.gb300_grouped_plan_create.argtypes = [ct.c_int, PP, I64, ct.POINTER(VP)]
    L.gb300_grouped_plan_create.restype = ct.c_int
    L.gb300_grouped_plan_run.argtypes = [VP, VP]
    L.gb300_grouped_plan_run.restype = ct.c_int
    L.gb300_grouped_plan_info.argtypes = [VP, ct.POINTER(I64), ct.POINTER(D), ct.POINTER(D)]
    L.gb300_grouped_plan_info.restype = ct.c_int
    L.gb300_grouped_plan_destroy.argtypes = [VP]
    L.gb300_grouped_plan_destroy.restype = None
    L.gb300_dgemm_grouped.argtypes = [PP, I64, VP]
    L.gb300_dgemm_grouped.restype = ct.c_int
    L.gb300_sgemm_grouped.argtypes = [PP, I64, VP]
    L.gb300_sgemm_grouped.restype = ct.c_int
    L.gb300_grouped_autotune.argtypes = [ct.c_int, ct.c_int]
    L.gb300_grouped_autotune.restype = ct.c_int
    L.gb300_grouped_tuning_save.argtypes = [ct.c_char_p]
    L.gb300_grouped_tuning_save.restype = ct.c_int
    L.gb300_grouped_tuning_load.argtypes = [ct.c_char_p]
    L.gb300_grouped_tuning_load.restype = ct.c_int
    L.gb300_grouped_shape_for.argtypes = [ct.c_int, I64, I64, I64, ct.POINTER(ct.c_int), ct.POINTER(ct.c_int)]
    L.gb300_grouped_shape_for.restype = ct.c_int
    L.gb300_server_config_init.argtypes = [ct.POINTER(ServerConfig)]
    L.gb300_server_config_init.restype = None
    L.gb300_server_create.argtypes = [ct.POINTER(ServerConfig), ct.POINTER(VP)]
    L.gb300_server_create.restype = ct.c_int
    L.gb300_server_submit.argtypes = [VP, ct.POINTER(ServeRequest), ct.POINTER(ct.c_uint64)]
    L.gb300_server_submit.restype = ct.c_int
    L.gb300_server_wait.argtypes = [VP, ct.c_uint64, ct.c_double, ct.POINTER(ServeResult)]
    L.gb300_server_wait.restype = ct.c_int
    L.gb300_server_poll.argtypes = [VP, ct.c_uint64, ct.POINTER(ct.c_int)]
    L.gb300_server_poll.restype = ct.c_int
    L.gb300_server_get_stats.argtypes = [VP, ct.POINTER(ServerStats)]
    L.gb300_server_get_stats.restype = ct.c_int
    L.gb300_server_reset_stats.argtypes = [VP]
    L.gb300_server_reset_stats.restype = None
    L.gb300_server_destroy.argtypes = [VP]
    L.gb300_server_destroy.restype = None
    L.gb300_select_device.argtypes = [ct.c_int]
    L.gb300_select_device.restype = ct.c_int
    L.gb300_profile_enable.argtypes = [ct.c_int]
    L.gb300_profile_enable.restype = None
    L.gb300_profile_read.argtypes = [ct.c_char_p, ct.POINTER(ct.c_double), ct.POINTER(I64)]
    L.gb300_profile_read.restype = ct.c_int
    L.gb300_debug_inject_stall.argtypes = [ct.c_int, ct.c_uint64]
    L.gb300_debug_inject_stall.restype = None
    _lib = L
    return L


def last_error() -> tuple[int, str]:
    L = lib()
    msg = L.gb300_last_error_message()
    return L.gb300_last_error(), (msg.decode() if msg else "")


def check(status: int) -> None:
    if status != OK:
        st, msg = last_error()
        raise Gb300Error(status, msg)


def opts(method: str | int = "auto", slices: int = 0, target_error: float = 0.0, residency: int = PTR_DETECT,
         stream: int | None = None, synchronous: bool = True) -> GemmOpts:
    o = GemmOpts()
    lib().gb300_gemm_opts_init(ct.byref(o))
    o.method = METHODS[method] if isinstance(method, str) else int(method)
    o.slices = slices
    o.target_error = target_error
    o.residency = residency
    o.stream = stream
    o.synchronous = 1 if synchronous else 0
    return o


def _addr(x) -> int:
    """Address of a numpy array, torch tensor or raw integer pointer."""
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data


def dgemm_ex(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, o: GemmOpts | None = None) -> GemmOpts:
    o = o if o is not None else opts()
    st = lib().gb300_dgemm_ex(order, transA, transB, m, n, k, alpha, _addr(A), lda, _addr(B), ldb, beta, _addr(C),
                              ldc, ct.byref(o))
    check(st)
    return o


def sgemm_ex(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, o: GemmOpts | None = None) -> GemmOpts:
    o = o if o is not None else opts(method="native")
    st = lib().gb300_sgemm_ex(order, transA, transB, m, n, k, alpha, _addr(A), lda, _addr(B), ldb, beta, _addr(C),
                              ldc, ct.byref(o))
    check(st)
    return o


def cblas_dgemm(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc) -> None:
    """The exact call Blaze's BLAS mode makes (32-bit integers); raises on a recorded error."""
    L = lib()
    L.gb300_clear_error()
    L.cblas_dgemm(order, transA, transB, m, n, k, alpha, _addr(A), lda, _addr(B), ldb, beta, _addr(C), ldc)
    st, msg = last_error()
    if st != OK:
        raise Gb300Error(st, msg)


def cblas_sgemm(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc) -> None:
    L = lib()
    L.gb300_clear_error()
    L.cblas_sgemm(order, transA, transB, m, n, k, alpha, _addr(A), lda, _addr(B), ldb, beta, _addr(C), ldc)
    st, msg = last_error()
    if st != OK:
        raise Gb300Error(st, msg)


def _raise_on_error():
    st, msg = last_error()
    if st != OK:
        raise Gb300Error(st, msg)


def cblas_gemv(order, transA, m, n, alpha, A, lda, x, incx, beta, y, incy, dtype="d") -> None:
    """cblas_dgemv (dtype "d") or cblas_sgemv ("s"): y = alpha op(A) x + beta y."""
    L = lib()
    L.gb300_clear_error()
    getattr(L, "cblas_%sgemv" % dtype)(order, transA, m, n, alpha, _addr(A), lda, _addr(x), incx, beta, _addr(y), incy)
    _raise_on_error()


def cblas_zgemm(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, single=False) -> None:
    """cblas_zgemm (complex128 operands) or cblas_cgemm (single=True, complex64): complex
    C = alpha op(A) op(B) + beta C, transposes 111 / 112 / 113 (conjugate)."""
    L = lib()
    import numpy as np
    ct_t = np.complex64 if single else np.complex128
    al = np.array([alpha], dtype=ct_t)
    be = np.array([beta], dtype=ct_t)
    L.gb300_clear_error()
    getattr(L, "cblas_cgemm" if single else "cblas_zgemm")(order, transA, transB, m, n, k, al.ctypes.data, _addr(A),
                                                          lda, _addr(B), ldb, be.ctypes.data, _addr(C), ldc)
    _raise_on_error()


def cblas_trmm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb, dtype="d") -> None:
    """cblas_dtrmm / cblas_strmm: B = alpha op(A) B (side 141) or alpha B op(A) (142), A triangular."""
    L = lib()
    L.gb300_clear_error()
    getattr(L, "cblas_%strmm" % dtype)(order, side, uplo, transA, diag, m, n, alpha, _addr(A), lda, _addr(B), ldb)
    _raise_on_error()


def cblas_zgemv(order, transA, m, n, alpha, A, lda, x, incx, beta, y, incy, single=False) -> None:
    """cblas_zgemv (complex128) or cblas_cgemv (single=True, complex64): complex
    y = alpha op(A) x + beta y, transposes 111 / 112 / 113 (conjugate)."""
    L = lib()
    import numpy as np
    ct_t = np.complex64 if single else np.complex128
    al = np.array([alpha], dtype=ct_t)
    be = np.array([beta], dtype=ct_t)
    L.gb300_clear_error()
    getattr(L, "cblas_cgemv" if single else "cblas_zgemv")(order, transA, m, n, al.ctypes.data, _addr(A), lda, _addr(x),
                                                          incx, be.ctypes.data, _addr(y), incy)
    _raise_on_error()


def cblas_trmv(order, uplo, transA, diag, n, A, lda, x, incx, dtype="d") -> None:
    """cblas_?trmv, dtype "s", "d", "c" or "z": x = op(A) x with A n x n triangular."""
    L = lib()
    L.gb300_clear_error()
    getattr(L, "cblas_%strmv" % dtype)(order, uplo, transA, diag, n, _addr(A), lda, _addr(x), incx)
    _raise_on_error()


def cblas_ztrmm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb, single=False) -> None:
    """cblas_ztrmm (complex128) or cblas_ctrmm (single=True, complex64): complex B = alpha op(A) B
    (side 141) or alpha B op(A) (142), A triangular."""
    L = lib()
    import numpy as np
    al = np.array([alpha], dtype=np.complex64 if single else np.complex128)
    L.gb300_clear_error()
    getattr(L, "cblas_ctrmm" if single else "cblas_ztrmm")(order, side, uplo, transA, diag, m, n, al.ctypes.data,
                                                          _addr(A), lda, _addr(B), ldb)
    _raise_on_error()


def cblas_trsm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb, dtype="d") -> None:
    """cblas_?trsm: B = alpha op(A)^-1 B (side 141) or alpha B op(A)^-1 (142), A triangular.
    dtype "d" / "s" (alpha a number) or "z" / "c" (alpha a complex number)."""
    L = lib()
    import numpy as np
    L.gb300_clear_error()
    if dtype in ("z", "c"):
        al = np.array([alpha], dtype=np.complex128 if dtype == "z" else np.complex64)
        getattr(L, "cblas_%strsm" % dtype)(order, side, uplo, transA, diag, m, n, al.ctypes.data, _addr(A), lda,
                                           _addr(B), ldb)
    else:
        getattr(L, "cblas_%strsm" % dtype)(order, side, uplo, transA, diag, m, n, alpha, _addr(A), lda, _addr(B), ldb)
    _raise_on_error()


def cblas_axpy(n, alpha, x, incx, y, incy, dtype="d") -> None:
    """cblas_?axpy: y = alpha x + y (strided; dtype "d", "s", "z" or "c")."""
    L = lib()
    import numpy as np
    L.gb300_clear_error()
    if dtype in ("z", "c"):
        al = np.array([alpha], dtype=np.complex128 if dtype == "z" else np.complex64)
        getattr(L, "cblas_%saxpy" % dtype)(n, al.ctypes.data, _addr(x), incx, _addr(y), incy)
    else:
        getattr(L, "cblas_%saxpy" % dtype)(n, alpha, _addr(x), incx, _addr(y), incy)
    _raise_on_error()


def cblas_dot(n, x, incx, y, incy, dtype="d", conj=False, sub=True):
    """The dot products: cblas_ddot / cblas_sdot (a float), or cblas_?dotu / cblas_?dotc (conj=True)
    for dtype "z" / "c" (a complex; sub=False calls the value-named form)."""
    L = lib()
    import numpy as np
    L.gb300_clear_error()
    if dtype in ("d", "s"):
        r = getattr(L, "cblas_%sdot" % dtype)(n, _addr(x), incx, _addr(y), incy)
        _raise_on_error()
        return float(r)
    out = np.zeros(1, dtype=np.complex128 if dtype == "z" else np.complex64)
    name = "cblas_%sdot%s%s" % (dtype, "c" if conj else "u", "_sub" if sub else "")
    getattr(L, name)(n, _addr(x), incx, _addr(y), incy, out.ctypes.data)
    _raise_on_error()
    return complex(out[0])


def dgemm_native_noalloc(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                         stream: int | None = None) -> None:
    """The allocation-free native product (device operands; fixed in-library scratch)."""
    check(lib().gb300_dgemm_native_noalloc(order, transA, transB, m, n, k, alpha, _addr(A), lda, _addr(B), ldb,
                                           beta, _addr(C), ldc, stream))


def problems(specs) -> ct.Array:
    """A ctypes array of GemmProblem from dicts with the CBLAS fields
    (order, transA, transB, m, n, k, alpha, beta, A, lda, B, ldb, C, ldc); pointers may be
    integers, numpy arrays or torch tensors."""
    arr = (GemmProblem * len(specs))()
    for i, sp in enumerate(specs):
        p = arr[i]
        p.order, p.transA, p.transB = sp["order"], sp["transA"], sp["transB"]
        p.m, p.n, p.k = sp["m"], sp["n"], sp["k"]
        p.alpha, p.beta = sp.get("alpha", 1.0), sp.get("beta", 0.0)
        p.A, p.lda = _addr(sp["A"]), sp["lda"]
        p.B, p.ldb = _addr(sp["B"]), sp["ldb"]
        p.C, p.ldc = _addr(sp["C"]), sp["ldc"]
    return arr


class GroupedPlan:
    """A captured grouped launch (gb300_grouped_plan_*)."""

    def __init__(self, probs, elem_bytes: int = 8):
        self.handle = ct.c_void_p()
        self._probs = probs
        check(lib().gb300_grouped_plan_create(elem_bytes, probs, len(probs), ct.byref(self.handle)))

    def run(self, stream: int | None = None) -> None:
        check(lib().gb300_grouped_plan_run(self.handle, stream))

    def info(self) -> tuple[int, float, float]:
        t, u, p = ct.c_int64(0), ct.c_double(0), ct.c_double(0)
        check(lib().gb300_grouped_plan_info(self.handle, ct.byref(t), ct.byref(u), ct.byref(p)))
        return t.value, u.value, p.value

    def close(self) -> None:
        if self.handle:
            lib().gb300_grouped_plan_destroy(self.handle)
            self.handle = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def dgemm_grouped(probs, stream: int | None = None) -> None:
    check(lib().gb300_dgemm_grouped(probs, len(probs), stream))


def sgemm_grouped(probs, stream: int | None = None) -> None:
    check(lib().gb300_sgemm_grouped(probs, len(probs), stream))


def grouped_autotune(elem_bytes: int = 8, effort: int = 1) -> None:
    check(lib().gb300_grouped_autotune(elem_bytes, effort))


def grouped_shape_for(elem_bytes: int, m: int, n: int, k: int) -> tuple[int, int, int]:
    r, c = ct.c_int(0), ct.c_int(0)
    s = lib().gb300_grouped_shape_for(elem_bytes, m, n, k, ct.byref(r), ct.byref(c))
    return s, r.value, c.value


class Server:
    """Continuous-batching request server (gb300_server_*); operands are device-resident."""

    def __init__(self, budget_bytes: int | None = None, slots: int | None = None, reserve_sms: int | None = None,
                 aging_ms: float | None = None, large_threshold: int | None = None, batch_threshold: int | None = None,
                 batch_max: int | None = None, large_slots: int | None = None):
        cfg = ServerConfig()
        lib().gb300_server_config_init(ct.byref(cfg))
        if budget_bytes is not None:
            cfg.memory_budget_bytes = budget_bytes
        if slots is not None:
            cfg.slots = slots
        if reserve_sms is not None:
            cfg.reserve_sms = reserve_sms
        if aging_ms is not None:
            cfg.aging_ms = aging_ms
        if large_threshold is not None:
            cfg.large_threshold = large_threshold
        if batch_threshold is not None:
            cfg.batch_threshold = batch_threshold
        if batch_max is not None:
            cfg.batch_max = batch_max
        if large_slots is not None:
            cfg.large_slots = large_slots
        self.handle = ct.c_void_p()
        check(lib().gb300_server_create(ct.byref(cfg), ct.byref(self.handle)))

    def submit(self, order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, accuracy="split",
               target_error: float = 0.0) -> int:
        r = ServeRequest()
        r.order, r.transA, r.transB, r.m, r.n, r.k = order, transA, transB, m, n, k
        r.alpha, r.beta = alpha, beta
        r.A, r.lda, r.B, r.ldb, r.C, r.ldc = _addr(A), lda, _addr(B), ldb, _addr(C), ldc
        r.accuracy = METHODS[accuracy] if isinstance(accuracy, str) else int(accuracy)
        r.target_error = target_error
        t = ct.c_uint64(0)
        st = lib().gb300_server_submit(self.handle, ct.byref(r), ct.byref(t))
        if st != OK:
            raise Gb300Error(st, last_error()[1])
        return t.value

    def wait(self, ticket: int, timeout_ms: float = -1.0) -> ServeResult:
        res = ServeResult()
        st = lib().gb300_server_wait(self.handle, ticket, timeout_ms, ct.byref(res))
        if st != OK:
            raise Gb300Error(st, last_error()[1] or f"request status {st}")
        return res

    def stats(self) -> ServerStats:
        s = ServerStats()
        check(lib().gb300_server_get_stats(self.handle, ct.byref(s)))
        return s

    def reset_stats(self) -> None:
        lib().gb300_server_reset_stats(self.handle)

    def close(self) -> None:
        if self.handle:
            lib().gb300_server_destroy(self.handle)
            self.handle = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def device_info() -> tuple[int, int, int]:
    sms, fr, tot = ct.c_int(0), ct.c_int64(0), ct.c_int64(0)
    check(lib().gb300_device_info(ct.byref(sms), ct.byref(fr), ct.byref(tot)))
    return sms.value, fr.value, tot.value


def measure_fp64_peak() -> float:
    v = ct.c_double(0.0)
    check(lib().gb300_measure_fp64_peak(ct.byref(v)))
    return v.value


def measure_fp32_peak() -> float:
    v = ct.c_double(0.0)
    check(lib().gb300_measure_fp32_peak(ct.byref(v)))
    return v.value


def launch_count() -> int:
    return int(lib().gb300_launch_count())


def pool_bytes() -> int:
    """Device bytes held by the library's own grow-only buffers."""
    return int(lib().gb300_pool_bytes())


def select_device(ordinal: int) -> None:
    check(lib().gb300_select_device(ordinal))


def profile_enable(on: bool = True) -> None:
    lib().gb300_profile_enable(1 if on else 0)


def profile_read(prefix: str | None = None) -> tuple[float, int]:
    ms, n = ct.c_double(0.0), ct.c_int64(0)
    check(lib().gb300_profile_read(prefix.encode() if prefix else None, ct.byref(ms), ct.byref(n)))
    return ms.value, n.value


def synchronize() -> None:
    check(lib().gb300_synchronize())
