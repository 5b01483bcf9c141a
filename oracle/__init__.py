"""CPU oracle for the dense matrix-multiplication path (TEST INFRASTRUCTURE ONLY).

Python bindings (ctypes + numpy) for ``oracle/_build/liboracle.so`` — the C restatement of
Blaze's CPU GEMM kernels, the seeded generators and the compensated (Dot2) FP64 reference — and,
when it has been built in a container that has the reference headers, for
``oracle/_ref/libblazeref.so`` (Blaze itself).

Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline legs use this module,
always as the checker or as the timed CPU baseline.  The shipped library never calls it.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libblazeref.so")

ROW_MAJOR, COL_MAJOR = 101, 102
NO_TRANS, TRANS = 111, 112

_lib = None
_ref = None


def build(quiet: bool = True) -> str:
    """Compile liboracle.so with oracle/Makefile (gcc, a few seconds)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return LIB_PATH


def reference_root() -> str | None:
    """Directory holding the reference's headers (``blaze/``), or None when it is absent.

    The location is the oracle recipe's (``make -C oracle print-ref``; the environment variable
    BLAZE_REFERENCE_ROOT overrides it)."""
    root = os.environ.get("BLAZE_REFERENCE_ROOT")
    if not root:
        out = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
        root = out.stdout.strip() if out.returncode == 0 else ""
    return root if root and os.path.isdir(os.path.join(root, "blaze")) else None


def build_ref(ref_root: str | None = None) -> str | None:
    """Compile oracle/_ref/libblazeref.so from the reference headers, if they are present."""
    if os.path.exists(REF_PATH):
        return REF_PATH
    ref_root = ref_root or reference_root()
    if ref_root is None:
        return None
    out = subprocess.run(["make", "-C", HERE, "ref", f"REF={ref_root}"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)
    return REF_PATH


_D = ct.POINTER(ct.c_double)
_F = ct.POINTER(ct.c_float)
_I64 = ct.c_int64


def _gemm_argtypes(P, S):
    return [ct.c_int, ct.c_int, ct.c_int, _I64, _I64, _I64, S, P, _I64, P, _I64, S, P, _I64]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ct.CDLL(LIB_PATH)
        L.orc_fill_uniform_d.argtypes = [_D, _I64, ct.c_uint32, ct.c_double, ct.c_double]
        L.orc_fill_uniform_s.argtypes = [_F, _I64, ct.c_uint32, ct.c_float, ct.c_float]
        L.orc_fill_spread_d.argtypes = [_D, _I64, ct.c_uint32, ct.c_int, ct.c_int]
        L.orc_fill_spread_s.argtypes = [_F, _I64, ct.c_uint32, ct.c_int, ct.c_int]
        L.orc_fill_int_d.argtypes = [_D, _I64, ct.c_uint32, ct.c_int, ct.c_int]
        L.orc_mt19937_raw.argtypes = [ct.c_uint32, ct.POINTER(ct.c_uint32), _I64]
        L.orc_gemm_default_d.argtypes = _gemm_argtypes(_D, ct.c_double)
        L.orc_gemm_default_s.argtypes = _gemm_argtypes(_F, ct.c_float)
        L.orc_gemm_small_d.argtypes = _gemm_argtypes(_D, ct.c_double)
        L.orc_gemm_small_s.argtypes = _gemm_argtypes(_F, ct.c_float)
        _P64 = ct.POINTER(ct.c_int64)
        L.orc_gemm_batch_small_d.argtypes = [_I64, _P64, _D, _D, _D, _D, ct.c_int]
        L.orc_gemm_batch_small_s.argtypes = [_I64, _P64, _F, _F, _F, _F, ct.c_int]
        L.orc_gemm_blocked_d.argtypes = _gemm_argtypes(_D, ct.c_double) + [ct.c_int]
        L.orc_gemm_blocked_s.argtypes = _gemm_argtypes(_F, ct.c_float) + [ct.c_int]
        L.orc_product_rows_dot2.argtypes = [ct.c_int, ct.c_int, ct.c_int, _I64, _I64, _I64, _D, _I64,
                                            _D, _I64, ct.POINTER(ct.c_int64), _I64, _D, ct.c_int]
        L.orc_fro_norm_d.argtypes = [_D, _I64, _I64, _I64, ct.c_int]
        L.orc_fro_norm_d.restype = ct.c_double
        L.orc_fro_norm_s.argtypes = [_F, _I64, _I64, _I64, ct.c_int]
        L.orc_fro_norm_s.restype = ct.c_double
        L.orc_max_threads.restype = ct.c_int
        L.orc_trsm_left.argtypes = [ct.c_int, ct.c_int, _I64, _I64, _D, _D]
        L.orc_trsm_left.restype = None
        _lib = L
    return _lib


def ref_lib():
    """Blaze itself (oracle/_ref), or None when it was not built here."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = ct.CDLL(REF_PATH)
        R.ref_gemm_d.argtypes = _gemm_argtypes(_D, ct.c_double)
        R.ref_gemm_d.restype = ct.c_int
        R.ref_gemm_s.argtypes = _gemm_argtypes(_F, ct.c_float)
        R.ref_gemm_s.restype = ct.c_int
        i64 = ct.c_int64
        R.ref_gemv_d.argtypes = [ct.c_int, ct.c_int, i64, i64, ct.c_double, _D, i64, _D, ct.c_double, _D]
        R.ref_gemv_d.restype = ct.c_int
        R.ref_gemm_z.argtypes = [ct.c_int, ct.c_int, ct.c_int, i64, i64, i64, _D, _D, i64, _D, i64, _D, _D, i64]
        R.ref_gemm_z.restype = ct.c_int
        R.ref_trmm_d.argtypes = [ct.c_int] * 5 + [i64, i64, ct.c_double, _D, i64, _D, i64]
        R.ref_trmm_d.restype = ct.c_int
        R.ref_gemv_z.argtypes = [ct.c_int, ct.c_int, i64, i64, _D, _D, i64, _D, _D, _D]
        R.ref_gemv_z.restype = ct.c_int
        R.ref_trmv.argtypes = [ct.c_int] * 5 + [i64, _D, i64, _D]
        R.ref_trmv.restype = ct.c_int
        R.ref_trmm_z.argtypes = [ct.c_int] * 5 + [i64, i64, _D, _D, i64, _D, i64]
        R.ref_trmm_z.restype = ct.c_int
        R.ref_dot.argtypes = [ct.c_int, ct.c_int, i64, _D, _D, _D]
        R.ref_dot.restype = ct.c_int
        R.ref_axpy.argtypes = [ct.c_int, i64, _D, _D, _D]
        R.ref_axpy.restype = ct.c_int
        _ref = R
    return _ref


def _p(x: np.ndarray):
    assert x.flags["C_CONTIGUOUS"] or x.flags["F_CONTIGUOUS"]
    return x.ctypes.data_as(_D if x.dtype == np.float64 else _F)


# ---- generators ---------------------------------------------------------------------------------
def uniform(n: int, seed: int, lo: float = -1.0, hi: float = 1.0, dtype=np.float64) -> np.ndarray:
    x = np.empty(n, dtype=dtype)
    if dtype == np.float64:
        lib().orc_fill_uniform_d(_p(x), n, seed, lo, hi)
    else:
        lib().orc_fill_uniform_s(_p(x), n, seed, lo, hi)
    return x


def spread(n: int, seed: int, emin: int = -20, emax: int = 20, dtype=np.float64) -> np.ndarray:
    x = np.empty(n, dtype=dtype)
    if dtype == np.float64:
        lib().orc_fill_spread_d(_p(x), n, seed, emin, emax)
    else:
        lib().orc_fill_spread_s(_p(x), n, seed, emin, emax)
    return x


def integers(n: int, seed: int, lo: int = -10, hi: int = 10) -> np.ndarray:
    x = np.empty(n, dtype=np.float64)
    lib().orc_fill_int_d(_p(x), n, seed, lo, hi)
    return x


def mt19937_raw(seed: int, n: int) -> np.ndarray:
    x = np.empty(n, dtype=np.uint32)
    lib().orc_mt19937_raw(seed, x.ctypes.data_as(ct.POINTER(ct.c_uint32)), n)
    return x


def matrix(rows: int, cols: int, seed: int, dist: str = "uniform", dtype=np.float64,
           ld: int | None = None, order: int = ROW_MAJOR) -> np.ndarray:
    """A stored matrix buffer: rows x cols logical, `order` storage, leading dimension `ld`.

    Returns the flat storage buffer (length ld*rows for row-major, ld*cols for column-major);
    padding elements are filled from the same stream.
    """
    if order == ROW_MAJOR:
        ld = cols if ld is None else ld
        n = max(ld * rows, 1)
    else:
        ld = rows if ld is None else ld
        n = max(ld * cols, 1)
    if dist == "uniform":
        return uniform(n, seed, dtype=dtype)
    if dist == "spread":
        return spread(n, seed, dtype=dtype)
    if dist == "int":
        return integers(n, seed).astype(dtype)
    raise ValueError(dist)


# ---- kernels -------------------------------------------------------------------------------------
def gemm(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, kernel="blocked",
         nthreads: int = 0):
    """CBLAS-semantics C = alpha*op(A)op(B) + beta*C with the Blaze restatement (in place on C).

    kernel: "blocked" (mmm), "default" (scalar i-k-j) or "small" (register-blocked small kernel)."""
    L = lib()
    sfx = "d" if C.dtype == np.float64 else "s"
    if kernel == "blocked":
        getattr(L, "orc_gemm_blocked_" + sfx)(order, transA, transB, m, n, k, alpha, _p(A), lda, _p(B), ldb, beta,
                                              _p(C), ldc, nthreads)
    elif kernel in ("default", "small"):
        getattr(L, f"orc_gemm_{kernel}_" + sfx)(order, transA, transB, m, n, k, alpha, _p(A), lda, _p(B), ldb, beta,
                                                _p(C), ldc)
    else:
        raise ValueError(kernel)
    return C


def batch_descriptor(specs):
    """(desc, alpha_beta) arrays of a product list for gemm_batch_small: per product order, transA,
    transB, m, n, k, lda, ldb, ldc and the element offsets offA, offB, offC."""
    keys = ("order", "transA", "transB", "m", "n", "k", "lda", "ldb", "ldc", "offA", "offB", "offC")
    desc = np.array([[int(sp[key]) for key in keys] for sp in specs], dtype=np.int64).reshape(-1, 12)
    ab = np.array([[sp["alpha"], sp["beta"]] for sp in specs], dtype=np.float64).reshape(-1, 2)
    return np.ascontiguousarray(desc), ab


def gemm_batch_small(desc, ab, A, B, C, nthreads: int = 0):
    """Blaze's small kernel over every product of a batch (in place on C), products spread over
    nthreads OpenMP threads (<= 0: all)."""
    L = lib()
    ab = np.ascontiguousarray(ab, dtype=C.dtype)
    f = L.orc_gemm_batch_small_d if C.dtype == np.float64 else L.orc_gemm_batch_small_s
    f(len(desc), desc.ctypes.data_as(ct.POINTER(ct.c_int64)), _p(ab), _p(A), _p(B), _p(C), nthreads)
    return C


def ref_gemm(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc):
    """The same call through Blaze itself (oracle/_ref); raises if it was not built."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("oracle/_ref/libblazeref.so not built")
    f = R.ref_gemm_d if C.dtype == np.float64 else R.ref_gemm_s
    if f(order, transA, transB, m, n, k, alpha, _p(A), lda, _p(B), ldb, beta, _p(C), ldc) != 0:
        raise RuntimeError("Blaze raised an exception for this call (see stderr)")
    return C


def product_rows_dot2(order, transA, transB, m, n, k, A, lda, B, ldb, rows=None, nthreads: int = 0):
    """Rows of op(A)op(B) (logical row-major, nrows x n) in compensated FP64."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    if rows is None:
        nrows, rp = m, None
    else:
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        nrows, rp = len(rows), rows.ctypes.data_as(ct.POINTER(ct.c_int64))
    P = np.empty((nrows, n), dtype=np.float64)
    lib().orc_product_rows_dot2(order, transA, transB, m, n, k, _p(A), lda, _p(B), ldb, rp, nrows, _p(P), nthreads)
    return P


def fro_norm_op(order, trans, rows, cols, X, ld) -> float:
    """Frobenius norm of the logical rows x cols operand op(X) (compensated)."""
    # the norm is invariant under transposition; walk the storage as it lies
    sr, sc = (rows, cols) if trans == NO_TRANS else (cols, rows)
    rm = 1 if order == ROW_MAJOR else 0
    if X.dtype == np.float64:
        return lib().orc_fro_norm_d(_p(X), sr, sc, ld, rm)
    return lib().orc_fro_norm_s(_p(X), sr, sc, ld, rm)


def logical(order, trans, rows, cols, X, ld) -> np.ndarray:
    """The logical rows x cols matrix op(X) as a numpy array (a view when possible)."""
    t = trans != NO_TRANS
    if order == ROW_MAJOR:
        if not t:
            return np.lib.stride_tricks.as_strided(X, (rows, cols), (ld * X.itemsize, X.itemsize))
        return np.lib.stride_tricks.as_strided(X, (rows, cols), (X.itemsize, ld * X.itemsize))
    if not t:
        return np.lib.stride_tricks.as_strided(X, (rows, cols), (X.itemsize, ld * X.itemsize))
    return np.lib.stride_tricks.as_strided(X, (rows, cols), (ld * X.itemsize, X.itemsize))


def normwise_error(C_logical: np.ndarray, Cref_logical: np.ndarray, normA: float, normB: float,
                   scale: float = 1.0) -> float:
    """||C - Cref||_F / (||A||_F ||B||_F), with an optional sqrt(m/nrows) sampling scale."""
    d = np.asarray(C_logical, dtype=np.float64) - np.asarray(Cref_logical, dtype=np.float64)
    num = float(np.sqrt(np.sum(d * d))) * scale
    den = normA * normB
    return num / den if den > 0 else num


def _cd(x):
    return np.ascontiguousarray(x).ctypes.data_as(_D)


def ref_gemv(order, transA, m, n, alpha, A, lda, x, beta, y):
    """y = alpha op(A) x + beta y (unit strides) through Blaze itself; y is updated in place."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("oracle/_ref/libblazeref.so was not built")
    if R.ref_gemv_d(order, transA, m, n, alpha, _cd(A), lda, _cd(x), beta, y.ctypes.data_as(_D)) != 0:
        raise RuntimeError("Blaze raised")


def ref_zgemm(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc):
    """Complex C = alpha op(A) op(B) + beta C through Blaze itself (complex128 arrays, CBLAS
    transposes 111 / 112 / 113); C is updated in place."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("oracle/_ref/libblazeref.so was not built")
    al = np.array([alpha.real, alpha.imag]); be = np.array([beta.real, beta.imag])
    Ad = np.ascontiguousarray(A).view(np.float64); Bd = np.ascontiguousarray(B).view(np.float64)
    if R.ref_gemm_z(order, transA, transB, m, n, k, _cd(al), _cd(Ad), lda, _cd(Bd), ldb, _cd(be),
                    C.view(np.float64).ctypes.data_as(_D), ldc) != 0:
        raise RuntimeError("Blaze raised")


def ref_trmm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb):
    """B = alpha op(A) B or alpha B op(A), A triangular, through Blaze itself; B updated in place."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("oracle/_ref/libblazeref.so was not built")
    if R.ref_trmm_d(order, side, uplo, transA, diag, m, n, alpha, _cd(A), lda, B.ctypes.data_as(_D), ldb) != 0:
        raise RuntimeError("Blaze raised")


def _ref_or_raise():
    R = ref_lib()
    if R is None:
        raise RuntimeError("oracle/_ref/libblazeref.so was not built")
    return R


def ref_zgemv(order, transA, m, n, alpha, A, lda, x, beta, y):
    """Complex y = alpha op(A) x + beta y (unit strides, complex128, transposes 111 / 112 / 113)
    through Blaze itself; y is updated in place."""
    R = _ref_or_raise()
    al = np.array([alpha.real, alpha.imag]); be = np.array([beta.real, beta.imag])
    Ad = np.ascontiguousarray(A).view(np.float64); xd = np.ascontiguousarray(x).view(np.float64)
    if R.ref_gemv_z(order, transA, m, n, _cd(al), _cd(Ad), lda, _cd(xd), _cd(be), y.view(np.float64).ctypes.data_as(_D)) != 0:
        raise RuntimeError("Blaze raised")


def ref_trmv(order, uplo, transA, diag, n, A, lda, x):
    """x = op(A) x (unit stride), A triangular, through Blaze itself; float64 or complex128; x is
    updated in place."""
    R = _ref_or_raise()
    cplx = int(np.iscomplexobj(x))
    Ad = np.ascontiguousarray(A).view(np.float64)
    if R.ref_trmv(cplx, order, uplo, transA, diag, n, _cd(Ad), lda, x.view(np.float64).ctypes.data_as(_D)) != 0:
        raise RuntimeError("Blaze raised")


def ref_ztrmm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb):
    """Complex B = alpha op(A) B or alpha B op(A), A triangular, through Blaze itself (complex128);
    B is updated in place."""
    R = _ref_or_raise()
    al = np.array([alpha.real, alpha.imag])
    Ad = np.ascontiguousarray(A).view(np.float64)
    if R.ref_trmm_z(order, side, uplo, transA, diag, m, n, _cd(al), _cd(Ad), lda, B.view(np.float64).ctypes.data_as(_D),
                    ldb) != 0:
        raise RuntimeError("Blaze raised")


def ref_dot(x, y, conj=False):
    """Blaze's x * y (or conj(x) * y) for unit-stride float64 / complex128 vectors."""
    R = _ref_or_raise()
    cplx = int(np.iscomplexobj(x))
    out = np.zeros(2)
    xd = np.ascontiguousarray(x).view(np.float64) if cplx else np.ascontiguousarray(x, dtype=np.float64)
    yd = np.ascontiguousarray(y).view(np.float64) if cplx else np.ascontiguousarray(y, dtype=np.float64)
    if R.ref_dot(cplx, int(conj), len(x), _cd(xd), _cd(yd), out.ctypes.data_as(_D)) != 0:
        raise RuntimeError("Blaze raised")
    return complex(out[0], out[1]) if cplx else float(out[0])


def ref_axpy(alpha, x, y):
    """Blaze's y += alpha * x for unit-stride float64 / complex128 vectors; y updated in place."""
    R = _ref_or_raise()
    cplx = int(np.iscomplexobj(y))
    al = np.array([complex(alpha).real, complex(alpha).imag])
    xd = np.ascontiguousarray(x).view(np.float64) if cplx else np.ascontiguousarray(x, dtype=np.float64)
    yd = y.view(np.float64) if cplx else y
    if R.ref_axpy(cplx, len(x), _cd(al), _cd(xd), yd.ctypes.data_as(_D)) != 0:
        raise RuntimeError("Blaze raised")


# ---- CBLAS-level restatements of the routines next to ?gemm that Blaze has no kernel for -------
CONJ_TRANS = 113


def triangle_logical(order, uplo, transA, diag, ka, A, lda) -> np.ndarray:
    """op(A) as a dense logical ka x ka array: the `uplo` triangle of the stored A (the other half
    is not read), ones on a unit diagonal, transposed for 112 and conjugate-transposed for 113."""
    cplx = np.iscomplexobj(A)
    flat = np.asarray(A).reshape(-1)
    idx = np.arange(ka)
    pos = (idx[:, None] * lda + idx[None, :]) if order == ROW_MAJOR else (idx[None, :] * lda + idx[:, None])
    full = flat[pos].astype(np.complex128 if cplx else np.float64)
    keep = np.tril(np.ones((ka, ka), dtype=bool)) if uplo == 122 else np.triu(np.ones((ka, ka), dtype=bool))
    full = np.where(keep, full, 0)
    if diag == 132:
        full[idx, idx] = 1
    if transA == TRANS:
        full = full.T
    elif transA == CONJ_TRANS:
        full = full.conj().T
    return np.ascontiguousarray(full)


def trsm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb) -> None:
    """B = alpha op(A)^-1 B (side 141) or alpha B op(A)^-1 (142) by substitution in the oracle's C
    restatement (orc_trsm_left), float64 or complex128; B is updated in place."""
    left = side == 141
    ka = m if left else n
    cplx = np.iscomplexobj(B)
    T = triangle_logical(order, uplo, transA, diag, ka, A, lda)
    flat = B.reshape(-1)
    ii, jj = np.arange(m)[:, None], np.arange(n)[None, :]
    pos = ii * ldb + jj if order == ROW_MAJOR else jj * ldb + ii
    X = alpha * flat[pos].astype(np.complex128 if cplx else np.float64)  # logical m x n
    lower = (uplo == 122) == (transA == NO_TRANS)  # op(A) lower triangular
    if not left:  # X op(A) = B  <=>  op(A)^T X^T = B^T
        T, X, lower = np.ascontiguousarray(T.T), X.T, not lower
    X = np.ascontiguousarray(X)
    Tv, Xv = (T.view(np.float64), X.view(np.float64)) if cplx else (T, X)
    lib().orc_trsm_left(int(cplx), int(lower), ka, X.shape[1], _cd(Tv), Xv.ctypes.data_as(_D))
    flat[pos] = X if left else X.T


def complex_uniform(count: int, seed: int) -> np.ndarray:
    """Complex128 values with real parts uniform(seed) and imaginary parts uniform(seed + 7919)."""
    re = uniform(max(count, 1), seed)[:count]
    im = uniform(max(count, 1), seed + 7919)[:count]
    return re + 1j * im


def triangular_operands(cplx: bool, ka: int, lda: int, rows_b: int, ldb: int, seed: int):
    """Seeded operands of a triangular solve: the stored ka x ka square of the triangle (pitch lda;
    off-diagonal entries u / ka, diagonal 1 + u / 2, u uniform in [-1, 1], well conditioned with or
    without a unit diagonal) and a solution X0 of rows_b x ldb stored elements."""
    A = (complex_uniform(ka * lda, seed) if cplx else uniform(ka * lda, seed).copy()) / ka
    d = np.arange(ka) * (lda + 1)
    A[d] = 1 + 0.5 * ka * A[d]
    X0 = complex_uniform(rows_b * ldb, seed + 1) if cplx else uniform(rows_b * ldb, seed + 1).copy()
    return A, X0
