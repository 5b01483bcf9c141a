"""The C-ABI library: it loads without a GPU, exports every function the public headers declare,
and its host-side argument handling follows the CBLAS contract."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

import blaze_gb300 as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include"))) if h.endswith(".h")]


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(G.LIB_PATH):
        G.build()
    return G.lib()


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for mname in re.findall(r"\b((?:cblas|gb300)_\w+)\s*\(", text):
            names.add(mname)
    # the wrappers/macros of the headers themselves are not library symbols
    names -= {"gb300_throw_if_error"}
    return sorted(names)


def test_headers_declare_the_cblas_surface_blaze_uses():
    names = declared_functions()
    for base in ("gemm", "gemv", "trmm", "trmv", "trsm", "axpy"):
        for p in "sdcz":
            assert f"cblas_{p}{base}" in names
    for f in ("cblas_sdot", "cblas_ddot", "cblas_cdotu_sub", "cblas_zdotc_sub", "cblas_cdotu", "cblas_zdotc"):
        assert f in names


def test_library_exports_every_declared_function(lib):
    missing = []
    for name in declared_functions():
        for sym in ([name, name + "_64"] if name.startswith("cblas_") or name.endswith("_checked") else [name]):
            try:
                getattr(lib, sym)
            except AttributeError:
                missing.append(sym)
    assert not missing, missing


def test_enum_values_are_the_cblas_abi():
    text = open(os.path.join(ROOT, "include", "gb300_cblas.h")).read()
    for name, val in (("CblasRowMajor", 101), ("CblasColMajor", 102), ("CblasNoTrans", 111), ("CblasTrans", 112),
                      ("CblasConjTrans", 113), ("CblasUpper", 121), ("CblasLower", 122), ("CblasNonUnit", 131),
                      ("CblasUnit", 132), ("CblasLeft", 141), ("CblasRight", 142)):
        assert re.search(rf"\b{name}\s*=\s*{val}\b", text), name


@pytest.mark.parametrize("args,param", [
    (dict(order=99), 1), (dict(ta=7), 2), (dict(tb=7), 3), (dict(m=-1), 4), (dict(n=-1), 5), (dict(k=-1), 6),
    (dict(lda=3), 9), (dict(ldb=3), 11), (dict(ldc=3), 14),
])
def test_argument_errors_name_the_parameter(lib, args, param):
    a = dict(order=G.RowMajor, ta=G.NoTrans, tb=G.NoTrans, m=8, n=8, k=8, lda=8, ldb=8, ldc=8)
    a.update(args)
    A = np.zeros(64); B = np.zeros(64); C = np.zeros(64)
    lib.gb300_clear_error()
    lib.cblas_dgemm(a["order"], a["ta"], a["tb"], a["m"], a["n"], a["k"], 1.0, A.ctypes.data, a["lda"],
                    B.ctypes.data, a["ldb"], 0.0, C.ctypes.data, a["ldc"])
    st, msg = G.last_error()
    assert st == G.ERR_INVALID_ARG
    assert f"parameter {param} " in msg


def test_quick_returns_do_not_touch_the_device(lib):
    C = np.full(4, 7.0)
    lib.gb300_clear_error()
    lib.cblas_dgemm(G.RowMajor, G.NoTrans, G.NoTrans, 0, 2, 2, 1.0, None, 2, None, 2, 0.0, C.ctypes.data, 2)
    assert G.last_error()[0] == G.OK
    lib.cblas_dgemm(G.RowMajor, G.NoTrans, G.NoTrans, 2, 2, 0, 1.0, None, 1, None, 2, 1.0, C.ctypes.data, 2)
    assert G.last_error()[0] == G.OK and np.all(C == 7.0)


def test_level1_and_trsm_need_the_device(lib):
    """No routine is a stub: axpy, the dot products and trsm validate, then need the GPU; on a
    host without one they say so and compute nothing."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    x = np.arange(4.0); y = np.ones(4)
    G.lib().gb300_clear_error()
    G.lib().cblas_daxpy(4, 2.0, x.ctypes.data, 1, y.ctypes.data, 1)
    assert G.last_error()[0] == G.ERR_NO_DEVICE and np.all(y == 1.0)
    G.lib().gb300_clear_error()
    assert G.lib().cblas_ddot(4, x.ctypes.data, 1, y.ctypes.data, 1) == 0.0
    assert G.last_error()[0] == G.ERR_NO_DEVICE
    A = np.eye(4); B = np.ones(8)
    G.lib().gb300_clear_error()
    G.lib().cblas_dtrsm(101, 141, 122, 111, 131, 4, 2, 1.0, A.ctypes.data, 4, B.ctypes.data, 2)
    assert G.last_error()[0] == G.ERR_NO_DEVICE and np.all(B == 1.0)


def test_no_device_is_reported_not_faked(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    A = np.ones(4); B = np.ones(4); C = np.zeros(4)
    lib.gb300_clear_error()
    lib.cblas_dgemm(G.RowMajor, G.NoTrans, G.NoTrans, 2, 2, 2, 1.0, A.ctypes.data, 2, B.ctypes.data, 2, 0.0,
                    C.ctypes.data, 2)
    assert G.last_error()[0] == G.ERR_NO_DEVICE
    assert np.all(C == 0.0)  # nothing was computed on the CPU


@pytest.mark.parametrize("routine,args,param", [
    ("gemv", dict(order=99), 1), ("gemv", dict(ta=7), 2), ("gemv", dict(m=-1), 3), ("gemv", dict(n=-1), 4),
    ("gemv", dict(lda=3), 7), ("gemv", dict(incx=0), 9), ("gemv", dict(incy=0), 12),
    ("zgemm", dict(order=99), 1), ("zgemm", dict(ta=7), 2), ("zgemm", dict(k=-1), 6), ("zgemm", dict(lda=3), 9),
    ("zgemm", dict(ldc=3), 14),
    ("trmm", dict(side=7), 2), ("trmm", dict(uplo=7), 3), ("trmm", dict(ta=7), 4), ("trmm", dict(diag=7), 5),
    ("trmm", dict(m=-1), 6), ("trmm", dict(lda=3), 10), ("trmm", dict(ldb=3), 12),
    ("zgemv", dict(order=99), 1), ("zgemv", dict(ta=7), 2), ("zgemv", dict(lda=3), 7), ("zgemv", dict(incy=0), 12),
    ("trmv", dict(order=99), 1), ("trmv", dict(uplo=7), 2), ("trmv", dict(ta=7), 3), ("trmv", dict(diag=7), 4),
    ("trmv", dict(n=-1), 5), ("trmv", dict(lda=3), 7), ("trmv", dict(incx=0), 9),
    ("ztrmv", dict(uplo=7), 2), ("ztrmv", dict(lda=3), 7), ("ztrmv", dict(incx=0), 9),
    ("ztrmm", dict(side=7), 2), ("ztrmm", dict(diag=7), 5), ("ztrmm", dict(lda=3), 10), ("ztrmm", dict(ldb=3), 12),
    ("trsm", dict(order=99), 1), ("trsm", dict(side=7), 2), ("trsm", dict(uplo=7), 3), ("trsm", dict(ta=7), 4),
    ("trsm", dict(diag=7), 5), ("trsm", dict(m=-1), 6), ("trsm", dict(n=-1), 7), ("trsm", dict(lda=3), 10),
    ("trsm", dict(ldb=3), 12), ("ztrsm", dict(side=7), 2), ("ztrsm", dict(ta=7), 4), ("ztrsm", dict(lda=3), 10),
])
def test_neighbour_routines_name_the_parameter(lib, routine, args, param):
    a = dict(order=G.RowMajor, ta=G.NoTrans, tb=G.NoTrans, m=8, n=8, k=8, lda=8, ldb=8, ldc=8, incx=1, incy=1,
             side=141, uplo=121, diag=131)
    a.update(args)
    A = np.zeros(128); B = np.zeros(128); C = np.zeros(128)
    one = np.array([1.0, 0.0]); zero = np.array([0.0, 0.0])
    lib.gb300_clear_error()
    if routine == "gemv":
        lib.cblas_dgemv(a["order"], a["ta"], a["m"], a["n"], 1.0, A.ctypes.data, a["lda"], B.ctypes.data, a["incx"],
                        0.0, C.ctypes.data, a["incy"])
    elif routine == "zgemm":
        lib.cblas_zgemm(a["order"], a["ta"], a["tb"], a["m"], a["n"], a["k"], one.ctypes.data, A.ctypes.data,
                        a["lda"], B.ctypes.data, a["ldb"], zero.ctypes.data, C.ctypes.data, a["ldc"])
    elif routine == "zgemv":
        lib.cblas_zgemv(a["order"], a["ta"], a["m"], a["n"], one.ctypes.data, A.ctypes.data, a["lda"], B.ctypes.data,
                        a["incx"], zero.ctypes.data, C.ctypes.data, a["incy"])
    elif routine in ("trmv", "ztrmv"):
        getattr(lib, "cblas_%s" % ("dtrmv" if routine == "trmv" else "ztrmv"))(
            a["order"], a["uplo"], a["ta"], a["diag"], a["n"], A.ctypes.data, a["lda"], B.ctypes.data, a["incx"])
    elif routine == "trsm":
        lib.cblas_dtrsm(a["order"], a["side"], a["uplo"], a["ta"], a["diag"], a["m"], a["n"], 1.0, A.ctypes.data,
                        a["lda"], B.ctypes.data, a["ldb"])
    elif routine == "ztrsm":
        lib.cblas_ztrsm(a["order"], a["side"], a["uplo"], a["ta"], a["diag"], a["m"], a["n"], one.ctypes.data,
                        A.ctypes.data, a["lda"], B.ctypes.data, a["ldb"])
    elif routine == "ztrmm":
        lib.cblas_ztrmm(a["order"], a["side"], a["uplo"], a["ta"], a["diag"], a["m"], a["n"], one.ctypes.data,
                        A.ctypes.data, a["lda"], B.ctypes.data, a["ldb"])
    else:
        lib.cblas_dtrmm(a["order"], a["side"], a["uplo"], a["ta"], a["diag"], a["m"], a["n"], 1.0, A.ctypes.data,
                        a["lda"], B.ctypes.data, a["ldb"])
    st, msg = G.last_error()
    assert st == G.ERR_INVALID_ARG
    assert f"parameter {param} " in msg


def test_call_trace_prints_enter_and_leave():
    """GB300_BLAS_TRACE=1: one enter and one leave line per call with the routine, the shape and
    the call's status (here the call fails: argument check, or no device on a CPU host)."""
    import subprocess
    import sys
    code = ("import numpy as np, blaze_gb300 as G\n"
            "A = np.ones(6); B = np.ones(12); C = np.zeros(8)\n"
            "G.lib().gb300_clear_error()\n"
            "G.lib().cblas_dgemm(101, 111, 111, 2, 4, 3, 1.0, A.ctypes.data, 3, B.ctypes.data, 4, 0.0, C.ctypes.data, 4)\n"
            "G.lib().cblas_dgemm(101, 111, 111, 2, 4, 3, 1.0, A.ctypes.data, 1, B.ctypes.data, 4, 0.0, C.ctypes.data, 4)\n")
    env = dict(os.environ, GB300_BLAS_TRACE="1")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, cwd=ROOT, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stderr.splitlines() if ln.startswith("libgb300blas: ")]
    enters = [ln for ln in lines if " enter cblas_dgemm m=2 n=4 k=3 " in ln]
    leaves = [ln for ln in lines if " leave cblas_dgemm status=" in ln]
    assert len(enters) == 2 and len(leaves) == 2, lines
    assert "status=1 " in leaves[1]  # the second call: parameter 9 (lda) is too small
