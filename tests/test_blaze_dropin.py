"""Blaze itself, built in BLAS mode with include/gb300_cblas.h as its BLAS header.

Where the reference headers exist (the build container), a Blaze program computing
`C = A*B`, `+=`, `-=` and `s*(A*B)` for every storage-order class and a CustomMatrix is compiled
(1) against a logging CPU stub, to check that every product reaches cblas_dgemm with the CBLAS
arguments blaze::gemm() derives (blaze/math/blas/gemm.h:115-131) and that the results are right,
(2) against the stub with an injected failure and (3) against libgb300blas.so on a host without a
GPU, to check that a library error reaches the Blaze caller as std::runtime_error (no silent CPU
result).  The recorded calls are also a committed fixture (tests/golden/blaze_calls.txt) that
the GPU tests replay."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "blaze_dropin"))
import build as dropin  # noqa: E402

pytestmark = pytest.mark.skipif(not dropin.available(), reason="Blaze headers are not present on this host")

EXPECTED_TRANS = {  # label -> (order, transA, transB): order from C, trans = (SO_C != SO_X)
    "rr_r": (101, 111, 111), "rc_r": (101, 111, 112), "cr_r": (101, 112, 111), "cc_r": (101, 112, 112),
    "rr_c": (102, 112, 112), "cc_c": (102, 111, 111), "custom": (101, 111, 111),
}
EXPECTED_AB = {"assign": (1.0, 0.0), "add": (1.0, 1.0), "sub": (-1.0, 1.0), "scaled": (2.5, 0.0)}


def run(exe, env):
    r = subprocess.run([exe], capture_output=True, text=True, env=dict(os.environ, **env), timeout=120)
    assert r.returncode == 0, r.stderr
    return [ln.split() for ln in r.stdout.splitlines() if ln.strip()]


def test_blaze_products_reach_cblas_dgemm_with_the_right_arguments(tmp_path):
    exe = dropin.build("stub")
    log = tmp_path / "log.txt"
    out = run(exe, {"GB300_STUB_LOG": str(log)})
    assert len(out) == 25
    for fields in out:
        assert fields[1] == "status=ok", fields
        assert float(fields[2].split("=")[1]) <= 1e-12, fields
    calls = [ln.split() for ln in log.read_text().splitlines()]
    assert len(calls) == len(out)
    for fields, call in zip(out, calls):
        label, op = fields[0].split("/")
        assert call[0] == "dgemm"
        assert tuple(int(x) for x in call[1:4]) == EXPECTED_TRANS[label], (fields, call)
        assert (float(call[7]), float(call[10])) == EXPECTED_AB[op], (fields, call)


def test_library_errors_surface_as_exceptions_in_blaze():
    exe = dropin.build("stub")
    out = run(exe, {"GB300_STUB_FAIL": "1"})
    assert all(f[1] == "status=exception" for f in out)
    assert all("injected failure" in " ".join(f) for f in out)


def test_real_library_without_gpu_raises_instead_of_computing_on_the_cpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import blaze_gb300 as G
    if not os.path.exists(G.LIB_PATH):
        G.build()
    exe = dropin.build("lib")
    out = run(exe, {})
    assert all(f[1] == "status=exception" for f in out), out
    assert all("no CUDA device" in " ".join(f) for f in out)


def test_recorded_call_fixture_matches_blaze():
    exe = dropin.build("stub")
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        log = os.path.join(d, "log.txt")
        run(exe, {"GB300_STUB_LOG": log})
        fresh = open(log).read().splitlines()
    committed = open(os.path.join(HERE, "golden", "blaze_calls.txt")).read().splitlines()
    assert fresh == committed


# ---- the routines next to ?gemm, reached through Blaze's own expressions (dropin_next.cpp) ----------
NEXT_ROUTINES = {  # label -> the CBLAS routine Blaze must call for it
    "gemv_r": "dgemv", "gemv_c_add": "dgemv", "gemv_t": "dgemv", "sgemv_r": "sgemv", "trmv_lower_r": "dtrmv",
    "trmv_upper_c": "dtrmv", "ztrmv_lower_r": "ztrmv", "zgemv_r": "zgemv", "zgemm_rr": "zgemm",
    "dtrmm_lower": "dtrmm", "ztrmm_upper": "ztrmm", "small_area": "dgemm", "skinny_cpu": None,
    "dotu_d": "ddot", "dotu_z": "zdotu_sub", "dotc_z": "zdotc_sub", "axpy_d": "daxpy", "axpy_z": "zaxpy",
    "trsm_lower_vec": "dtrsm", "trsm_upper_right": "dtrsm", "trsm_mixed": "dtrsm", "ztrsm_lower": "ztrsm",
}


def test_blaze_expressions_reach_the_neighbouring_routines(tmp_path):
    exe = dropin.build("stub", "next")
    log = tmp_path / "log.txt"
    out = run(exe, {"GB300_STUB_LOG": str(log)})
    assert [f[0] for f in out] == list(NEXT_ROUTINES)
    for fields in out:
        assert fields[1] == "status=ok", fields
        tol = 1e-4 if fields[0].startswith("s") else 1e-12
        assert float(fields[2].split("=")[1]) <= tol, fields
    calls = [ln.split() for ln in log.read_text().splitlines()]
    reaching = [lab for lab, r in NEXT_ROUTINES.items() if r]  # skinny_cpu makes no BLAS call
    assert [c[0] for c in calls] == [NEXT_ROUTINES[lab] for lab in reaching]
    # y += A*x is gemv with beta = 1 (DMatDVecMultExpr's BLAS add-assign kernel); x^T*A is the
    # transposed gemv; the column-major upper triangle is the row-major lower one's mirror
    by = dict(zip(reaching, calls))
    assert by["small_area"][1:7] == ["101", "111", "111", "40", "96", "30"]
    assert by["gemv_c_add"][1:3] == ["102", "111"] and float(by["gemv_c_add"][8]) == 1.0
    assert by["gemv_t"][2] == "112"
    assert by["trmv_lower_r"][1:5] == ["101", "122", "111", "131"]
    assert by["trmv_upper_c"][1:5] == ["102", "121", "111", "131"]
    assert by["dtrmm_lower"][1:6] == ["101", "141", "122", "111", "131"]
    # blaze::trsm: a vector right-hand side is an m x 1 system (ldb = 1 row-major); a column-major B
    # with a row-major A gets the transposed, flipped triangle (blaze/math/blas/trsm.h:195-199)
    assert by["trsm_lower_vec"][1:8] == ["101", "141", "122", "111", "131", "3", "1"]
    assert by["trsm_upper_right"][1:6] == ["102", "142", "121", "111", "131"]
    assert by["trsm_mixed"][1:6] == ["102", "141", "121", "112", "131"]


def test_neighbouring_call_fixture_matches_blaze():
    exe = dropin.build("stub", "next")
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        log = os.path.join(d, "log.txt")
        run(exe, {"GB300_STUB_LOG": log})
        fresh = open(log).read().splitlines()
    committed = open(os.path.join(HERE, "golden", "blaze_next_calls.txt")).read().splitlines()
    assert fresh == committed


def test_real_library_without_gpu_raises_for_the_neighbouring_routines_too():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import blaze_gb300 as G
    if not os.path.exists(G.LIB_PATH):
        G.build()
    exe = dropin.build("lib", "next")
    out = run(exe, {})
    assert len(out) == len(NEXT_ROUTINES)
    for f in out:
        if NEXT_ROUTINES[f[0]] is None:  # Blaze's own small kernel: no library call
            assert f[1] == "status=ok", f
        else:
            assert f[1] == "status=exception" and "no CUDA device" in " ".join(f), f


# ---- products Blaze's kernel selection keeps on the CPU, and include/gb300_blaze.h (dropin_gated.cpp)
def _gated_run(intercept, tmp_path):
    exe = dropin.build("stub", "gated", intercept)
    log = tmp_path / ("log_i.txt" if intercept else "log_p.txt")
    out = run(exe, {"GB300_STUB_LOG": str(log)})
    calls = [ln.split() for ln in log.read_text().splitlines()] if log.exists() else []
    return out, calls


def test_gated_products_stay_on_the_cpu_without_the_interception_header(tmp_path):
    out, calls = _gated_run(False, tmp_path)
    for f in out:
        assert f[1] == "status=ok", f
    ungated = [f for f in out if f[3] == "gated=0"]
    assert len(ungated) == 1 and len(out) == 14
    # only the product Blaze's selection already sends to BLAS makes a call
    assert len(calls) == 1 and calls[0][0] == "dgemm"
    assert calls[0][4:7] == [f.split("=")[1] for f in ungated[0][4:7]]


def test_interception_header_sends_every_gated_product_to_gemm(tmp_path):
    out, calls = _gated_run(True, tmp_path)
    assert len(calls) == len(out) == 14
    for f, c in zip(out, calls):
        assert f[1] == "status=ok", f
        tol = 1e-4 if f[0].startswith("small_float") else 1e-12
        assert float(f[2].split("=")[1]) <= tol, f
        assert c[0] == ("sgemm" if f[0].startswith("small_float") else "dgemm"), (f, c)
        assert c[4:7] == [x.split("=")[1] for x in f[4:7]], (f, c)  # m, n, k as Blaze's gemm() maps them
    by = {f[0]: c for f, c in zip(out, calls)}
    # the assignment forms keep Blaze's alpha / beta (the same as its own BLAS kernels)
    assert (by["small_rr"][7], by["small_rr"][10]) == ("1", "0")
    assert (by["small_rr/add"][7], by["small_rr/add"][10]) == ("1", "1")
    assert (by["small_rr/sub"][7], by["small_rr/sub"][10]) == ("-1", "1")
    assert (by["small_rr/scaled"][7], by["small_rr/scaled"][10]) == ("2.5", "0")
    # storage orders map like blaze::gemm: order from C, a transposition where an operand's differs
    assert by["skinny_cr"][1:4] == ["101", "112", "111"]
    assert by["skinny_cc"][1:4] == ["102", "111", "111"]
    assert by["small_rc"][1:4] == ["101", "111", "112"]
    # the intercepted call is the one Blaze itself makes for an ungated product
    plain_out, plain_calls = _gated_run(False, tmp_path)
    assert by["large_rr"] == plain_calls[0]


def test_gated_call_fixture_matches_blaze():
    exe = dropin.build("stub", "gated", True)
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        log = os.path.join(d, "log.txt")
        run(exe, {"GB300_STUB_LOG": log})
        fresh = open(log).read().splitlines()
    committed = open(os.path.join(HERE, "golden", "blaze_gated_calls.txt")).read().splitlines()
    assert fresh == committed


def test_intercepted_products_raise_from_the_real_library_without_a_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import blaze_gb300 as G
    if not os.path.exists(G.LIB_PATH):
        G.build()
    exe = dropin.build("lib", "gated", True)
    out = run(exe, {})
    assert len(out) == 14
    # every intercepted product reaches the library (which has no device here), none is computed on
    # the CPU behind the caller's back
    for f in out:
        assert f[1] == "status=exception" and "no CUDA device" in " ".join(f), f


# ---- Blaze's OpenMP tiles (dropin_smp.cpp) and the reference's own operation test ----------------
def test_openmp_tiles_reach_cblas_dgemm_concurrently_inside_the_operands(tmp_path):
    exe = dropin.build("stub", "smp")
    log = tmp_path / "log.txt"
    out = run(exe, {"GB300_STUB_LOG": str(log), "GB300_STUB_LOG_PTRS": "1", "OMP_NUM_THREADS": "4"})
    assert len(out) == 5
    for f in out:
        assert f[1] == "status=ok" and float(f[2].split("=")[1]) <= 1e-12, f
    lines = dropin.smp_fixture(log.read_text().splitlines())
    committed = open(os.path.join(HERE, "golden", "blaze_smp_calls.txt")).read().splitlines()
    assert lines == committed
    # several tiles per product, each an offset view with the whole matrix's leading dimension
    tiles = [ln.split() for ln in lines if not ln.startswith("product")]
    assert len(tiles) == 20
    assert any(int(t[12]) > 0 for t in tiles) and any(int(t[14]) > 0 for t in tiles)
    assert all(int(t[11]) != int(t[5] if t[1] == "101" else t[4]) for t in tiles)  # ldc != tile width


def test_blazetest_dmatdmatmult_operation_test_passes_through_the_seam(tmp_path):
    """blazetest's MDaMDa (every storage-order combination and assignment form of DynamicMatrix
    products) built in BLAS and debug mode against the stub: the test's own checks pass, and the
    distinct ?gemm calls it makes are the committed fixture the GPU tests replay."""
    exe = dropin.build_blazetest("double")
    if exe is None:
        pytest.skip("blazetest sources are not present")
    log = tmp_path / "log.txt"
    r = subprocess.run([exe], capture_output=True, text=True, env=dict(os.environ, GB300_STUB_LOG=str(log)),
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    counts = {}
    for ln in log.read_text().splitlines():
        counts[ln] = counts.get(ln, 0) + 1
    fresh = [f"{ln} {counts[ln]}" for ln in sorted(counts)]
    committed = open(os.path.join(HERE, "golden", "blazetest_mdamda_calls.txt")).read().splitlines()
    assert fresh == committed
    assert sum(int(ln.split()[-1]) for ln in committed) == 3672
