"""Compile the Blaze drop-in test program (needs the reference headers; test infrastructure).

    build(kind, program, intercept)
                           kind = "stub": linked against stub_cblas.cpp (CPU stand-in that logs calls)
                           kind = "lib":  linked against blaze_gb300/libgb300blas.so
                           program = "main" (dropin_main.cpp: ?gemm), "next" (dropin_next.cpp:
                           gemv / trmv / complex gemm / trmm through Blaze's expressions) or
                           "gated" (dropin_gated.cpp: the products Blaze's kernel selection keeps
                           on the CPU) or "smp" (dropin_smp.cpp: Blaze's OpenMP evaluation with
                           BLAZE_BLAS_IS_PARALLEL=0, concurrent tile calls)
                           intercept = True: compiled with include/gb300_blaze.h
    build_blazetest(elem)  the reference's own operation test blazetest/src/mathtest/operations/
                           dmatdmatmult/MDaMDa.cpp (row- and column-major DynamicMatrix operands in
                           every storage-order combination and assignment form, its sizes 0..6 and
                           15..64), element type `elem`, in BLAS mode and Blaze's debug mode (the
                           kernel-selection gates off, so every product reaches ?gemm), linked
                           against the logging stub
Returns the executable path, or None when the Blaze headers are not available here.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build")

def _reference_root() -> str:
    import sys

    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import oracle

    return oracle.reference_root() or ""


REF = _reference_root()

FLAGS = ["-std=c++17", "-O1", "-DBLAZE_BLAS_MODE=1", "-DBLAZE_BLAS_IS_PARALLEL=1",
         "-DBLAZE_BLAS_INCLUDE_FILE=<gb300_cblas.h>", "-DGB300_BLAS_THROW", "-I" + os.path.join(ROOT, "include")]


def available() -> bool:
    return bool(REF) and os.path.isdir(os.path.join(REF, "blaze")) and shutil.which("g++") is not None


# matrix x vector products take Blaze's BLAS kernels (off by default, blaze/config/BLAS.h) from
# modest sizes on, and small-area matrix products take them too (blaze/config/Thresholds.h)
NEXT_FLAGS = ["-DBLAZE_USE_BLAS_MATRIX_VECTOR_MULTIPLICATION=1", "-DBLAZE_DMATDVECMULT_THRESHOLD=1000UL",
              "-DBLAZE_TDMATDVECMULT_THRESHOLD=1000UL", "-DBLAZE_TDVECDMATMULT_THRESHOLD=1000UL",
              "-DBLAZE_TDVECTDMATMULT_THRESHOLD=1000UL", "-DBLAZE_DMATDMATMULT_THRESHOLD=1UL"]


def build(kind: str, program: str = "main", intercept: bool = False) -> str | None:
    if not available():
        return None
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, f"dropin_{kind}" if program == "main" else f"dropin_{program}_{kind}")
    if intercept:
        exe += "_intercept"
    srcs = [os.path.join(HERE, f"dropin_{program}.cpp")]
    deps = list(srcs) + [os.path.join(ROOT, "include", "gb300_cblas.h"), os.path.join(ROOT, "include", "gb300_blaze.h")]
    extra = []
    if kind == "stub":
        srcs.append(os.path.join(HERE, "stub_cblas.cpp"))
        deps.append(srcs[-1])
    else:
        lib_dir = os.path.join(ROOT, "blaze_gb300")
        extra = ["-L" + lib_dir, "-lgb300blas", "-Wl,-rpath," + lib_dir]
    if os.path.exists(exe) and all(os.path.getmtime(exe) >= os.path.getmtime(d) for d in deps):
        return exe
    flags = FLAGS + (NEXT_FLAGS if program == "next" else []) + (["-DGB300_INTERCEPT"] if intercept else [])
    if program == "smp":
        flags = [f for f in flags if not f.startswith("-DBLAZE_BLAS_IS_PARALLEL")] + \
            ["-DBLAZE_BLAS_IS_PARALLEL=0", "-fopenmp"]
    cmd = ["g++", *flags, "-isystem", REF, *srcs, "-o", exe, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("Blaze drop-in build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    return exe


def build_blazetest(elem: str = "double") -> str | None:
    if not available():
        return None
    src = os.path.join(REF, "blazetest", "src", "mathtest", "operations", "dmatdmatmult", "MDaMDa.cpp")
    if not os.path.exists(src):
        return None
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, f"blazetest_mdamda_{elem}_stub")
    stub = os.path.join(HERE, "stub_cblas.cpp")
    deps = [stub, os.path.join(ROOT, "include", "gb300_cblas.h")]
    if os.path.exists(exe) and all(os.path.getmtime(exe) >= os.path.getmtime(d) for d in deps):
        return exe
    flags = FLAGS + ["-DBLAZE_USE_DEBUG_MODE=1", f"-DBLAZETEST_MATHTEST_TYPE_A={elem}",
                     f"-DBLAZETEST_MATHTEST_TYPE_B={elem}"]
    cmd = ["g++", *flags, "-isystem", REF, "-isystem", os.path.join(REF, "blazetest"), src, stub, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("blazetest build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    return exe


def smp_fixture(raw_lines):
    """Log of dropin_smp.cpp (GB300_STUB_LOG_PTRS=1) -> fixture lines: each "product" marker, then
    its tile calls with the operand addresses replaced by element offsets inside the product's
    matrices, sorted (the threads log in any order)."""
    out, calls, base = [], [], None

    def flush():
        out.extend(sorted(calls))
        calls.clear()

    for ln in raw_lines:
        f = ln.split()
        if f[0] == "product":
            flush()
            base = [int(x, 16) for x in f[5:8]]
            out.append(" ".join(f[:5]))
        else:
            offs = [(int(x, 16) - b) // 8 for x, b in zip(f[12:15], base)]
            calls.append(" ".join(f[:12] + [str(o) for o in offs]))
    flush()
    return out
