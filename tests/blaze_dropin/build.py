"""Compile the Blaze drop-in test program (needs the reference headers; test infrastructure).

    build(kind, program, intercept)
                           kind = "stub": linked against stub_cblas.cpp (CPU stand-in that logs calls)
                           kind = "lib":  linked against blaze_gb300/libgb300blas.so
                           program = "main" (dropin_main.cpp: ?gemm), "next" (dropin_next.cpp:
                           gemv / trmv / complex gemm / trmm through Blaze's expressions) or
                           "gated" (dropin_gated.cpp: the products Blaze's kernel selection keeps
                           on the CPU)
                           intercept = True: compiled with include/gb300_blaze.h
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
    cmd = ["g++", *flags, "-isystem", REF, *srcs, "-o", exe, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("Blaze drop-in build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    return exe
