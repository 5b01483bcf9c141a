"""Build libgb300blas.so in-tree: nvcc for sm_103a, translation units compiled in parallel.

    python -m blaze_gb300.nvcc_build     (or __graft_entry__.build())

Objects go to blaze_gb300/_build/, the library to blaze_gb300/libgb300blas.so.  The CUDA runtime
is linked statically, so loading the library needs no driver (a GPU is needed only to run it).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgb300blas.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-Xcompiler", "-Wall", "-I", INCLUDE, "-I", CSRC]

# (source, object, extra flags)
UNITS = [
    ("runtime.cpp", "runtime.o", []),
    ("api.cpp", "api.o", []),
    ("cblas.cpp", "cblas32.o", []),
    ("cblas.cpp", "cblas64.o", ["-DGB300_BLAS_ILP64"]),
    ("native_gemm.cu", "native_gemm.o", []),
    ("split_gemm.cu", "split_gemm.o", []),
    ("peaks.cu", "peaks.o", []),
    ("profile.cpp", "profile.o", []),
    ("grouped.cu", "grouped.o", []),
    ("serve.cpp", "serve.o", []),
    ("level23.cu", "level23.o", []),
    ("level1.cu", "level1.o", []),
    ("trsm.cu", "trsm.o", []),
    ("api_next.cpp", "api_next.o", []),
]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, obj: str, extra, verbose: bool) -> str:
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-x", "cu", "-c", os.path.join(CSRC, src), "-o", os.path.join(BUILD, obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile {src} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _headers()
    todo = [(s, o, x) for (s, o, x) in UNITS
            if force or verbose or _stale(os.path.join(BUILD, o), [os.path.join(CSRC, s), *hdrs, __file__])]
    logs = []
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_compile, s, o, x, verbose) for (s, o, x) in todo]
            for f in futs:
                logs.append(f.result())
    objs = [os.path.join(BUILD, o) for (_, o, _) in UNITS]
    if todo or not os.path.exists(LIB) or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        for l in logs:
            sys.stderr.write(l)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
