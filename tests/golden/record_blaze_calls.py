"""Record the CBLAS calls Blaze itself makes in BLAS mode, by running the drop-in programs of
tests/blaze_dropin/ against their logging stub:

- tests/golden/blaze_calls.txt: `C = A*B`, `C += A*B`, `C -= A*B` and `C = s*(A*B)` (all
  storage-order classes and a CustomMatrix); one call per line: routine order transA transB m n k
  alpha lda ldb beta ldc;
- tests/golden/blaze_next_calls.txt: matrix x vector (dense and triangular), complex products and
  triangular products (dropin_next.cpp); one call per line: the routine name, then its CBLAS
  arguments in order without the pointers (complex scalars as re,im);
- tests/golden/blaze_gated_calls.txt: the products Blaze's kernel selection keeps on the CPU
  (dropin_gated.cpp), built with include/gb300_blaze.h, which sends them to ?gemm; the format of
  blaze_calls.txt;
- tests/golden/blaze_smp_calls.txt: Blaze's OpenMP evaluation with BLAZE_BLAS_IS_PARALLEL=0
  (dropin_smp.cpp, four threads): per product a line "product <label> <M> <N> <K>", then its
  concurrent tile calls in the format of blaze_calls.txt followed by the element offsets of the
  tile's A, B and C inside the whole matrices (the calls of a product sorted, since the threads
  log in any order);
- tests/golden/blazetest_mdamda_calls.txt: every distinct ?gemm call of the reference's own
  operation test blazetest/src/mathtest/operations/dmatdmatmult/MDaMDa.cpp (double) in BLAS and
  debug mode, sorted, each with the number of times it was made.

The GPU tests replay all of them through the real library.  Needs the reference headers.
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "blaze_dropin"))
import build as dropin  # noqa: E402

for program, out, intercept in (("main", "blaze_calls.txt", False), ("next", "blaze_next_calls.txt", False),
                                ("gated", "blaze_gated_calls.txt", True)):
    exe = dropin.build("stub", program, intercept)
    if exe is None:
        raise SystemExit("reference headers not available")
    with tempfile.TemporaryDirectory() as d:
        log = os.path.join(d, "log.txt")
        subprocess.run([exe], check=True, env=dict(os.environ, GB300_STUB_LOG=log), capture_output=True)
        lines = open(log).read().splitlines()
    with open(os.path.join(HERE, out), "w") as f:
        f.write("\n".join(lines) + "\n")
    print(f"{out}: recorded {len(lines)} calls")


exe = dropin.build("stub", "smp")
with tempfile.TemporaryDirectory() as d:
    log = os.path.join(d, "log.txt")
    subprocess.run([exe], check=True, capture_output=True,
                   env=dict(os.environ, GB300_STUB_LOG=log, GB300_STUB_LOG_PTRS="1", OMP_NUM_THREADS="4"))
    lines = dropin.smp_fixture(open(log).read().splitlines())
with open(os.path.join(HERE, "blaze_smp_calls.txt"), "w") as f:
    f.write("\n".join(lines) + "\n")
print(f"blaze_smp_calls.txt: {sum(1 for ln in lines if not ln.startswith('product'))} tile calls")

exe = dropin.build_blazetest("double")
with tempfile.TemporaryDirectory() as d:
    log = os.path.join(d, "log.txt")
    subprocess.run([exe], check=True, capture_output=True, env=dict(os.environ, GB300_STUB_LOG=log))
    raw = open(log).read().splitlines()
counts = {}
for ln in raw:
    counts[ln] = counts.get(ln, 0) + 1
with open(os.path.join(HERE, "blazetest_mdamda_calls.txt"), "w") as f:
    f.write("\n".join(f"{ln} {counts[ln]}" for ln in sorted(counts)) + "\n")
print(f"blazetest_mdamda_calls.txt: {len(counts)} distinct calls of {len(raw)}")
