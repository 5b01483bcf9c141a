"""Record the CBLAS calls Blaze itself makes for `C = A*B`, `C += A*B`, `C -= A*B` and
`C = s*(A*B)` in BLAS mode (all storage-order classes and a CustomMatrix), by running the
drop-in program of tests/blaze_dropin/ against its logging stub.  Writes
tests/golden/blaze_calls.txt (one call per line: routine order transA transB m n k alpha lda ldb
beta ldc), which the GPU tests replay through the real library.  Needs the reference headers.
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "blaze_dropin"))
import build as dropin  # noqa: E402

exe = dropin.build("stub")
if exe is None:
    raise SystemExit("reference headers not available")
with tempfile.TemporaryDirectory() as d:
    log = os.path.join(d, "log.txt")
    subprocess.run([exe], check=True, env=dict(os.environ, GB300_STUB_LOG=log), capture_output=True)
    lines = open(log).read().splitlines()
with open(os.path.join(HERE, "blaze_calls.txt"), "w") as f:
    f.write("\n".join(lines) + "\n")
print(f"recorded {len(lines)} calls")
