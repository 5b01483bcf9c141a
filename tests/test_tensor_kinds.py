"""Which tcgen05 MMA kinds the target has: the residue (Ozaki scheme II) form keeps its 8-bit
residues in BF16 because sm_103a, unlike sm_100a, has no INT8 tensor-core MMA (tcgen05.mma
.kind::i8).  ptxas decides this at compile time, so the check needs nvcc, not a GPU."""
import os
import shutil
import subprocess

import pytest

NVCC = next((c for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")) if c and
             os.path.exists(c)), None)

SRC = r"""
#include <cstdint>
__global__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::KIND [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(d), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
"""


def compile_kind(tmp_path, kind, arch):
    src = tmp_path / f"mma_{kind}.cu"
    src.write_text(SRC.replace("KIND", kind))
    r = subprocess.run([NVCC, "-gencode", f"arch=compute_{arch},code=sm_{arch}", "-c", str(src), "-o",
                        str(tmp_path / f"mma_{kind}_{arch}.o")], capture_output=True, text=True)
    return r.returncode, r.stdout + r.stderr


@pytest.mark.skipif(NVCC is None, reason="nvcc not available")
def test_sm103a_has_bf16_but_no_int8_tensor_mma(tmp_path):
    rc, out = compile_kind(tmp_path, "f16", "103a")
    assert rc == 0, out
    rc, out = compile_kind(tmp_path, "i8", "103a")
    assert rc != 0 and "not supported" in out, out
    # the same instruction is accepted for sm_100a, so the rejection is the target's, not the syntax's
    rc, out = compile_kind(tmp_path, "i8", "100a")
    assert rc == 0, out
