"""Generate the golden GEMM fixtures from Blaze itself.

Run in a container that has the reference headers (Blaze is header-only):

    make -C oracle ref                       # builds oracle/_ref/libblazeref.so from the headers
    python tests/golden/make_golden.py       # writes tests/golden/gemm_golden.npz

Every case is C = alpha*op(A)*op(B) + beta*C in CBLAS conventions, evaluated by Blaze's default
(non-BLAS) kernels on blaze::CustomMatrix views of the buffers (oracle/blaze_ref.cpp).  Inputs
are not stored: they are regenerated from their seeds by the oracle's MT19937 generator, whose
first values are pinned by tests/test_oracle.py; the fixture keeps a checksum of each input so a
generator change is caught.  Shapes follow blazetest's dmatdmatmult suites
(blazetest/src/mathtest/operations/dmatdmatmult/MDaMDa.cpp: every (i,j,k) in 0..6 plus
combinations of 15, 16, 32, 37, 63, 64) and add shapes that cross the GPU kernels' 128-element
tile edges and padded leading dimensions.
"""
from __future__ import annotations

import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "gemm_golden.npz")


def stored_dims(order, trans, rows, cols):
    """(storage rows, storage cols) of a logical rows x cols operand in CBLAS (order, trans)."""
    t = trans != O.NO_TRANS
    r, c = (cols, rows) if t else (rows, cols)
    return (r, c) if order == O.ROW_MAJOR else (c, r)


def cases():
    out = []
    seed = 1000
    small = list(itertools.product(range(7), repeat=3))
    for (m, n, k) in small:
        out.append(("d", O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, 0.0, 0))
    mid = [(15, 16, 32), (37, 63, 15), (64, 64, 64), (63, 37, 16), (32, 15, 63), (16, 64, 37), (37, 37, 37)]
    big = [(1, 300, 5), (257, 1, 130), (200, 3, 1)]
    layouts = [(o, a, b) for o in (O.ROW_MAJOR, O.COL_MAJOR) for a in (O.NO_TRANS, O.TRANS) for b in (O.NO_TRANS, O.TRANS)]
    ab = [(1.0, 0.0), (1.0, 1.0), (-1.0, 1.0), (2.5, 0.0), (0.5, -1.5), (0.0, 2.0)]
    for dt in ("d", "s"):
        for i, (m, n, k) in enumerate(mid + big):
            for j, (order, ta, tb) in enumerate(layouts):
                al, be = ab[(i + j) % len(ab)]
                pad = (i + j) % 3  # 0, 1 or 2 extra elements of leading dimension
                out.append((dt, order, ta, tb, m, n, k, al, be, pad))
    # one larger product per storage-order combination (double), crossing 128-wide tile edges
    for j, (order, ta, tb) in enumerate(layouts):
        out.append(("d", order, ta, tb, 150 + j, 136 - j, 200 + 3 * j, (1.0, -2.0, 0.5)[j % 3], (0.0, 1.0, -1.0)[j % 3], j % 3))
    return out


def main():
    if O.build_ref() is None:
        raise SystemExit("reference headers not found; cannot build oracle/_ref")
    rec = {k: [] for k in ("dtype", "order", "ta", "tb", "m", "n", "k", "alpha", "beta", "lda", "ldb", "ldc",
                           "seed", "sumA", "sumB", "sumC0", "offset", "size")}
    outs = []
    off = 0
    for idx, (dt, order, ta, tb, m, n, k, al, be, pad) in enumerate(cases()):
        dtype = np.float64 if dt == "d" else np.float32
        ra, ca = stored_dims(order, ta, m, k)
        rb, cb = stored_dims(order, tb, k, n)
        rc, cc = stored_dims(order, O.NO_TRANS, m, n)
        lda, ldb, ldc = max(ca, 1) + pad, max(cb, 1) + pad, max(cc, 1) + pad
        seed = 7 + 3 * idx
        A = O.uniform(max(ra * lda, 1), seed, dtype=dtype)
        B = O.uniform(max(rb * ldb, 1), seed + 1, dtype=dtype)
        C = O.uniform(max(rc * ldc, 1), seed + 2, dtype=dtype)
        rec["sumC0"].append(float(np.sum(C, dtype=np.float64)))
        O.ref_gemm(order, ta, tb, m, n, k, al, A, lda, B, ldb, be, C, ldc)
        for key, v in (("dtype", 0 if dt == "d" else 1), ("order", order), ("ta", ta), ("tb", tb), ("m", m), ("n", n),
                       ("k", k), ("alpha", al), ("beta", be), ("lda", lda), ("ldb", ldb), ("ldc", ldc), ("seed", seed),
                       ("sumA", float(np.sum(A, dtype=np.float64))), ("sumB", float(np.sum(B, dtype=np.float64))),
                       ("offset", off), ("size", C.size)):
            rec[key].append(v)
        outs.append(C.astype(np.float64))
        off += C.size
    arrays = {k: np.array(v) for k, v in rec.items()}
    arrays["C"] = np.concatenate(outs)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: {len(rec['m'])} cases, {off} output elements")


if __name__ == "__main__":
    main()
