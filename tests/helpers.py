"""Shared helpers of the test-suite: golden fixtures, operand layouts and tolerances."""
from __future__ import annotations

import os

import numpy as np

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gemm_golden.npz")

# Blaze's relaxed equality (blaze/math/shims/Equal.h:214-223; complex values part by part,
# :406-408): |a-b| <= max(acc, acc*|a|) with acc = 1e-8 for double and 1e-6 for float
# (blaze/util/Limits.h:366,398).
BLAZE_ACC = {np.float64: 1e-8, np.float32: 1e-6}


def blaze_equal(a: np.ndarray, b: np.ndarray, acc: float) -> np.ndarray:
    if np.iscomplexobj(a) or np.iscomplexobj(b):  # Blaze compares the real and imaginary parts
        a, b = np.asarray(a, dtype=np.complex128), np.asarray(b, dtype=np.complex128)
        return blaze_equal(a.real, b.real, acc) & blaze_equal(a.imag, b.imag, acc)
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) <= np.maximum(acc, acc * np.abs(a))


def stored_dims(order, trans, rows, cols):
    """(storage rows, storage cols) of a logical rows x cols operand in CBLAS (order, trans)."""
    t = trans != O.NO_TRANS
    r, c = (cols, rows) if t else (rows, cols)
    return (r, c) if order == O.ROW_MAJOR else (c, r)


_GOLDEN_CACHE = None


def load_golden():
    global _GOLDEN_CACHE
    if _GOLDEN_CACHE is not None:
        return _GOLDEN_CACHE
    with np.load(GOLDEN) as f:
        z = {key: f[key] for key in f.files}
    cases = []
    for i in range(len(z["m"])):
        c = {key: z[key][i].item() for key in z if key != "C"}
        c["dtype"] = np.float64 if c["dtype"] == 0 else np.float32
        c["C_ref"] = z["C"][c["offset"]: c["offset"] + c["size"]].astype(c["dtype"])
        cases.append(c)
    _GOLDEN_CACHE = cases
    return cases


def golden_inputs(c):
    """Regenerate the stored A, B and initial C buffers of a golden case from its seed."""
    dt = c["dtype"]
    ra, _ = stored_dims(c["order"], c["ta"], c["m"], c["k"])
    rb, _ = stored_dims(c["order"], c["tb"], c["k"], c["n"])
    rc, _ = stored_dims(c["order"], O.NO_TRANS, c["m"], c["n"])
    A = O.uniform(max(ra * c["lda"], 1), c["seed"], dtype=dt)
    B = O.uniform(max(rb * c["ldb"], 1), c["seed"] + 1, dtype=dt)
    C = O.uniform(max(rc * c["ldc"], 1), c["seed"] + 2, dtype=dt)
    return A, B, C


def logical_C(c, C):
    """The logical m x n result of a stored C buffer of a golden-style case."""
    return O.logical(c["order"], O.NO_TRANS, c["m"], c["n"], C, c["ldc"])


def normwise(C, Cref, normA, normB):
    d = np.asarray(C, np.float64) - np.asarray(Cref, np.float64)
    den = normA * normB
    num = float(np.sqrt(np.sum(d * d)))
    return num / den if den > 0 else num


def check_result(c, C_out, C_ref, C0=None):
    """Elementwise Blaze-relaxed check for double; normwise k*2^-24 (plus relaxed 1e-4) for float.

    Only the logical m x n part is compared; padding of the leading dimension must be untouched
    (compared with the initial buffer C0 when given)."""
    dt = c["dtype"]
    m, n, k = c["m"], c["n"], c["k"]
    L = logical_C(c, C_out)
    R = logical_C(c, C_ref)
    if m == 0 or n == 0:
        return
    if dt == np.float64:
        ok = blaze_equal(R, L, BLAZE_ACC[np.float64])
        assert ok.all(), f"{np.count_nonzero(~ok)} elements differ; max |d| = {np.max(np.abs(L - R))}"
    else:
        scale = max(1.0, float(np.max(np.abs(R)))) if R.size else 1.0
        err = float(np.max(np.abs(L.astype(np.float64) - R.astype(np.float64)))) if R.size else 0.0
        assert err <= max(k, 1) * 2.0 ** -22 * scale + 1e-6, f"float max |d| = {err}"
    if C0 is not None:
        mask = np.ones(C_out.shape, bool)
        idx = np.arange(C_out.size).reshape(-1)
        # positions of logical elements inside the storage buffer
        ld = c["ldc"]
        if c["order"] == O.ROW_MAJOR:
            pos = (np.arange(m)[:, None] * ld + np.arange(n)[None, :]).ravel()
        else:
            pos = (np.arange(n)[:, None] * ld + np.arange(m)[None, :]).ravel()
        mask[pos] = False
        assert np.array_equal(C_out[mask], C0[mask]), "padding of C was modified"
        del idx
