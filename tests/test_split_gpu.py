"""Tensor-core forms (split-precision FP64-accurate, BF16x3, BF16) through the C-ABI on a GB300:
normwise error against the compensated FP64 oracle within each form's stated bound, every
storage-order combination, alpha/beta, skinny and split-k shapes, exponent-spread inputs,
exactness of the integer slice products at their largest magnitudes, and non-finite inputs."""
import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O
from helpers import check_result, golden_inputs, load_golden, normwise, stored_dims

pytestmark = pytest.mark.gpu

FP64_BOUND = 2.0 ** -53


@pytest.fixture(scope="module", autouse=True)
def lib():
    L = G.lib()
    G.device_info()
    return L


def product(order, ta, tb, m, n, k, dist="uniform", seed=1, pad=0, alpha=1.0, beta=0.0, method="split", slices=0):
    ra, ca = stored_dims(order, ta, m, k)
    rb, cb = stored_dims(order, tb, k, n)
    rc, cc = stored_dims(order, O.NO_TRANS, m, n)
    lda, ldb, ldc = ca + pad, cb + pad, cc + pad
    gen = O.uniform if dist == "uniform" else O.spread
    A = gen(max(ra * lda, 1), seed)
    B = gen(max(rb * ldb, 1), seed + 1)
    C = O.uniform(max(rc * ldc, 1), seed + 2)
    C0 = C.copy()
    o = G.dgemm_ex(order, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, G.opts(method=method, slices=slices))
    P = O.product_rows_dot2(order, ta, tb, m, n, k, A, lda, B, ldb)
    Cl0 = O.logical(order, O.NO_TRANS, m, n, C0, ldc)
    out = O.logical(order, O.NO_TRANS, m, n, C, ldc)
    nA = O.fro_norm_op(order, ta, m, k, A, lda)
    nB = O.fro_norm_op(order, tb, k, n, B, ldb)
    err = normwise((out - beta * Cl0) / alpha, P, nA, nB)
    return err, o, out, P


LAYOUTS = [(o, a, b) for o in (O.ROW_MAJOR, O.COL_MAJOR) for a in (O.NO_TRANS, O.TRANS) for b in (O.NO_TRANS, O.TRANS)]


@pytest.mark.parametrize("order,ta,tb", LAYOUTS)
@pytest.mark.parametrize("dist", ["uniform", "spread"])
def test_split_meets_fp64_bound(order, ta, tb, dist):
    m, n, k = 300, 517, 777
    err, o, _, _ = product(order, ta, tb, m, n, k, dist=dist, pad=3, alpha=1.25, beta=-0.5)
    assert o.method_used in (G.METHOD_SPLIT, G.METHOD_SPLIT_CRT)
    assert 2 <= o.slices_used <= 15
    assert o.error_bound <= k * FP64_BOUND
    assert err <= o.error_bound, (err, o.error_bound)
    assert err <= k * FP64_BOUND


@pytest.mark.parametrize("slices", [2, 3, 4, 5, 6, 7, 8])
def test_error_falls_with_slices(slices):
    """Each added slice buys about 8 bits; the reported a-priori bound always holds."""
    err, o, _, _ = product(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, 200, 264, 1000, slices=slices, seed=5)
    assert o.slices_used == slices
    assert err <= o.error_bound
    assert err <= 2.0 ** (-8 * slices + 1)


@pytest.mark.parametrize("method,bound", [("bf16x3", 2.0 ** -14), ("bf16", 2.0 ** -6)])
def test_bf16_forms_within_stated_error(method, bound):
    for order, ta, tb in LAYOUTS[::3]:
        err, o, _, _ = product(order, ta, tb, 333, 290, 650, method=method, seed=9)
        assert o.method_used == G.METHODS[method]
        assert err <= o.error_bound and err <= bound, (method, err, o.error_bound)


@pytest.mark.parametrize("m,n,k", [(256, 256, 16384), (2000, 64, 3000), (1, 700, 900), (900, 1, 300), (5, 7, 3)])
def test_skinny_and_split_k_shapes(m, n, k):
    err, o, _, _ = product(O.COL_MAJOR, O.TRANS, O.NO_TRANS, m, n, k, seed=13)
    assert err <= max(o.error_bound, 1e-300) and err <= k * FP64_BOUND


def test_golden_cases_split():
    """Blaze's own outputs for every double golden case through cblas_dgemm in split mode."""
    prev = G.lib().gb300_set_default_method(G.METHOD_SPLIT)
    try:
        for c in load_golden():
            if c["dtype"] != np.float64:
                continue
            A, B, C = golden_inputs(c)
            C0 = C.copy()
            G.cblas_dgemm(c["order"], c["ta"], c["tb"], c["m"], c["n"], c["k"], c["alpha"], A, c["lda"], B, c["ldb"],
                          c["beta"], C, c["ldc"])
            check_result(c, C, c["C_ref"], C0)
    finally:
        G.lib().gb300_set_default_method(prev)


def test_integer_slices_are_exact_at_the_largest_digit_sums():
    """Operands whose every digit is +-128 with one sign make each 256-product group sum to
    exactly +-2^22, the largest magnitude the scheme relies on; products of integers that the
    split represents exactly must come back exact."""
    m, n, k = 128, 256, 4096
    # entries 1 - 2^-9: first digit rint(0.998*128) = 128, remainder -0.25*... ; use powers of two
    A = np.full(m * k, 0.99609375)  # 255/256: scaled by 2^0 -> x*128 = 127.5 -> digit 128 (ties to even)
    B = np.full(k * n, 0.99609375)
    C = np.zeros(m * n)
    G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method="split"))
    assert np.all(C == k * 0.99609375 ** 2)
    # integers in [-1000, 1000]: the exact product is an integer the split reproduces exactly
    A = O.integers(m * k, 3, -1000, 1000)
    B = O.integers(k * n, 4, -1000, 1000)
    G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method="split"))
    exact = A.astype(np.int64).reshape(m, k) @ B.astype(np.int64).reshape(k, n)
    assert np.array_equal(C.reshape(m, n), exact.astype(np.float64))


def test_nonfinite_inputs_poison_their_rows_and_columns():
    m, n, k = 130, 260, 300
    A = O.uniform(m * k, 1); B = O.uniform(k * n, 2)
    A[5 * k + 7] = np.inf
    B[11 * n + 3] = np.nan
    C = np.zeros(m * n)
    G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method="split"))
    C = C.reshape(m, n)
    assert np.all(np.isnan(C[5, :])) and np.all(np.isnan(C[:, 3]))
    mask = np.ones((m, n), bool); mask[5, :] = False; mask[:, 3] = False
    assert np.isfinite(C[mask]).all()


def test_auto_picks_a_fp64_accurate_form():
    m = n = k = 512
    err, o, _, _ = product(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, method="auto", seed=17)
    assert o.method_used in (G.METHOD_SPLIT, G.METHOD_SPLIT_CRT, G.METHOD_NATIVE)
    assert err <= k * FP64_BOUND


def test_split_stall_reports_timeout_and_recovers():
    m = n = k = 256
    A = O.uniform(m * k, 61); B = O.uniform(k * n, 62); C = np.zeros(m * n)
    G.lib().gb300_debug_inject_stall(1, 20_000_000)
    with pytest.raises(G.Gb300Error) as ei:
        G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method="split"))
    assert ei.value.status == G.ERR_DEVICE_TIMEOUT
    G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method="split"))
    assert np.allclose(C.reshape(m, n), A.reshape(m, k) @ B.reshape(k, n), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("order,ta,tb", LAYOUTS[::2])
@pytest.mark.parametrize("dist", ["uniform", "spread"])
@pytest.mark.parametrize("scheme", ["split_crt", "digits"])
def test_both_fp64_accurate_schemes(order, ta, tb, dist, scheme):
    """The residue (CRT) scheme and the digit scheme both meet the FP64 bound on every layout."""
    m, n, k = 260, 300, 1111
    if scheme == "digits":
        # a slice count selects the digit scheme; 7 slices reach the bound for both distributions
        err, o, _, _ = product(order, ta, tb, m, n, k, dist=dist, seed=21, method="split", slices=7)
        assert o.method_used == G.METHOD_SPLIT and o.slices_used == 7
    else:
        err, o, _, _ = product(order, ta, tb, m, n, k, dist=dist, seed=21, method="split_crt")
        assert o.method_used == G.METHOD_SPLIT_CRT and 2 <= o.slices_used <= 15
    assert err <= o.error_bound <= k * FP64_BOUND, (scheme, err, o.error_bound)


def test_crt_scheme_is_the_default_split_for_large_k_and_exact_on_integers():
    m, n, k = 256, 256, 20000
    A = O.integers(m * k, 31, -1000, 1000)
    B = O.integers(k * n, 32, -1000, 1000)
    C = np.zeros(m * n)
    o = G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n, G.opts(method="split"))
    assert o.method_used == G.METHOD_SPLIT_CRT
    exact = A.astype(np.int64).reshape(m, k) @ B.astype(np.int64).reshape(k, n)
    assert np.array_equal(C.reshape(m, n), exact.astype(np.float64))


def test_crt_with_a_moduli_cap_reports_its_weaker_bound():
    m, n, k = 200, 200, 800
    err, o, _, _ = product(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, method="split_crt", slices=8, seed=41)
    assert o.slices_used == 8
    assert err <= o.error_bound


@pytest.mark.parametrize("slices", [1, 2, 3, 4, 5, 7, 8, 11, 12, 13, 15])
def test_crt_every_modulus_count_is_exact_on_small_integers(slices):
    """Each modulus count has its own reconstruction table (1 to 4 result limbs, singles and
    pairs): with entries in [-3, 3] every count carries the scaled product exactly (one modulus
    is raised to two)."""
    m, n, k = 130, 260, 64
    A = O.integers(m * k, 51 + slices, -3, 3)
    B = O.integers(k * n, 52 + slices, -3, 3)
    C = np.zeros(m * n)
    o = G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n,
                   G.opts(method="split_crt", slices=slices))
    assert o.method_used == G.METHOD_SPLIT_CRT
    assert o.slices_used == max(2, slices)
    exact = A.astype(np.int64).reshape(m, k) @ B.astype(np.int64).reshape(k, n)
    assert np.array_equal(C.reshape(m, n), exact.astype(np.float64))


def test_crt_segmented_k_residues_are_summed_and_reduced():
    """Few output tiles make the product split k into segments whose residues the combine kernel
    adds and reduces again; integer inputs must still come back exact."""
    m, n, k = 100, 120, 9000
    A = O.integers(m * k, 61, -500, 500)
    B = O.integers(k * n, 62, -500, 500)
    C = np.zeros(m * n)
    o = G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n,
                   G.opts(method="split_crt"))
    assert o.method_used == G.METHOD_SPLIT_CRT
    exact = A.astype(np.int64).reshape(m, k) @ B.astype(np.int64).reshape(k, n)
    assert np.array_equal(C.reshape(m, n), exact.astype(np.float64))


@pytest.mark.parametrize("order,ta,tb", [(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS), (O.COL_MAJOR, O.TRANS, O.TRANS)])
def test_rows_of_extreme_magnitude_keep_their_own_scale(order, ta, tb):
    """Rows of A and columns of B at the ends of the double range: zero, subnormal values whose high
    word is zero, subnormals with a non-zero high word, 1e300, 1e-300, one large value among ones.
    Every output entry is checked against its own row and column scale, so a wrong row exponent
    cannot hide behind the largest entries."""
    m, n, k = 64, 96, 300
    rng = np.random.default_rng(5)
    Al = rng.uniform(-1, 1, (m, k))
    Bl = rng.uniform(-1, 1, (k, n))
    Al[0] = 0.0
    Al[1] = np.ldexp(np.round(Al[1] * 2 ** 14), -1074)        # low word only
    Al[2] = np.ldexp(Al[2], -1030)                              # subnormal, high word non-zero
    Al[3] *= 1e300
    Al[4] *= 1e-300
    Al[5, 17] = 1e200
    Bl[:, 0] = np.ldexp(np.round(Bl[:, 0] * 2 ** 12), -1074)
    Bl[:, 1] *= 1e-250
    Bl[:, 2] *= 1e5
    Bl[:, 3] = 0.0

    def stored(L, trans):
        X = L.T if trans == O.TRANS else L
        return np.ascontiguousarray(X if order == O.ROW_MAJOR else X.T).ravel()

    A, B = stored(Al, ta), stored(Bl, tb)
    ra, ca = stored_dims(order, ta, m, k)
    rb, cb = stored_dims(order, tb, k, n)
    lda, ldb = ca, cb
    ldc = n if order == O.ROW_MAJOR else m
    C = np.zeros(m * n)
    o = G.dgemm_ex(order, ta, tb, m, n, k, 1.0, A, lda, B, ldb, 0.0, C, ldc, G.opts(method="split"))
    assert o.method_used in (G.METHOD_SPLIT, G.METHOD_SPLIT_CRT)
    out = O.logical(order, O.NO_TRANS, m, n, C, ldc)
    P = O.product_rows_dot2(order, ta, tb, m, n, k, A, lda, B, ldb)
    scale = np.outer(np.abs(Al).max(axis=1), np.abs(Bl).max(axis=0)) * k
    # the rounding of both operands to beta-bit integers bounds an entry's error by about
    # k 2^(e_i + f_j - beta) with beta near 40 here
    tol = np.maximum(scale * 2.0 ** -36, 4 * k * 2.0 ** -1074)
    assert np.isfinite(out).all()
    bad = np.abs(out - P) > tol
    assert not bad.any(), [(int(i), int(j), out[i, j], P[i, j]) for i, j in zip(*np.nonzero(bad))][:8]
    assert np.all(out[0] == 0.0) and np.all(out[:, 3] == 0.0)
    assert np.count_nonzero(out[1]) > n // 2 and np.count_nonzero(out[:, 0]) > m // 2


MODULI = [257, 256, 255, 253, 251, 247, 241, 239, 233, 229, 227, 223, 217, 211, 199]


def _crt_beta(qa, qb, k, nmod):
    """The residue plan's rounding exponent for fixed moduli: the largest b whose integer products
    fit the moduli (the planning kernel's need(b) <= have, in FP64 as there)."""
    import math
    have = sum(math.log2(p) for p in MODULI[:nmod])
    sqa, sqb, hk = math.sqrt(qa * (1 + 2.0 ** -10)), math.sqrt(qb * (1 + 2.0 ** -10)), 0.5 * math.sqrt(k)
    need = lambda b: 1.0875 + math.log2(math.ldexp(sqa, b) + hk) + math.log2(math.ldexp(sqb, b) + hk)
    bhi = min(55, math.floor((have - 1.0875 - math.log2(sqa) - math.log2(sqb)) / 2.0))
    return max(b for b in range(-59, bhi + 1) if need(b) <= have)


def test_crt_drain_groups_exact_at_their_largest_sums():
    """The worst case of the residue products' FP32 accumulation: every 257-residue of one
    1024-long k block is 128 in both operands (the 256-residues are +-128), so each drain group
    there sums 128 * 128 products to its largest magnitude.  Block g of k holds values
    Y / 2^(b0 - 7 + g) with Y = 128 mod 256 * 257, so the block whose exponent equals the plan's
    beta has exactly those residues; the plan's beta is recovered from the returned bound.  Every
    entry is exact at that scale, so the result must be the correctly rounded exact product."""
    from fractions import Fraction
    m = n = 2048   # 64 pair tiles: k is not split into segments
    k, blk, nmod = 8192, 1024, 13
    rng = np.random.default_rng(11)

    def block_values(count, b):
        lo_t = -(-(2 ** (b - 1) - 128) // 65792)
        hi_t = (2 ** b - 1 - 128) // 65792
        return [65792 * int(t) + 128 for t in rng.integers(lo_t, hi_t + 1, count)]

    # a first draft fixes the operand statistics; the block exponents sit at and below its beta
    b0 = _crt_beta(k * 0.58, k * 0.58, k, nmod)
    for _ in range(3):
        exps = [b0 - 7 + g for g in range(k // blk)]
        ya = [y for g, b in enumerate(exps) for y in block_values(blk, b)]
        yb = [y for g, b in enumerate(exps) for y in block_values(blk, b)]
        a = np.array([y / 2.0 ** exps[p // blk] for p, y in enumerate(ya)])
        b = np.array([y / 2.0 ** exps[p // blk] for p, y in enumerate(yb)])
        beta = _crt_beta(float(np.sum(a * a)), float(np.sum(b * b)), k, nmod)
        if beta == b0:
            break
        b0 = beta
    assert beta == b0
    assert a.max() < 1.0 and a.min() >= 0.5 and b.max() < 1.0 and b.min() >= 0.5  # row exponents 0
    A = np.tile(a, m)            # m x k, every row a
    B = np.repeat(b, n)          # k x n, every column b
    C = np.zeros(m * n)
    o = G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, C, n,
                   G.opts(method="split_crt", slices=nmod))
    assert o.method_used == G.METHOD_SPLIT_CRT and o.slices_used == nmod
    # the beta that ran, from its bound 2^(-b-1)(rA + rB) + 2^(-2b-2) rA rB + 2^-52
    rA, rB = np.sqrt(k / np.sum(a * a)), np.sqrt(k / np.sum(b * b))
    bnd = {bb: 2.0 ** (-bb - 1) * (rA + rB) + 2.0 ** (-2 * bb - 2) * rA * rB + 2.0 ** -52 for bb in range(b0 - 8, b0 + 9)}
    # (the device's norms come from FP32 sums; bounds of neighbouring exponents differ by 2x)
    ran = [bb for bb, v in bnd.items() if abs(v - o.error_bound) <= 1e-3 * o.error_bound]
    assert ran == [b0], (ran, b0, o.error_bound)
    # exact product: sum_p Y_p Z_p 2^-(2 e_p), correctly rounded
    top = max(exps)
    num = sum(ya[p] * yb[p] << (2 * (top - exps[p // blk])) for p in range(k))
    exact = float(Fraction(num, 2 ** (2 * top)))
    assert np.all(C == exact), (float(C.min()), float(C.max()), exact)


def test_column_parts_join_the_callers_stream():
    """A large residue product runs its tensor-core work as two column parts and reconstructs the
    first part on a second stream.  Two asynchronous calls on a user stream (the second with
    beta = 1, so it reads the first's C) must be complete once that stream alone is synchronised."""
    torch = pytest.importorskip("torch")
    m, n, k = 4096, 4096, 512   # 16 x 16 = 256 pair tiles, at least one per SM: two column parts
    A = O.uniform(m * k, 71)
    B = O.uniform(k * n, 72)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dC = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    o = G.opts(method="split_crt", residency=G.PTR_DEVICE, stream=s.cuda_stream, synchronous=False)
    G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, dA, k, dB, n, 0.0, dC, n, o)
    G.dgemm_ex(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, dA, k, dB, n, 1.0, dC, n, o)
    s.synchronize()
    got = dC.cpu().numpy().reshape(m, n)
    rows = np.arange(0, m, 97)
    P = O.product_rows_dot2(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, A, k, B, n, rows=rows)
    err = np.max(np.abs(got[rows] - 2.0 * P))
    assert err <= 1e-11, err
