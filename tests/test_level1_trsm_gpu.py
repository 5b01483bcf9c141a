"""cblas_?trsm, cblas_?axpy and the dot products on a GB300, through the C-ABI:

- every dot / axpy / trsm case of tests/golden/next_golden.npz (Blaze's own x * y, conj(x) * y,
  y += alpha * x, and triangular systems whose right-hand sides Blaze formed as op(A) X0) within
  Blaze's relaxed equality, the check of blazetest's BLAS operation test;
- triangular solves past several 512-row leaf blocks of the recursion,
  every side / triangle /
  transposition / diagonal, against the oracle's substitution;
- strided and negative-stride vectors, incy = 0, n <= 0, alpha = 0 (B not read, A may be NULL);
- float forms (compensated float dot products: the double-rounded exact sum), device operands used
  in place, and dot products that give the same bits on every call."""
import os

import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O
from helpers import blaze_equal

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "next_golden.npz")
ACC = 1e-8
CONJ = 113


@pytest.fixture(scope="module")
def golden():
    z = np.load(GOLDEN)
    return {k: z[k] for k in z.files}


def cases(golden, prefix):
    return sorted({int(k[len(prefix):].split("_")[0]) for k in golden if k.startswith(prefix) and k.endswith("_meta")})


def positions(order, m, n, ld):
    ii, jj = np.arange(m)[:, None], np.arange(n)[None, :]
    return (ii * ld + jj) if order == O.ROW_MAJOR else (jj * ld + ii)


# ---- golden fixtures -----------------------------------------------------------------------------
def test_dot_matches_blaze(golden):
    for q in cases(golden, "dot"):
        cplx, conj, n, seed = (int(v) for v in golden[f"dot{q}_meta"])
        x = O.complex_uniform(n, seed) if cplx else O.uniform(n, seed).copy()
        y = O.complex_uniform(n, seed + 1) if cplx else O.uniform(n, seed + 1).copy()
        want = golden[f"dot{q}_r"][0]
        for sub in ((True, False) if cplx else (True,)):
            got = G.cblas_dot(n, x, 1, y, 1, dtype="z" if cplx else "d", conj=bool(conj), sub=sub)
            assert blaze_equal(np.array([got]), np.array([want]), ACC).all(), (q, got, want)


def test_axpy_matches_blaze(golden):
    for q in cases(golden, "axpy"):
        cplx, n, seed = (int(v) for v in golden[f"axpy{q}_meta"])
        al = golden[f"axpy{q}_alpha"][0]
        x = O.complex_uniform(n, seed) if cplx else O.uniform(n, seed).copy()
        y = O.complex_uniform(n, seed + 1) if cplx else O.uniform(n, seed + 1).copy()
        G.cblas_axpy(n, al if cplx else float(al.real), x, 1, y, 1, dtype="z" if cplx else "d")
        assert blaze_equal(y, golden[f"axpy{q}_y"], ACC).all(), q


def test_trsm_matches_blaze(golden):
    """op(A) X = alpha B with B = op(A) X0 formed by Blaze: the solve gives back alpha X0, the
    padding of B untouched."""
    assert len(cases(golden, "trsm")) >= 250
    for q in cases(golden, "trsm"):
        cplx, order, side, uplo, ta, diag, m, n, lda, ldb, pad, seed = (int(v) for v in golden[f"trsm{q}_meta"])
        al = golden[f"trsm{q}_alpha"][0]
        al = complex(al) if cplx else float(al.real)
        ka = m if side == 141 else n
        rb = m if order == O.ROW_MAJOR else n
        A, X0 = O.triangular_operands(bool(cplx), ka, lda, rb, ldb, seed)
        B = golden[f"trsm{q}_B"].copy()
        G.cblas_trsm(order, side, uplo, ta, diag, m, n, al, A, lda, B, ldb, dtype="z" if cplx else "d")
        E = X0.copy()
        pos = positions(order, m, n, ldb)
        E[pos] = al * E[pos]
        assert blaze_equal(B, E, ACC).all(), (q, order, side, uplo, ta, diag, m, n)
        mask = np.ones(B.size, bool)
        mask[pos.reshape(-1)] = False
        assert np.array_equal(B[mask], golden[f"trsm{q}_B"][mask]), q


# ---- triangular solves past several recursion blocks ---------------------------------------------
SOLVES = [
    # (cplx, order, side, uplo, trans, diag, m, n)
    (0, 101, 141, 122, 111, 131, 700, 96),
    (0, 101, 141, 121, 111, 132, 700, 96),
    (0, 101, 141, 122, 112, 131, 520, 64),
    (0, 101, 142, 122, 111, 131, 80, 1100),
    (0, 101, 142, 121, 112, 132, 80, 610),
    (0, 102, 141, 121, 111, 131, 777, 33),
    (0, 102, 142, 122, 112, 131, 45, 513),
    (0, 102, 141, 122, 112, 132, 257, 300),
    (1, 101, 141, 122, 113, 131, 530, 40),
    (1, 101, 142, 121, 111, 131, 40, 530),
    (1, 102, 141, 121, 112, 132, 300, 24),
    (1, 102, 142, 122, 113, 131, 24, 600),
]


@pytest.mark.parametrize("case", SOLVES)
def test_trsm_large_against_oracle(case):
    cplx, order, side, uplo, ta, diag, m, n = case
    ka = m if side == 141 else n
    lda = ka + 3
    rb, cb = (m, n) if order == O.ROW_MAJOR else (n, m)
    ldb = cb + 5
    A, B = O.triangular_operands(bool(cplx), ka, lda, rb, ldb, 4242 + m + n)
    al = (0.75 - 0.5j) if cplx else -1.25
    want = B.copy()
    O.trsm(order, side, uplo, ta, diag, m, n, al, A, lda, want, ldb)
    got = B.copy()
    G.cblas_trsm(order, side, uplo, ta, diag, m, n, al, A, lda, got, ldb, dtype="z" if cplx else "d")
    pos = positions(order, m, n, ldb)
    X, Xr = got[pos], want[pos]
    assert np.linalg.norm(X - Xr) <= 1e-12 * np.linalg.norm(Xr), case
    assert blaze_equal(got, want, ACC).all(), case
    # the residual of the system itself
    T = O.triangle_logical(order, uplo, ta, diag, ka, A, lda)
    Bl = B[pos]
    R = (T @ X if side == 141 else X @ T) - al * Bl
    assert np.linalg.norm(R) <= 1e-13 * np.linalg.norm(T) * np.linalg.norm(X), case


def test_trsm_float_forms():
    for cplx in (0, 1):
        for side, uplo, ta in ((141, 122, 111), (142, 121, 112), (141, 121, CONJ if cplx else 112)):
            m, n = (300, 40) if side == 141 else (40, 300)
            ka = m if side == 141 else n
            A, B = O.triangular_operands(bool(cplx), ka, ka, m, n, 99 + side + uplo)
            al = (0.5 + 0.5j) if cplx else 2.0
            want = B.copy()
            O.trsm(101, side, uplo, ta, 131, m, n, al, A, ka, want, n)
            dt = np.complex64 if cplx else np.float32
            Af, Bf = A.astype(dt), B.astype(dt)
            G.cblas_trsm(101, side, uplo, ta, 131, m, n, al, Af, ka, Bf, n, dtype="c" if cplx else "s")
            err = np.linalg.norm(Bf.astype(np.complex128 if cplx else np.float64) - want) / np.linalg.norm(want)
            assert err <= 1e-5, (cplx, side, uplo, ta, err)


def test_trsm_alpha_zero_and_empty():
    B = np.full(6 * 4, np.nan)
    G.cblas_trsm(101, 141, 122, 111, 131, 6, 4, 0.0, None, 6, B, 4)  # A not read
    assert np.all(B == 0.0)
    B = np.arange(12.0)
    G.cblas_trsm(101, 141, 122, 111, 131, 0, 4, 1.0, None, 1, B, 4)  # m = 0: nothing to do
    assert np.array_equal(B, np.arange(12.0))


def test_trsm_device_operands_in_place():
    torch = pytest.importorskip("torch")
    m, n = 600, 50
    A, B = O.triangular_operands(False, m, m, m, n, 31)
    want = B.copy()
    O.trsm(101, 141, 121, 112, 131, m, n, 1.0, A, m, want, n)
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    torch.cuda.synchronize()
    G.cblas_trsm(101, 141, 121, 112, 131, m, n, 1.0, dA, m, dB, n)
    torch.cuda.synchronize()
    assert blaze_equal(dB.cpu().numpy(), want, ACC).all()


# ---- vectors -------------------------------------------------------------------------------------
@pytest.mark.parametrize("incx,incy", [(1, 1), (3, 2), (-2, 1), (1, -3), (-1, -1), (0, 1)])
def test_axpy_and_dot_strides(incx, incy):
    n = 1237
    ax, ay = abs(incx), abs(incy)
    x = O.uniform(1 + (n - 1) * ax, 5).copy()
    y = O.uniform(1 + (n - 1) * ay, 6).copy()
    # logical element i of a vector with a negative stride sits at (n - 1 - i) * |inc|
    xi = np.arange(n) * ax if incx >= 0 else (n - 1 - np.arange(n)) * ax
    yi = np.arange(n) * ay if incy >= 0 else (n - 1 - np.arange(n)) * ay
    want = float(np.sum(x[xi] * y[yi]))
    got = G.cblas_dot(n, x, incx, y, incy)
    assert abs(got - want) <= 1e-13 * np.sum(np.abs(x[xi] * y[yi]))
    z = y.copy()
    G.cblas_axpy(n, 0.5, x, incx, z, incy)
    ref = y.copy()
    ref[yi] = 0.5 * x[xi] + y[yi]
    assert blaze_equal(z, ref, ACC).all()


def test_axpy_incy_zero_and_quick_returns():
    x = O.uniform(10, 1).copy()
    y = np.array([2.0])
    G.cblas_axpy(10, 3.0, x, 1, y, 0)  # all ten updates land on y[0], in order
    ref = 2.0
    for v in x:
        ref = ref + 3.0 * v
    assert abs(y[0] - ref) <= 1e-14 * 40
    y = np.arange(5.0)
    G.cblas_axpy(5, 0.0, None, 1, y, 1)  # alpha = 0: y as it was, x not read
    G.cblas_axpy(0, 2.0, None, 1, y, 1)
    assert np.array_equal(y, np.arange(5.0))
    assert G.cblas_dot(0, None, 1, None, 1) == 0.0
    assert G.cblas_dot(-3, None, 1, None, 1, dtype="z") == 0j


def test_complex_dot_and_axpy_strided():
    n = 999
    x = O.complex_uniform(2 * n, 3)
    y = O.complex_uniform(3 * n, 4)
    xs = x[::2][:n]
    xv, yv = x[: 2 * n], y[: 3 * (n - 1) + 1]
    u = G.cblas_dot(n, xv, 2, yv, -3, dtype="z")
    c = G.cblas_dot(n, xv, 2, yv, -3, dtype="z", conj=True)
    yi = (n - 1 - np.arange(n)) * 3
    assert abs(u - np.sum(xs * yv[yi])) <= 1e-12 * n
    assert abs(c - np.sum(xs.conj() * yv[yi])) <= 1e-12 * n
    z = yv.copy()
    G.cblas_axpy(n, 0.25 - 2j, xv, 2, z, -3, dtype="z")
    ref = yv.copy()
    ref[yi] = (0.25 - 2j) * xs + yv[yi]
    assert blaze_equal(z, ref, ACC).all()


def test_float_dot_is_compensated():
    """sdot / cdotu sum in the compensated scheme and round once: the result is the float
    nearest the exact sum, within one unit in the last place, even with heavy cancellation."""
    rng = np.random.default_rng(11)
    n = 1 << 20
    h = n // 2
    x = rng.uniform(-1, 1, n).astype(np.float32)
    y = rng.uniform(-1, 1, n).astype(np.float32)
    # the second half nearly cancels the first: the sum is about 1e-6 of sum |x y|, where plain float
    # accumulation would be off by about 1e-5 absolute
    x[h:] = x[:h]
    y[h:] = (-y[:h] * (1 + 2.0 ** -10 * rng.uniform(-1, 1, h))).astype(np.float32)
    exact = float(np.sum(x.astype(np.float64) * y.astype(np.float64)))  # products exact in double
    mag = float(np.sum(np.abs(x.astype(np.float64) * y)))
    got = G.cblas_dot(n, x, 1, y, 1, dtype="s")
    assert abs(got - exact) <= 2 * np.spacing(np.float32(abs(exact))) + 1e-12 * mag, (got, exact)
    xc = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    yc = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    ex = np.sum(xc.conj().astype(np.complex128) * yc.astype(np.complex128))
    gc = G.cblas_dot(n, xc, 1, yc, 1, dtype="c", conj=True)
    assert abs(gc.real - ex.real) <= 2 * np.spacing(np.float32(abs(ex.real))) + 1e-12 * n
    assert abs(gc.imag - ex.imag) <= 2 * np.spacing(np.float32(abs(ex.imag))) + 1e-12 * n


def test_large_dot_deterministic_and_device_resident():
    torch = pytest.importorskip("torch")
    n = 50_000_003
    g = torch.Generator(device="cuda").manual_seed(5)
    dx = torch.rand(n, device="cuda", dtype=torch.float64, generator=g) * 2 - 1
    dy = torch.rand(n, device="cuda", dtype=torch.float64, generator=g) * 2 - 1
    torch.cuda.synchronize()  # the library works on its own stream: the operands must be ready
    a = G.cblas_dot(n, dx, 1, dy, 1)
    b = G.cblas_dot(n, dx, 1, dy, 1)
    assert a == b  # fixed reduction order
    ref = float(torch.dot(dx, dy).item())
    assert abs(a - ref) <= 1e-12 * float(torch.sum(torch.abs(dx * dy)).item())
    dz = dy.clone()
    torch.cuda.synchronize()
    G.cblas_axpy(n, -2.0, dx, 1, dz, 1)
    torch.cuda.synchronize()
    assert torch.equal(dz, dy - 2.0 * dx)  # 2 x is exact, so y - 2 x rounds once, like the FMA


def test_ilp64_entries_compute_the_same():
    """The _64 symbols (BLAZE_BLAS_IS_64BIT) of the new routines give the 32-bit entries' results."""
    import ctypes as ct
    L = G.lib()
    I64, VP = ct.c_int64, ct.c_void_p
    L.cblas_ddot_64.argtypes = [I64, VP, I64, VP, I64]
    L.cblas_ddot_64.restype = ct.c_double
    L.cblas_daxpy_64.argtypes = [I64, ct.c_double, VP, I64, VP, I64]
    L.cblas_daxpy_64.restype = None
    L.cblas_dtrsm_64.argtypes = [ct.c_int] * 5 + [I64, I64, ct.c_double, VP, I64, VP, I64]
    L.cblas_dtrsm_64.restype = None
    L.cblas_zdotc_sub_64.argtypes = [I64, VP, I64, VP, I64, VP]
    L.cblas_zdotc_sub_64.restype = None
    n = 3001
    x, y = O.uniform(n, 81).copy(), O.uniform(n, 82).copy()
    assert L.cblas_ddot_64(n, x.ctypes.data, 1, y.ctypes.data, 1) == G.cblas_dot(n, x, 1, y, 1)
    y1, y2 = y.copy(), y.copy()
    L.cblas_daxpy_64(n, -0.5, x.ctypes.data, 1, y1.ctypes.data, 1)
    G.cblas_axpy(n, -0.5, x, 1, y2, 1)
    assert np.array_equal(y1, y2)
    zx, zy = O.complex_uniform(n, 83), O.complex_uniform(n, 84)
    out = np.zeros(1, dtype=np.complex128)
    L.cblas_zdotc_sub_64(n, zx.ctypes.data, 1, zy.ctypes.data, 1, out.ctypes.data)
    assert out[0] == G.cblas_dot(n, zx, 1, zy, 1, dtype="z", conj=True)
    m, k = 700, 40
    A, B = O.triangular_operands(False, m, m, m, k, 85)
    B1, B2 = B.copy(), B.copy()
    L.cblas_dtrsm_64(101, 141, 122, 111, 131, m, k, 1.5, A.ctypes.data, m, B1.ctypes.data, k)
    G.cblas_trsm(101, 141, 122, 111, 131, m, k, 1.5, A, m, B2, k)
    assert np.array_equal(B1, B2)
    assert G.last_error()[0] == G.OK
