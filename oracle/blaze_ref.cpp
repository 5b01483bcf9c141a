// blaze_ref.cpp — builds Blaze itself (the reference, header-only) into oracle/_ref/libblazeref.so.
//
// TEST INFRASTRUCTURE ONLY: used in this container to pin the C restatement (oracle_blaze.c)
// and to write the golden fixtures under tests/golden/.  It is compiled from the reference's
// own headers by oracle/Makefile (`make -C oracle ref`); no reference source is copied here.
//
// Each entry point wraps the caller's buffers in blaze::CustomMatrix views with the storage
// orders a CBLAS (order, transA, transB) triple describes, exactly as blaze::gemm() derives them
// in reverse (blaze/math/blas/gemm.h:115-131: order from C, transX = (SO_C != SO_X)), and then
// evaluates the product with Blaze's default kernels (BLAZE_BLAS_MODE=0):
//     beta == 0:  C = alpha * (A * B)                (DMatScalarMultExpr<...MultExpr>, assign)
//     otherwise:  C *= beta;  C += alpha * (A * B)   (addAssign of the scaled product)
// so the four expression classes DMatDMatMultExpr, DMatTDMatMultExpr, TDMatDMatMultExpr and
// TDMatTDMatMultExpr are all reached.  The library is built without OpenMP, so Blaze evaluates
// serially: its SMP layer rejects some unaligned CustomMatrix views with odd leading dimensions
// ("Invalid submatrix alignment"), while the serial kernels accept every layout.
#include <blaze/Math.h>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <exception>

namespace {

using blaze::columnMajor;
using blaze::rowMajor;
using blaze::unaligned;
using blaze::unpadded;

template <typename T, bool SO>
using View = blaze::CustomMatrix<T, unaligned, unpadded, SO>;

template <typename T, bool SOC, bool SOA, bool SOB>
void run(int64_t m, int64_t n, int64_t k, T alpha, const T* A, int64_t lda, const T* B,
         int64_t ldb, T beta, T* C, int64_t ldc) {
    View<T, SOA> a(const_cast<T*>(A), m, k, lda);
    View<T, SOB> b(const_cast<T*>(B), k, n, ldb);
    View<T, SOC> c(C, m, n, ldc);
    if (beta == T(0)) {
        c = alpha * (a * b);
    } else {
        c *= beta;
        c += alpha * (a * b);
    }
}

template <typename T>
void dispatch(int order, int tA, int tB, int64_t m, int64_t n, int64_t k, T alpha, const T* A,
              int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc) {
    const bool rm = (order == 101);
    const bool ta = (tA != 111), tb = (tB != 111);
    // storage order of each operand view: same as C unless transposed
    const bool soA = rm ? (ta ? columnMajor : rowMajor) : (ta ? rowMajor : columnMajor);
    const bool soB = rm ? (tb ? columnMajor : rowMajor) : (tb ? rowMajor : columnMajor);
#define GB_CASE(SC, SA, SB)                                                                     \
    if ((rm ? rowMajor : columnMajor) == SC && soA == SA && soB == SB) {                        \
        run<T, SC, SA, SB>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);                       \
        return;                                                                                 \
    }
    GB_CASE(rowMajor, rowMajor, rowMajor)
    GB_CASE(rowMajor, rowMajor, columnMajor)
    GB_CASE(rowMajor, columnMajor, rowMajor)
    GB_CASE(rowMajor, columnMajor, columnMajor)
    GB_CASE(columnMajor, rowMajor, rowMajor)
    GB_CASE(columnMajor, rowMajor, columnMajor)
    GB_CASE(columnMajor, columnMajor, rowMajor)
    GB_CASE(columnMajor, columnMajor, columnMajor)
#undef GB_CASE
}

}  // namespace

extern "C" {

// Returns 0, or 1 when Blaze threw (the message is printed to stderr).
int ref_gemm_d(int order, int tA, int tB, int64_t m, int64_t n, int64_t k, double alpha,
               const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
               double* C, int64_t ldc) {
    try {
        dispatch<double>(order, tA, tB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "blaze: %s\n", e.what());
        return 1;
    }
    return 0;
}

int ref_gemm_s(int order, int tA, int tB, int64_t m, int64_t n, int64_t k, float alpha,
               const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C,
               int64_t ldc) {
    try {
        dispatch<float>(order, tA, tB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "blaze: %s\n", e.what());
        return 1;
    }
    return 0;
}

}  // extern "C"

// ---- the neighbouring BLAS routines on the same seam, evaluated by Blaze -----------------------
namespace {

template <typename T>
using VView = blaze::CustomVector<T, unaligned, unpadded>;

// y = alpha * op(A) * x + beta * y (unit strides); op(A) is the logical rows x cols view of the
// CBLAS operand, a CustomMatrix in the storage order (order, trans) describes.
template <typename T, bool SO>
void gemv_run(int64_t rows, int64_t cols, bool conj_a, T alpha, const T* A, int64_t lda, const T* x, T beta, T* y) {
    View<T, SO> a(const_cast<T*>(A), rows, cols, lda);
    VView<T> vx(const_cast<T*>(x), cols);
    VView<T> vy(y, rows);
    if (conj_a) {  // conjugate transpose: Blaze's conj() of the transposed view
        blaze::DynamicMatrix<T, SO> ca(conj(a));
        if (beta == T(0)) {
            vy = alpha * (ca * vx);
        } else {
            vy *= beta;
            vy += alpha * (ca * vx);
        }
        return;
    }
    if (beta == T(0)) {
        vy = alpha * (a * vx);
    } else {
        vy *= beta;
        vy += alpha * (a * vx);
    }
}

template <typename T>
void gemv_dispatch(int order, int tA, int64_t m, int64_t n, T alpha, const T* A, int64_t lda, const T* x, T beta,
                   T* y) {
    const bool rm = (order == 101), ta = (tA != 111), ca = (tA == 113);
    const int64_t rows = ta ? n : m, cols = ta ? m : n;
    const bool so = rm ? (ta ? columnMajor : rowMajor) : (ta ? rowMajor : columnMajor);
    if (so == rowMajor) gemv_run<T, rowMajor>(rows, cols, ca, alpha, A, lda, x, beta, y);
    else gemv_run<T, columnMajor>(rows, cols, ca, alpha, A, lda, x, beta, y);
}

// Complex C = alpha * op(A) * op(B) + beta * C; op = conj(trans(.)) for CblasConjTrans.
template <typename T, bool SOC, bool SOA, bool SOB>
void cgemm_run(int64_t m, int64_t n, int64_t k, bool ca, bool cb, std::complex<T> alpha, const std::complex<T>* A,
               int64_t lda, const std::complex<T>* B, int64_t ldb, std::complex<T> beta, std::complex<T>* C,
               int64_t ldc) {
    using CT = std::complex<T>;
    View<CT, SOA> a(const_cast<CT*>(A), m, k, lda);
    View<CT, SOB> b(const_cast<CT*>(B), k, n, ldb);
    View<CT, SOC> c(C, m, n, ldc);
    blaze::DynamicMatrix<CT, SOA> aa(a);
    blaze::DynamicMatrix<CT, SOB> bb(b);
    if (ca) aa = conj(aa);
    if (cb) bb = conj(bb);
    if (beta == CT(0)) {
        c = alpha * (aa * bb);
    } else {
        c *= beta;
        c += alpha * (aa * bb);
    }
}

template <typename T>
void cgemm_dispatch(int order, int tA, int tB, int64_t m, int64_t n, int64_t k, std::complex<T> alpha,
                    const std::complex<T>* A, int64_t lda, const std::complex<T>* B, int64_t ldb,
                    std::complex<T> beta, std::complex<T>* C, int64_t ldc) {
    const bool rm = (order == 101);
    const bool ta = (tA != 111), tb = (tB != 111), ca = (tA == 113), cb = (tB == 113);
    const bool soA = rm ? (ta ? columnMajor : rowMajor) : (ta ? rowMajor : columnMajor);
    const bool soB = rm ? (tb ? columnMajor : rowMajor) : (tb ? rowMajor : columnMajor);
#define GB_CASE(SC, SA, SB)                                                                        \
    if ((rm ? rowMajor : columnMajor) == SC && soA == SA && soB == SB) {                           \
        cgemm_run<T, SC, SA, SB>(m, n, k, ca, cb, alpha, A, lda, B, ldb, beta, C, ldc);            \
        return;                                                                                    \
    }
    GB_CASE(rowMajor, rowMajor, rowMajor)
    GB_CASE(rowMajor, rowMajor, columnMajor)
    GB_CASE(rowMajor, columnMajor, rowMajor)
    GB_CASE(rowMajor, columnMajor, columnMajor)
    GB_CASE(columnMajor, rowMajor, rowMajor)
    GB_CASE(columnMajor, rowMajor, columnMajor)
    GB_CASE(columnMajor, columnMajor, rowMajor)
    GB_CASE(columnMajor, columnMajor, columnMajor)
#undef GB_CASE
}

// op(T) for a triangular A (ka x ka view in storage order SO): only the uplo triangle is read,
// diag Unit takes ones on the diagonal; op = transpose (ta) and conjugate (ca).
template <typename T, bool SO>
blaze::DynamicMatrix<T, SO> triangle_op(const View<T, SO>& a, int64_t ka, int lower, int ta, int ca, int unit) {
    blaze::DynamicMatrix<T, SO> t(ka, ka, T(0));
    for (int64_t i = 0; i < ka; ++i)
        for (int64_t j = 0; j < ka; ++j) {
            const bool in = lower ? (j <= i) : (j >= i);
            if (in) t(i, j) = (unit && i == j) ? T(1) : a(i, j);
        }
    blaze::DynamicMatrix<T, SO> op = ta ? blaze::DynamicMatrix<T, SO>(trans(t)) : t;
    if (ca) op = conj(op);
    return op;
}

// Blaze's own evaluation of a product with a triangular op(T): op(T) held by blaze::LowerMatrix /
// UpperMatrix (the Uni* adaptors for a unit diagonal), multiplied by f with Blaze's default kernels.
template <typename T, bool SO, typename F>
void with_triangle(const blaze::DynamicMatrix<T, SO>& op, bool low_op, int unit, F&& f) {
    if (low_op) {
        if (unit) f(blaze::UniLowerMatrix<blaze::DynamicMatrix<T, SO>>(op));
        else f(blaze::LowerMatrix<blaze::DynamicMatrix<T, SO>>(op));
    } else {
        if (unit) f(blaze::UniUpperMatrix<blaze::DynamicMatrix<T, SO>>(op));
        else f(blaze::UpperMatrix<blaze::DynamicMatrix<T, SO>>(op));
    }
}

// B = alpha * op(A) * B (side Left) or alpha * B * op(A) (side Right), A triangular.
template <typename T, bool SO>
void trmm_run(int side_left, int lower, int ta, int ca, int unit, int64_t m, int64_t n, T alpha, const T* A,
              int64_t lda, T* B, int64_t ldb) {
    const int64_t ka = side_left ? m : n;
    View<T, SO> a(const_cast<T*>(A), ka, ka, lda);
    View<T, SO> b(B, m, n, ldb);
    const blaze::DynamicMatrix<T, SO> op = triangle_op<T, SO>(a, ka, lower, ta, ca, unit);
    blaze::DynamicMatrix<T, SO> res;
    with_triangle<T, SO>(op, ta ? !lower : lower, unit, [&](const auto& tri) {
        res = side_left ? blaze::DynamicMatrix<T, SO>(alpha * (tri * b)) : blaze::DynamicMatrix<T, SO>(alpha * (b * tri));
    });
    b = res;
}

// x = op(A) * x (unit stride), A n x n triangular.
template <typename T, bool SO>
void trmv_run(int lower, int ta, int ca, int unit, int64_t n, const T* A, int64_t lda, T* x) {
    View<T, SO> a(const_cast<T*>(A), n, n, lda);
    VView<T> vx(x, n);
    const blaze::DynamicMatrix<T, SO> op = triangle_op<T, SO>(a, n, lower, ta, ca, unit);
    blaze::DynamicVector<T> res;
    with_triangle<T, SO>(op, ta ? !lower : lower, unit, [&](const auto& tri) { res = tri * vx; });
    vx = res;
}

}  // namespace

extern "C" {

int ref_gemv_d(int order, int tA, int64_t m, int64_t n, double alpha, const double* A, int64_t lda, const double* x,
               double beta, double* y) {
    try {
        gemv_dispatch<double>(order, tA, m, n, alpha, A, lda, x, beta, y);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "blaze: %s\n", e.what());
        return 1;
    }
    return 0;
}

// alpha, beta, A, B, C as interleaved (re, im) doubles
int ref_gemm_z(int order, int tA, int tB, int64_t m, int64_t n, int64_t k, const double* alpha, const double* A,
               int64_t lda, const double* B, int64_t ldb, const double* beta, double* C, int64_t ldc) {
    using CT = std::complex<double>;
    try {
        cgemm_dispatch<double>(order, tA, tB, m, n, k, CT(alpha[0], alpha[1]), reinterpret_cast<const CT*>(A), lda,
                               reinterpret_cast<const CT*>(B), ldb, CT(beta[0], beta[1]), reinterpret_cast<CT*>(C), ldc);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "blaze: %s\n", e.what());
        return 1;
    }
    return 0;
}

int ref_trmm_d(int order, int side, int uplo, int tA, int diag, int64_t m, int64_t n, double alpha, const double* A,
               int64_t lda, double* B, int64_t ldb) {
    try {
        const int left = side == 141, lower = uplo == 122, ta = tA != 111, unit = diag == 132;
        if (order == 101) trmm_run<double, rowMajor>(left, lower, ta, 0, unit, m, n, alpha, A, lda, B, ldb);
        else trmm_run<double, columnMajor>(left, lower, ta, 0, unit, m, n, alpha, A, lda, B, ldb);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "blaze: %s\n", e.what());
        return 1;
    }
    return 0;
}

// complex y = alpha * op(A) * x + beta * y; alpha, beta, A, x, y interleaved (re, im)
int ref_gemv_z(int order, int tA, int64_t m, int64_t n, const double* alpha, const double* A, int64_t lda,
               const double* x, const double* beta, double* y) {
    using CT = std::complex<double>;
    try {
        gemv_dispatch<CT>(order, tA, m, n, CT(alpha[0], alpha[1]), reinterpret_cast<const CT*>(A), lda,
                          reinterpret_cast<const CT*>(x), CT(beta[0], beta[1]), reinterpret_cast<CT*>(y));
    } catch (const std::exception& e) {
        std::fprintf(stderr, "blaze: %s\n", e.what());
        return 1;
    }
    return 0;
}

// x = op(A) * x, A triangular; real (cplx == 0) or interleaved complex doubles
int ref_trmv(int cplx, int order, int uplo, int tA, int diag, int64_t n, const double* A, int64_t lda, double* x) {
    using CT = std::complex<double>;
    try {
        const int lower = uplo == 122, ta = tA != 111, ca = tA == 113, unit = diag == 132;
        if (cplx) {
            const CT* a = reinterpret_cast<const CT*>(A);
            CT* v = reinterpret_cast<CT*>(x);
            if (order == 101) trmv_run<CT, rowMajor>(lower, ta, ca, unit, n, a, lda, v);
            else trmv_run<CT, columnMajor>(lower, ta, ca, unit, n, a, lda, v);
        } else {
            if (order == 101) trmv_run<double, rowMajor>(lower, ta, 0, unit, n, A, lda, x);
            else trmv_run<double, columnMajor>(lower, ta, 0, unit, n, A, lda, x);
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "blaze: %s\n", e.what());
        return 1;
    }
    return 0;
}

// complex B = alpha * op(A) * B or alpha * B * op(A), A triangular; interleaved (re, im)
int ref_trmm_z(int order, int side, int uplo, int tA, int diag, int64_t m, int64_t n, const double* alpha,
               const double* A, int64_t lda, double* B, int64_t ldb) {
    using CT = std::complex<double>;
    try {
        const int left = side == 141, lower = uplo == 122, ta = tA != 111, ca = tA == 113, unit = diag == 132;
        const CT al(alpha[0], alpha[1]);
        const CT* a = reinterpret_cast<const CT*>(A);
        CT* b = reinterpret_cast<CT*>(B);
        if (order == 101) trmm_run<CT, rowMajor>(left, lower, ta, ca, unit, m, n, al, a, lda, b, ldb);
        else trmm_run<CT, columnMajor>(left, lower, ta, ca, unit, m, n, al, a, lda, b, ldb);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "blaze: %s\n", e.what());
        return 1;
    }
    return 0;
}

// Dot products as blazetest's BLAS operation test writes them (blazetest/mathtest/blas/
// OperationTest.h:139-140, 183-184): x * y for dotu, conj(x) * y for dotc, x a row vector;
// real (cplx == 0) or interleaved complex doubles; the result (re, im) goes to out.
int ref_dot(int cplx, int conj_x, int64_t n, const double* x, const double* y, double* out) {
    using CT = std::complex<double>;
    try {
        if (cplx) {
            blaze::CustomVector<CT, unaligned, unpadded, blaze::rowVector> vx(
                const_cast<CT*>(reinterpret_cast<const CT*>(x)), n);
            VView<CT> vy(const_cast<CT*>(reinterpret_cast<const CT*>(y)), n);
            const CT r = conj_x ? CT(conj(vx) * vy) : CT(vx * vy);
            out[0] = r.real();
            out[1] = r.imag();
        } else {
            blaze::CustomVector<double, unaligned, unpadded, blaze::rowVector> vx(const_cast<double*>(x), n);
            VView<double> vy(const_cast<double*>(y), n);
            out[0] = vx * vy;
            out[1] = 0.0;
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "blaze: %s\n", e.what());
        return 1;
    }
    return 0;
}

// y += alpha * x as blazetest's BLAS operation test checks axpy (OperationTest.h:231-232); real
// or interleaved complex doubles, alpha (re, im).
int ref_axpy(int cplx, int64_t n, const double* alpha, const double* x, double* y) {
    using CT = std::complex<double>;
    try {
        if (cplx) {
            VView<CT> vx(const_cast<CT*>(reinterpret_cast<const CT*>(x)), n);
            VView<CT> vy(reinterpret_cast<CT*>(y), n);
            vy += CT(alpha[0], alpha[1]) * vx;
        } else {
            VView<double> vx(const_cast<double*>(x), n);
            VView<double> vy(y, n);
            vy += alpha[0] * vx;
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "blaze: %s\n", e.what());
        return 1;
    }
    return 0;
}

}  // extern "C"
