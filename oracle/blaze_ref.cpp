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
