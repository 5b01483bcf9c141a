// cblas.cpp — the CBLAS symbols Blaze's BLAS mode links against (include/gb300_cblas.h).
//
// Compiled twice: once with 32-bit integers (the standard names) and once with
// -DGB300_BLAS_ILP64 (names with a _64 suffix), matching blaze/math/blas/Types.h:56-64.
//
// cblas_dgemm / cblas_sgemm run on the GPU (api.cpp), and so does every other function Blaze's
// wrappers name (the headers under blaze/math/blas/cblas/): cblas_?gemv, cblas_?trmv, cblas_cgemm /
// cblas_zgemm, cblas_?trmm, cblas_?trsm, cblas_?axpy and the dot products, real and complex
// (api_next.cpp).
#include <string>

#include "../../include/gb300_blas.h"
#include "../../include/gb300_cblas.h"
#include "gb300_internal.h"
#include "runtime.h"

namespace {
void not_supported(const char* name) {
    gb::set_error(GB300_ERR_NOT_SUPPORTED,
                  std::string(name) + ": not provided by libgb300blas");
}
}  // namespace

extern "C" {

void cblas_sgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                 gb300_blas_int n, gb300_blas_int k, float alpha, const float* A, gb300_blas_int lda, const float* B,
                 gb300_blas_int ldb, float beta, float* C, gb300_blas_int ldc) {
    gb::gemm_entry<float>(int(order), int(transA), int(transB), int64_t(m), int64_t(n), int64_t(k), alpha, A,
                          int64_t(lda), B, int64_t(ldb), beta, C, int64_t(ldc), nullptr, "cblas_sgemm");
}

void cblas_dgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                 gb300_blas_int n, gb300_blas_int k, double alpha, const double* A, gb300_blas_int lda,
                 const double* B, gb300_blas_int ldb, double beta, double* C, gb300_blas_int ldc) {
    gb::gemm_entry<double>(int(order), int(transA), int(transB), int64_t(m), int64_t(n), int64_t(k), alpha, A,
                           int64_t(lda), B, int64_t(ldb), beta, C, int64_t(ldc), nullptr, "cblas_dgemm");
}

// Aliases used by the throwing C++ wrappers of gb300_cblas.h (GB300_BLAS_THROW).
__attribute__((visibility("default"))) void gb300_cblas_sgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA,
    CBLAS_TRANSPOSE transB, gb300_blas_int m, gb300_blas_int n, gb300_blas_int k, float alpha, const float* A,
    gb300_blas_int lda, const float* B, gb300_blas_int ldb, float beta, float* C, gb300_blas_int ldc) {
    cblas_sgemm(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

__attribute__((visibility("default"))) void gb300_cblas_dgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA,
    CBLAS_TRANSPOSE transB, gb300_blas_int m, gb300_blas_int n, gb300_blas_int k, double alpha, const double* A,
    gb300_blas_int lda, const double* B, gb300_blas_int ldb, double beta, double* C, gb300_blas_int ldc) {
    cblas_dgemm(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

// Aliases of the routines below for the same throwing wrappers.
__attribute__((visibility("default"))) void gb300_cblas_sgemv_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA,
    gb300_blas_int m, gb300_blas_int n, float alpha, const float* A, gb300_blas_int lda, const float* x,
    gb300_blas_int incX, float beta, float* y, gb300_blas_int incY) {
    cblas_sgemv(order, transA, m, n, alpha, A, lda, x, incX, beta, y, incY);
}
__attribute__((visibility("default"))) void gb300_cblas_dgemv_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA,
    gb300_blas_int m, gb300_blas_int n, double alpha, const double* A, gb300_blas_int lda, const double* x,
    gb300_blas_int incX, double beta, double* y, gb300_blas_int incY) {
    cblas_dgemv(order, transA, m, n, alpha, A, lda, x, incX, beta, y, incY);
}
__attribute__((visibility("default"))) void gb300_cblas_cgemv_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA,
    gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda, const void* x,
    gb300_blas_int incX, const void* beta, void* y, gb300_blas_int incY) {
    cblas_cgemv(order, transA, m, n, alpha, A, lda, x, incX, beta, y, incY);
}
__attribute__((visibility("default"))) void gb300_cblas_zgemv_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA,
    gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda, const void* x,
    gb300_blas_int incX, const void* beta, void* y, gb300_blas_int incY) {
    cblas_zgemv(order, transA, m, n, alpha, A, lda, x, incX, beta, y, incY);
}
__attribute__((visibility("default"))) void gb300_cblas_cgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA,
    CBLAS_TRANSPOSE transB, gb300_blas_int m, gb300_blas_int n, gb300_blas_int k, const void* alpha, const void* A,
    gb300_blas_int lda, const void* B, gb300_blas_int ldb, const void* beta, void* C, gb300_blas_int ldc) {
    cblas_cgemm(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
__attribute__((visibility("default"))) void gb300_cblas_zgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA,
    CBLAS_TRANSPOSE transB, gb300_blas_int m, gb300_blas_int n, gb300_blas_int k, const void* alpha, const void* A,
    gb300_blas_int lda, const void* B, gb300_blas_int ldb, const void* beta, void* C, gb300_blas_int ldc) {
    cblas_zgemm(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
__attribute__((visibility("default"))) void gb300_cblas_strmm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO
    uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, float alpha, const float* A,
    gb300_blas_int lda, float* B, gb300_blas_int ldb) {
    cblas_strmm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
__attribute__((visibility("default"))) void gb300_cblas_dtrmm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO
    uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, double alpha, const double* A,
    gb300_blas_int lda, double* B, gb300_blas_int ldb) {
    cblas_dtrmm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
__attribute__((visibility("default"))) void gb300_cblas_ctrmm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO
    uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void*
    A, gb300_blas_int lda, void* B, gb300_blas_int ldb) {
    cblas_ctrmm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
__attribute__((visibility("default"))) void gb300_cblas_ztrmm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO
    uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void*
    A, gb300_blas_int lda, void* B, gb300_blas_int ldb) {
    cblas_ztrmm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
__attribute__((visibility("default"))) void gb300_cblas_strmv_checked(CBLAS_ORDER order, CBLAS_UPLO uplo,
    CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n, const float* A, gb300_blas_int lda, float* x,
    gb300_blas_int incX) {
    cblas_strmv(order, uplo, transA, diag, n, A, lda, x, incX);
}
__attribute__((visibility("default"))) void gb300_cblas_dtrmv_checked(CBLAS_ORDER order, CBLAS_UPLO uplo,
    CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n, const double* A, gb300_blas_int lda, double* x,
    gb300_blas_int incX) {
    cblas_dtrmv(order, uplo, transA, diag, n, A, lda, x, incX);
}
__attribute__((visibility("default"))) void gb300_cblas_ctrmv_checked(CBLAS_ORDER order, CBLAS_UPLO uplo,
    CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n, const void* A, gb300_blas_int lda, void* x,
    gb300_blas_int incX) {
    cblas_ctrmv(order, uplo, transA, diag, n, A, lda, x, incX);
}
__attribute__((visibility("default"))) void gb300_cblas_ztrmv_checked(CBLAS_ORDER order, CBLAS_UPLO uplo,
    CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n, const void* A, gb300_blas_int lda, void* x,
    gb300_blas_int incX) {
    cblas_ztrmv(order, uplo, transA, diag, n, A, lda, x, incX);
}

// Aliases of the level-1 routines and ?trsm for the same throwing wrappers.
__attribute__((visibility("default"))) void gb300_cblas_strsm_checked(CBLAS_ORDER order, CBLAS_SIDE side,
    CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, float alpha,
    const float* A, gb300_blas_int lda, float* B, gb300_blas_int ldb) {
    cblas_strsm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
__attribute__((visibility("default"))) void gb300_cblas_saxpy_checked(gb300_blas_int n, float alpha, const float* x,
    gb300_blas_int incX, float* y, gb300_blas_int incY) {
    cblas_saxpy(n, alpha, x, incX, y, incY);
}
__attribute__((visibility("default"))) void gb300_cblas_dtrsm_checked(CBLAS_ORDER order, CBLAS_SIDE side,
    CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, double alpha,
    const double* A, gb300_blas_int lda, double* B, gb300_blas_int ldb) {
    cblas_dtrsm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
__attribute__((visibility("default"))) void gb300_cblas_daxpy_checked(gb300_blas_int n, double alpha,
    const double* x, gb300_blas_int incX, double* y, gb300_blas_int incY) {
    cblas_daxpy(n, alpha, x, incX, y, incY);
}
__attribute__((visibility("default"))) void gb300_cblas_ctrsm_checked(CBLAS_ORDER order, CBLAS_SIDE side,
    CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha,
    const void* A, gb300_blas_int lda, void* B, gb300_blas_int ldb) {
    cblas_ctrsm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
__attribute__((visibility("default"))) void gb300_cblas_caxpy_checked(gb300_blas_int n, const void* alpha,
    const void* x, gb300_blas_int incX, void* y, gb300_blas_int incY) {
    cblas_caxpy(n, alpha, x, incX, y, incY);
}
__attribute__((visibility("default"))) void gb300_cblas_ztrsm_checked(CBLAS_ORDER order, CBLAS_SIDE side,
    CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha,
    const void* A, gb300_blas_int lda, void* B, gb300_blas_int ldb) {
    cblas_ztrsm(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
__attribute__((visibility("default"))) void gb300_cblas_zaxpy_checked(gb300_blas_int n, const void* alpha,
    const void* x, gb300_blas_int incX, void* y, gb300_blas_int incY) {
    cblas_zaxpy(n, alpha, x, incX, y, incY);
}
__attribute__((visibility("default"))) float gb300_cblas_sdot_checked(gb300_blas_int n, const float* x,
    gb300_blas_int incX, const float* y, gb300_blas_int incY) {
    return cblas_sdot(n, x, incX, y, incY);
}
__attribute__((visibility("default"))) double gb300_cblas_ddot_checked(gb300_blas_int n, const double* x,
    gb300_blas_int incX, const double* y, gb300_blas_int incY) {
    return cblas_ddot(n, x, incX, y, incY);
}
__attribute__((visibility("default"))) void gb300_cblas_cdotu_sub_checked(gb300_blas_int n, const void* x,
    gb300_blas_int incX, const void* y, gb300_blas_int incY, void* dotu) {
    cblas_cdotu_sub(n, x, incX, y, incY, dotu);
}
__attribute__((visibility("default"))) void gb300_cblas_cdotu_checked(gb300_blas_int n, const void* x,
    gb300_blas_int incX, const void* y, gb300_blas_int incY, void* dotu) {
    cblas_cdotu(n, x, incX, y, incY, dotu);
}
__attribute__((visibility("default"))) void gb300_cblas_cdotc_sub_checked(gb300_blas_int n, const void* x,
    gb300_blas_int incX, const void* y, gb300_blas_int incY, void* dotc) {
    cblas_cdotc_sub(n, x, incX, y, incY, dotc);
}
__attribute__((visibility("default"))) void gb300_cblas_cdotc_checked(gb300_blas_int n, const void* x,
    gb300_blas_int incX, const void* y, gb300_blas_int incY, void* dotc) {
    cblas_cdotc(n, x, incX, y, incY, dotc);
}
__attribute__((visibility("default"))) void gb300_cblas_zdotu_sub_checked(gb300_blas_int n, const void* x,
    gb300_blas_int incX, const void* y, gb300_blas_int incY, void* dotu) {
    cblas_zdotu_sub(n, x, incX, y, incY, dotu);
}
__attribute__((visibility("default"))) void gb300_cblas_zdotu_checked(gb300_blas_int n, const void* x,
    gb300_blas_int incX, const void* y, gb300_blas_int incY, void* dotu) {
    cblas_zdotu(n, x, incX, y, incY, dotu);
}
__attribute__((visibility("default"))) void gb300_cblas_zdotc_sub_checked(gb300_blas_int n, const void* x,
    gb300_blas_int incX, const void* y, gb300_blas_int incY, void* dotc) {
    cblas_zdotc_sub(n, x, incX, y, incY, dotc);
}
__attribute__((visibility("default"))) void gb300_cblas_zdotc_checked(gb300_blas_int n, const void* x,
    gb300_blas_int incX, const void* y, gb300_blas_int incY, void* dotc) {
    cblas_zdotc(n, x, incX, y, incY, dotc);
}

// ---- the neighbouring routines on the GPU (api_next.cpp) ----------------------------------------
void cblas_cgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                 gb300_blas_int n, gb300_blas_int k, const void* alpha, const void* A, gb300_blas_int lda, const void* B,
                 gb300_blas_int ldb, const void* beta, void* C, gb300_blas_int ldc) {
    gb::cgemm_entry<float>(int(order), int(transA), int(transB), int64_t(m), int64_t(n), int64_t(k),
                           static_cast<const float*>(alpha), static_cast<const float*>(A), int64_t(lda),
                           static_cast<const float*>(B), int64_t(ldb), static_cast<const float*>(beta),
                           static_cast<float*>(C), int64_t(ldc), "cblas_cgemm");
}
void cblas_zgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                 gb300_blas_int n, gb300_blas_int k, const void* alpha, const void* A, gb300_blas_int lda, const void* B,
                 gb300_blas_int ldb, const void* beta, void* C, gb300_blas_int ldc) {
    gb::cgemm_entry<double>(int(order), int(transA), int(transB), int64_t(m), int64_t(n), int64_t(k),
                            static_cast<const double*>(alpha), static_cast<const double*>(A), int64_t(lda),
                            static_cast<const double*>(B), int64_t(ldb), static_cast<const double*>(beta),
                            static_cast<double*>(C), int64_t(ldc), "cblas_zgemm");
}
void cblas_sgemv(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n, float alpha,
                 const float* A, gb300_blas_int lda, const float* x, gb300_blas_int incx, float beta, float* y,
                 gb300_blas_int incy) {
    gb::gemv_entry<float>(int(order), int(transA), int64_t(m), int64_t(n), alpha, A, int64_t(lda), x, int64_t(incx),
                          beta, y, int64_t(incy), "cblas_sgemv");
}
void cblas_dgemv(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n, double alpha,
                 const double* A, gb300_blas_int lda, const double* x, gb300_blas_int incx, double beta, double* y,
                 gb300_blas_int incy) {
    gb::gemv_entry<double>(int(order), int(transA), int64_t(m), int64_t(n), alpha, A, int64_t(lda), x, int64_t(incx),
                           beta, y, int64_t(incy), "cblas_dgemv");
}
void cblas_cgemv(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n, const void* alpha,
                 const void* A, gb300_blas_int lda, const void* x, gb300_blas_int incx, const void* beta, void* y,
                 gb300_blas_int incy) {
    gb::cgemv_entry<float>(int(order), int(transA), int64_t(m), int64_t(n), static_cast<const float*>(alpha),
                           static_cast<const float*>(A), int64_t(lda), static_cast<const float*>(x), int64_t(incx),
                           static_cast<const float*>(beta), static_cast<float*>(y), int64_t(incy), "cblas_cgemv");
}
void cblas_zgemv(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n, const void* alpha,
                 const void* A, gb300_blas_int lda, const void* x, gb300_blas_int incx, const void* beta, void* y,
                 gb300_blas_int incy) {
    gb::cgemv_entry<double>(int(order), int(transA), int64_t(m), int64_t(n), static_cast<const double*>(alpha),
                            static_cast<const double*>(A), int64_t(lda), static_cast<const double*>(x), int64_t(incx),
                            static_cast<const double*>(beta), static_cast<double*>(y), int64_t(incy), "cblas_zgemv");
}
void cblas_strmm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                 gb300_blas_int m, gb300_blas_int n, float alpha, const float* A, gb300_blas_int lda, float* B,
                 gb300_blas_int ldb) {
    gb::trmm_entry<float>(int(order), int(side), int(uplo), int(transA), int(diag), int64_t(m), int64_t(n), alpha, A,
                          int64_t(lda), B, int64_t(ldb), "cblas_strmm");
}
void cblas_dtrmm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                 gb300_blas_int m, gb300_blas_int n, double alpha, const double* A, gb300_blas_int lda, double* B,
                 gb300_blas_int ldb) {
    gb::trmm_entry<double>(int(order), int(side), int(uplo), int(transA), int(diag), int64_t(m), int64_t(n), alpha, A,
                           int64_t(lda), B, int64_t(ldb), "cblas_dtrmm");
}
void cblas_ctrmm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                 gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda, void* B,
                 gb300_blas_int ldb) {
    gb::ctrmm_entry<float>(int(order), int(side), int(uplo), int(transA), int(diag), int64_t(m), int64_t(n),
                           static_cast<const float*>(alpha), static_cast<const float*>(A), int64_t(lda),
                           static_cast<float*>(B), int64_t(ldb), "cblas_ctrmm");
}
void cblas_ztrmm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                 gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda, void* B,
                 gb300_blas_int ldb) {
    gb::ctrmm_entry<double>(int(order), int(side), int(uplo), int(transA), int(diag), int64_t(m), int64_t(n),
                            static_cast<const double*>(alpha), static_cast<const double*>(A), int64_t(lda),
                            static_cast<double*>(B), int64_t(ldb), "cblas_ztrmm");
}
void cblas_strmv(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n,
                 const float* A, gb300_blas_int lda, float* x, gb300_blas_int incx) {
    gb::trmv_entry<float, false>(int(order), int(uplo), int(transA), int(diag), int64_t(n), A, int64_t(lda), x,
                                 int64_t(incx), "cblas_strmv");
}
void cblas_dtrmv(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n,
                 const double* A, gb300_blas_int lda, double* x, gb300_blas_int incx) {
    gb::trmv_entry<double, false>(int(order), int(uplo), int(transA), int(diag), int64_t(n), A, int64_t(lda), x,
                                  int64_t(incx), "cblas_dtrmv");
}
void cblas_ctrmv(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n,
                 const void* A, gb300_blas_int lda, void* x, gb300_blas_int incx) {
    gb::trmv_entry<float, true>(int(order), int(uplo), int(transA), int(diag), int64_t(n),
                                static_cast<const float*>(A), int64_t(lda), static_cast<float*>(x), int64_t(incx),
                                "cblas_ctrmv");
}
void cblas_ztrmv(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n,
                 const void* A, gb300_blas_int lda, void* x, gb300_blas_int incx) {
    gb::trmv_entry<double, true>(int(order), int(uplo), int(transA), int(diag), int64_t(n),
                                 static_cast<const double*>(A), int64_t(lda), static_cast<double*>(x), int64_t(incx),
                                 "cblas_ztrmv");
}
void cblas_strsm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
    gb300_blas_int m, gb300_blas_int n, float alpha, const float* A, gb300_blas_int lda, float* B,
    gb300_blas_int ldb) {
    gb::trsm_entry<float, false>(int(order), int(side), int(uplo), int(transA), int(diag), int64_t(m), int64_t(n),
        &alpha, A, int64_t(lda), B, int64_t(ldb), "cblas_strsm");
}
void cblas_saxpy(gb300_blas_int n, float alpha, const float* x, gb300_blas_int incX, float* y, gb300_blas_int incY) {
    gb::axpy_entry<float, false>(int64_t(n), &alpha, x, int64_t(incX), y, int64_t(incY), "cblas_saxpy");
}
void cblas_dtrsm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
    gb300_blas_int m, gb300_blas_int n, double alpha, const double* A, gb300_blas_int lda, double* B,
    gb300_blas_int ldb) {
    gb::trsm_entry<double, false>(int(order), int(side), int(uplo), int(transA), int(diag), int64_t(m), int64_t(n),
        &alpha, A, int64_t(lda), B, int64_t(ldb), "cblas_dtrsm");
}
void cblas_daxpy(gb300_blas_int n, double alpha, const double* x, gb300_blas_int incX, double* y,
    gb300_blas_int incY) {
    gb::axpy_entry<double, false>(int64_t(n), &alpha, x, int64_t(incX), y, int64_t(incY), "cblas_daxpy");
}
void cblas_ctrsm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
    gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda, void* B,
    gb300_blas_int ldb) {
    gb::trsm_entry<float, true>(int(order), int(side), int(uplo), int(transA), int(diag), int64_t(m), int64_t(n),
        static_cast<const float*>(alpha), static_cast<const float*>(A), int64_t(lda), static_cast<float*>(B),
        int64_t(ldb), "cblas_ctrsm");
}
void cblas_caxpy(gb300_blas_int n, const void* alpha, const void* x, gb300_blas_int incX, void* y,
    gb300_blas_int incY) {
    gb::axpy_entry<float, true>(int64_t(n), static_cast<const float*>(alpha), static_cast<const float*>(x),
        int64_t(incX), static_cast<float*>(y), int64_t(incY), "cblas_caxpy");
}
void cblas_ztrsm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
    gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda, void* B,
    gb300_blas_int ldb) {
    gb::trsm_entry<double, true>(int(order), int(side), int(uplo), int(transA), int(diag), int64_t(m), int64_t(n),
        static_cast<const double*>(alpha), static_cast<const double*>(A), int64_t(lda), static_cast<double*>(B),
        int64_t(ldb), "cblas_ztrsm");
}
void cblas_zaxpy(gb300_blas_int n, const void* alpha, const void* x, gb300_blas_int incX, void* y,
    gb300_blas_int incY) {
    gb::axpy_entry<double, true>(int64_t(n), static_cast<const double*>(alpha), static_cast<const double*>(x),
        int64_t(incX), static_cast<double*>(y), int64_t(incY), "cblas_zaxpy");
}
float cblas_sdot(gb300_blas_int n, const float* x, gb300_blas_int incX, const float* y, gb300_blas_int incY) {
    float r = 0.f;
    gb::dot_entry<float, false, false>(int64_t(n), x, int64_t(incX), y, int64_t(incY), &r, "cblas_sdot");
    return r;
}
double cblas_ddot(gb300_blas_int n, const double* x, gb300_blas_int incX, const double* y, gb300_blas_int incY) {
    double r = 0.0;
    gb::dot_entry<double, false, false>(int64_t(n), x, int64_t(incX), y, int64_t(incY), &r, "cblas_ddot");
    return r;
}
void cblas_cdotu_sub(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y, gb300_blas_int incY,
    void* dotu) {
    gb::dot_entry<float, true, false>(int64_t(n), static_cast<const float*>(x), int64_t(incX),
        static_cast<const float*>(y), int64_t(incY), static_cast<float*>(dotu), "cblas_cdotu_sub");
}
void cblas_cdotu(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y, gb300_blas_int incY,
    void* dotu) {
    gb::dot_entry<float, true, false>(int64_t(n), static_cast<const float*>(x), int64_t(incX),
        static_cast<const float*>(y), int64_t(incY), static_cast<float*>(dotu), "cblas_cdotu");
}
void cblas_cdotc_sub(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y, gb300_blas_int incY,
    void* dotc) {
    gb::dot_entry<float, true, true>(int64_t(n), static_cast<const float*>(x), int64_t(incX),
        static_cast<const float*>(y), int64_t(incY), static_cast<float*>(dotc), "cblas_cdotc_sub");
}
void cblas_cdotc(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y, gb300_blas_int incY,
    void* dotc) {
    gb::dot_entry<float, true, true>(int64_t(n), static_cast<const float*>(x), int64_t(incX),
        static_cast<const float*>(y), int64_t(incY), static_cast<float*>(dotc), "cblas_cdotc");
}
void cblas_zdotu_sub(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y, gb300_blas_int incY,
    void* dotu) {
    gb::dot_entry<double, true, false>(int64_t(n), static_cast<const double*>(x), int64_t(incX),
        static_cast<const double*>(y), int64_t(incY), static_cast<double*>(dotu), "cblas_zdotu_sub");
}
void cblas_zdotu(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y, gb300_blas_int incY,
    void* dotu) {
    gb::dot_entry<double, true, false>(int64_t(n), static_cast<const double*>(x), int64_t(incX),
        static_cast<const double*>(y), int64_t(incY), static_cast<double*>(dotu), "cblas_zdotu");
}
void cblas_zdotc_sub(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y, gb300_blas_int incY,
    void* dotc) {
    gb::dot_entry<double, true, true>(int64_t(n), static_cast<const double*>(x), int64_t(incX),
        static_cast<const double*>(y), int64_t(incY), static_cast<double*>(dotc), "cblas_zdotc_sub");
}
void cblas_zdotc(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y, gb300_blas_int incY,
    void* dotc) {
    gb::dot_entry<double, true, true>(int64_t(n), static_cast<const double*>(x), int64_t(incX),
        static_cast<const double*>(y), int64_t(incY), static_cast<double*>(dotc), "cblas_zdotc");
}

}  // extern "C"
