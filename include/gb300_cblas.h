/*
 * gb300_cblas.h — drop-in CBLAS header for Blaze's BLAS mode, backed by GB300 (sm_103a) kernels.
 *
 * Use with Blaze:
 *     g++ ... -DBLAZE_BLAS_MODE=1 -DBLAZE_BLAS_IS_PARALLEL=1 \
 *             -DBLAZE_BLAS_INCLUDE_FILE="<gb300_cblas.h>" -I<this dir> ... -lgb300blas
 * Blaze includes this file inside `extern "C" { ... }` (blaze/system/BLAS.h:57-58) and its inline
 * wrappers in blaze/math/blas/cblas/ headers call the cblas_* functions declared here.
 *
 * Implemented on the GPU: cblas_dgemm and cblas_sgemm (the dense matrix-multiplication path,
 * reached from blaze::gemm(), blaze/math/blas/gemm.h:105-131, and blaze/math/blas/cblas/gemm.h:
 * 116-162), the other routines Blaze's expressions call (cblas_?gemv, cblas_?trmv, cblas_cgemm /
 * cblas_zgemm, cblas_?trmm), and the rest of what Blaze's wrappers name: cblas_?trsm (blaze::trsm),
 * cblas_?axpy (blaze::axpy) and the dot products (blaze::dotu, blaze::dotc).  There is no CPU
 * fallback.
 *
 * Integer type: `blas_int_t` is int32 unless BLAZE_BLAS_IS_64BIT is set, matching
 * blaze/math/blas/Types.h:56-64.  The library exports the 32-bit ABI under the standard names;
 * the 64-bit (ILP64) variants are exported as cblas_*_64 and selected here when
 * BLAZE_BLAS_IS_64BIT (or GB300_BLAS_ILP64) is defined.
 *
 * Errors: CBLAS routines return void.  Invalid arguments and device failures are recorded in a
 * thread-local status readable with gb300_last_error() / gb300_last_error_message().
 * Defining GB300_BLAS_THROW before inclusion in C++ wraps every routine the library implements so
 * that a non-zero status throws std::runtime_error right after the call (the behaviour of Blaze's
 * own BLAZE_THROW_RUNTIME_ERROR, blaze/util/Exception.h).
 */
#ifndef GB300_CBLAS_H
#define GB300_CBLAS_H

#include <stdint.h>

/* Standard CBLAS enumerations (values are the CBLAS ABI). */
#ifndef CBLAS_ENUM_DEFINED_H
#define CBLAS_ENUM_DEFINED_H
typedef enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_ORDER;
typedef enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;
typedef CBLAS_ORDER CBLAS_LAYOUT;
#endif

#if defined(BLAZE_BLAS_IS_64BIT) && BLAZE_BLAS_IS_64BIT
#define GB300_BLAS_ILP64 1
#endif

#ifdef GB300_BLAS_ILP64
typedef int64_t gb300_blas_int;
#define GB300_CBLAS_NAME(x) x##_64
#else
typedef int32_t gb300_blas_int;
#define GB300_CBLAS_NAME(x) x
#endif

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ---- status of the calling thread's last call --------------------------------------------- */
int gb300_last_error(void);
const char* gb300_last_error_message(void);
void gb300_clear_error(void);

#if defined(GB300_BLAS_ILP64)
#define cblas_sgemm cblas_sgemm_64
#define cblas_dgemm cblas_dgemm_64
#define cblas_cgemm cblas_cgemm_64
#define cblas_zgemm cblas_zgemm_64
#define cblas_sgemv cblas_sgemv_64
#define cblas_dgemv cblas_dgemv_64
#define cblas_cgemv cblas_cgemv_64
#define cblas_zgemv cblas_zgemv_64
#define cblas_strmm cblas_strmm_64
#define cblas_dtrmm cblas_dtrmm_64
#define cblas_ctrmm cblas_ctrmm_64
#define cblas_ztrmm cblas_ztrmm_64
#define cblas_strmv cblas_strmv_64
#define cblas_dtrmv cblas_dtrmv_64
#define cblas_ctrmv cblas_ctrmv_64
#define cblas_ztrmv cblas_ztrmv_64
#define cblas_strsm cblas_strsm_64
#define cblas_dtrsm cblas_dtrsm_64
#define cblas_ctrsm cblas_ctrsm_64
#define cblas_ztrsm cblas_ztrsm_64
#define cblas_saxpy cblas_saxpy_64
#define cblas_daxpy cblas_daxpy_64
#define cblas_caxpy cblas_caxpy_64
#define cblas_zaxpy cblas_zaxpy_64
#define cblas_sdot cblas_sdot_64
#define cblas_ddot cblas_ddot_64
#define cblas_cdotu cblas_cdotu_64
#define cblas_zdotu cblas_zdotu_64
#define cblas_cdotc cblas_cdotc_64
#define cblas_zdotc cblas_zdotc_64
#define cblas_cdotu_sub cblas_cdotu_sub_64
#define cblas_zdotu_sub cblas_zdotu_sub_64
#define cblas_cdotc_sub cblas_cdotc_sub_64
#define cblas_zdotc_sub cblas_zdotc_sub_64
#define gb300_cblas_sgemm_checked gb300_cblas_sgemm_checked_64
#define gb300_cblas_dgemm_checked gb300_cblas_dgemm_checked_64
#define gb300_cblas_sgemv_checked gb300_cblas_sgemv_checked_64
#define gb300_cblas_dgemv_checked gb300_cblas_dgemv_checked_64
#define gb300_cblas_cgemv_checked gb300_cblas_cgemv_checked_64
#define gb300_cblas_zgemv_checked gb300_cblas_zgemv_checked_64
#define gb300_cblas_cgemm_checked gb300_cblas_cgemm_checked_64
#define gb300_cblas_zgemm_checked gb300_cblas_zgemm_checked_64
#define gb300_cblas_strmm_checked gb300_cblas_strmm_checked_64
#define gb300_cblas_dtrmm_checked gb300_cblas_dtrmm_checked_64
#define gb300_cblas_ctrmm_checked gb300_cblas_ctrmm_checked_64
#define gb300_cblas_ztrmm_checked gb300_cblas_ztrmm_checked_64
#define gb300_cblas_strmv_checked gb300_cblas_strmv_checked_64
#define gb300_cblas_dtrmv_checked gb300_cblas_dtrmv_checked_64
#define gb300_cblas_ctrmv_checked gb300_cblas_ctrmv_checked_64
#define gb300_cblas_ztrmv_checked gb300_cblas_ztrmv_checked_64
#define gb300_cblas_strsm_checked gb300_cblas_strsm_checked_64
#define gb300_cblas_saxpy_checked gb300_cblas_saxpy_checked_64
#define gb300_cblas_dtrsm_checked gb300_cblas_dtrsm_checked_64
#define gb300_cblas_daxpy_checked gb300_cblas_daxpy_checked_64
#define gb300_cblas_ctrsm_checked gb300_cblas_ctrsm_checked_64
#define gb300_cblas_caxpy_checked gb300_cblas_caxpy_checked_64
#define gb300_cblas_ztrsm_checked gb300_cblas_ztrsm_checked_64
#define gb300_cblas_zaxpy_checked gb300_cblas_zaxpy_checked_64
#define gb300_cblas_sdot_checked gb300_cblas_sdot_checked_64
#define gb300_cblas_ddot_checked gb300_cblas_ddot_checked_64
#define gb300_cblas_cdotu_sub_checked gb300_cblas_cdotu_sub_checked_64
#define gb300_cblas_cdotu_checked gb300_cblas_cdotu_checked_64
#define gb300_cblas_cdotc_sub_checked gb300_cblas_cdotc_sub_checked_64
#define gb300_cblas_cdotc_checked gb300_cblas_cdotc_checked_64
#define gb300_cblas_zdotu_sub_checked gb300_cblas_zdotu_sub_checked_64
#define gb300_cblas_zdotu_checked gb300_cblas_zdotu_checked_64
#define gb300_cblas_zdotc_sub_checked gb300_cblas_zdotc_sub_checked_64
#define gb300_cblas_zdotc_checked gb300_cblas_zdotc_checked_64
#endif

/* Under GB300_BLAS_THROW (C++), each routine that runs on the GPU is declared as
 * gb300_<routine>_checked and <routine> becomes an inline wrapper that throws on a non-zero
 * status (end of this file). */
#if defined(__cplusplus) && defined(GB300_BLAS_THROW)
#define GB300_ENTRY(name) gb300_##name##_checked
#else
#define GB300_ENTRY(name) name
#endif

/* ---- GEMM: implemented on the GPU ---------------------------------------------------------- */
/* C = alpha*op(A)*op(B) + beta*C.  Replaces the cblas_sgemm call of
 * blaze/math/blas/cblas/gemm.h:121 (float). */
#if defined(__cplusplus) && defined(GB300_BLAS_THROW)
void gb300_cblas_sgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB,
#else
void cblas_sgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB,
#endif
                 gb300_blas_int m, gb300_blas_int n, gb300_blas_int k, float alpha, const float* A,
                 gb300_blas_int lda, const float* B, gb300_blas_int ldb, float beta, float* C,
                 gb300_blas_int ldc);

/* C = alpha*op(A)*op(B) + beta*C.  Replaces the cblas_dgemm call of
 * blaze/math/blas/cblas/gemm.h:161 (double). */
#if defined(__cplusplus) && defined(GB300_BLAS_THROW)
void gb300_cblas_dgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB,
#else
void cblas_dgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB,
#endif
                 gb300_blas_int m, gb300_blas_int n, gb300_blas_int k, double alpha, const double* A,
                 gb300_blas_int lda, const double* B, gb300_blas_int ldb, double beta, double* C,
                 gb300_blas_int ldc);

/* ---- Blaze's other wrappers, all on the GPU: ?gemv, ?trmv, complex ?gemm, ?trmm, ?trsm, ?axpy
 * and the dot products, real and complex (complex operands are interleaved (re, im) pairs, alpha /
 * beta point at one pair). */
/* blaze/math/blas/cblas/gemm.h:201,243 */
void GB300_ENTRY(cblas_cgemm)(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                 gb300_blas_int n, gb300_blas_int k, const void* alpha, const void* A, gb300_blas_int lda,
                 const void* B, gb300_blas_int ldb, const void* beta, void* C, gb300_blas_int ldc);
void GB300_ENTRY(cblas_zgemm)(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                 gb300_blas_int n, gb300_blas_int k, const void* alpha, const void* A, gb300_blas_int lda,
                 const void* B, gb300_blas_int ldb, const void* beta, void* C, gb300_blas_int ldc);
/* blaze/math/blas/cblas/gemv.h:116,153,193,235 */
void GB300_ENTRY(cblas_sgemv)(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n, float alpha,
                 const float* A, gb300_blas_int lda, const float* x, gb300_blas_int incX, float beta, float* y,
                 gb300_blas_int incY);
void GB300_ENTRY(cblas_dgemv)(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n, double alpha,
                 const double* A, gb300_blas_int lda, const double* x, gb300_blas_int incX, double beta,
                 double* y, gb300_blas_int incY);
void GB300_ENTRY(cblas_cgemv)(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n,
                 const void* alpha, const void* A, gb300_blas_int lda, const void* x, gb300_blas_int incX,
                 const void* beta, void* y, gb300_blas_int incY);
void GB300_ENTRY(cblas_zgemv)(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n,
                 const void* alpha, const void* A, gb300_blas_int lda, const void* x, gb300_blas_int incX,
                 const void* beta, void* y, gb300_blas_int incY);
/* blaze/math/blas/cblas/trmm.h:116,153,... */
void GB300_ENTRY(cblas_strmm)(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                 gb300_blas_int m, gb300_blas_int n, float alpha, const float* A, gb300_blas_int lda, float* B,
                 gb300_blas_int ldb);
void GB300_ENTRY(cblas_dtrmm)(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                 gb300_blas_int m, gb300_blas_int n, double alpha, const double* A, gb300_blas_int lda,
                 double* B, gb300_blas_int ldb);
void GB300_ENTRY(cblas_ctrmm)(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                 gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda,
                 void* B, gb300_blas_int ldb);
void GB300_ENTRY(cblas_ztrmm)(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                 gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda,
                 void* B, gb300_blas_int ldb);
/* blaze/math/blas/cblas/trmv.h:111,145,181,218 */
void GB300_ENTRY(cblas_strmv)(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n,
                 const float* A, gb300_blas_int lda, float* x, gb300_blas_int incX);
void GB300_ENTRY(cblas_dtrmv)(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n,
                 const double* A, gb300_blas_int lda, double* x, gb300_blas_int incX);
void GB300_ENTRY(cblas_ctrmv)(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n,
                 const void* A, gb300_blas_int lda, void* x, gb300_blas_int incX);
void GB300_ENTRY(cblas_ztrmv)(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag, gb300_blas_int n,
                 const void* A, gb300_blas_int lda, void* x, gb300_blas_int incX);
/* blaze/math/blas/cblas/trsm.h:115,153,193,234 */
void GB300_ENTRY(cblas_strsm)(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
    CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, float alpha, const float* A, gb300_blas_int lda, float* B,
    gb300_blas_int ldb);
/* blaze/math/blas/cblas/axpy.h:103,133,165,198 */
void GB300_ENTRY(cblas_saxpy)(gb300_blas_int n, float alpha, const float* x, gb300_blas_int incX, float* y,
    gb300_blas_int incY);
void GB300_ENTRY(cblas_dtrsm)(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
    CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, double alpha, const double* A, gb300_blas_int lda,
    double* B, gb300_blas_int ldb);
void GB300_ENTRY(cblas_daxpy)(gb300_blas_int n, double alpha, const double* x, gb300_blas_int incX, double* y,
    gb300_blas_int incY);
void GB300_ENTRY(cblas_ctrsm)(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
    CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda,
    void* B, gb300_blas_int ldb);
void GB300_ENTRY(cblas_caxpy)(gb300_blas_int n, const void* alpha, const void* x, gb300_blas_int incX, void* y,
    gb300_blas_int incY);
void GB300_ENTRY(cblas_ztrsm)(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
    CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda,
    void* B, gb300_blas_int ldb);
void GB300_ENTRY(cblas_zaxpy)(gb300_blas_int n, const void* alpha, const void* x, gb300_blas_int incX, void* y,
    gb300_blas_int incY);
/* blaze/math/blas/cblas/dotu.h:99,127 and dotc.h:99,127 */
float GB300_ENTRY(cblas_sdot)(gb300_blas_int n, const float* x, gb300_blas_int incX, const float* y,
    gb300_blas_int incY);
double GB300_ENTRY(cblas_ddot)(gb300_blas_int n, const double* x, gb300_blas_int incX, const double* y,
    gb300_blas_int incY);
/* Both forms of the complex dot products: dotu.h / dotc.h reference each under its own branch
 * (the _sub form unless OPENBLAS_VERSION).  The value-returning forms exist in some CBLAS flavours;
 * the library exports them with the result written through the trailing pointer. */
void GB300_ENTRY(cblas_cdotu_sub)(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotu);
void GB300_ENTRY(cblas_cdotu)(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotu);
void GB300_ENTRY(cblas_cdotc_sub)(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotc);
void GB300_ENTRY(cblas_cdotc)(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotc);
void GB300_ENTRY(cblas_zdotu_sub)(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotu);
void GB300_ENTRY(cblas_zdotu)(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotu);
void GB300_ENTRY(cblas_zdotc_sub)(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotc);
void GB300_ENTRY(cblas_zdotc)(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotc);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
} /* extern "C" */
#endif

/* ---- optional throwing wrappers for C++ callers (Blaze) ------------------------------------- */
#if defined(__cplusplus) && defined(GB300_BLAS_THROW)
extern "C++" {
#include <stdexcept>
#include <string>
inline void gb300_throw_if_error(const char* routine) {
    const int st = gb300_last_error();
    if (st != 0) {
        std::string msg = std::string(routine) + ": " + gb300_last_error_message();
        gb300_clear_error();
        throw std::runtime_error(msg);
    }
}
}
extern "C" {
static inline void cblas_sgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB,
                               gb300_blas_int m, gb300_blas_int n, gb300_blas_int k, float alpha,
                               const float* A, gb300_blas_int lda, const float* B, gb300_blas_int ldb,
                               float beta, float* C, gb300_blas_int ldc) {
    gb300_cblas_sgemm_checked(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    gb300_throw_if_error("cblas_sgemm");
}
static inline void cblas_dgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB,
                               gb300_blas_int m, gb300_blas_int n, gb300_blas_int k, double alpha,
                               const double* A, gb300_blas_int lda, const double* B, gb300_blas_int ldb,
                               double beta, double* C, gb300_blas_int ldc) {
    gb300_cblas_dgemm_checked(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    gb300_throw_if_error("cblas_dgemm");
}
static inline void cblas_sgemv(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n, float
                              alpha, const float* A, gb300_blas_int lda, const float* x, gb300_blas_int incX, float
                              beta, float* y, gb300_blas_int incY) {
    gb300_cblas_sgemv_checked(order, transA, m, n, alpha, A, lda, x, incX, beta, y, incY);
    gb300_throw_if_error("cblas_sgemv");
}
static inline void cblas_dgemv(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n, double
                              alpha, const double* A, gb300_blas_int lda, const double* x, gb300_blas_int incX, double
                              beta, double* y, gb300_blas_int incY) {
    gb300_cblas_dgemv_checked(order, transA, m, n, alpha, A, lda, x, incX, beta, y, incY);
    gb300_throw_if_error("cblas_dgemv");
}
static inline void cblas_cgemv(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n, const
                              void* alpha, const void* A, gb300_blas_int lda, const void* x, gb300_blas_int incX,
                              const void* beta, void* y, gb300_blas_int incY) {
    gb300_cblas_cgemv_checked(order, transA, m, n, alpha, A, lda, x, incX, beta, y, incY);
    gb300_throw_if_error("cblas_cgemv");
}
static inline void cblas_zgemv(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n, const
                              void* alpha, const void* A, gb300_blas_int lda, const void* x, gb300_blas_int incX,
                              const void* beta, void* y, gb300_blas_int incY) {
    gb300_cblas_zgemv_checked(order, transA, m, n, alpha, A, lda, x, incX, beta, y, incY);
    gb300_throw_if_error("cblas_zgemv");
}
static inline void cblas_cgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                              gb300_blas_int n, gb300_blas_int k, const void* alpha, const void* A, gb300_blas_int
                              lda, const void* B, gb300_blas_int ldb, const void* beta, void* C, gb300_blas_int ldc) {
    gb300_cblas_cgemm_checked(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    gb300_throw_if_error("cblas_cgemm");
}
static inline void cblas_zgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                              gb300_blas_int n, gb300_blas_int k, const void* alpha, const void* A, gb300_blas_int
                              lda, const void* B, gb300_blas_int ldb, const void* beta, void* C, gb300_blas_int ldc) {
    gb300_cblas_zgemm_checked(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    gb300_throw_if_error("cblas_zgemm");
}
static inline void cblas_strmm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG
                              diag, gb300_blas_int m, gb300_blas_int n, float alpha, const float* A, gb300_blas_int
                              lda, float* B, gb300_blas_int ldb) {
    gb300_cblas_strmm_checked(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
    gb300_throw_if_error("cblas_strmm");
}
static inline void cblas_dtrmm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG
                              diag, gb300_blas_int m, gb300_blas_int n, double alpha, const double* A, gb300_blas_int
                              lda, double* B, gb300_blas_int ldb) {
    gb300_cblas_dtrmm_checked(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
    gb300_throw_if_error("cblas_dtrmm");
}
static inline void cblas_ctrmm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG
                              diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A,
                              gb300_blas_int lda, void* B, gb300_blas_int ldb) {
    gb300_cblas_ctrmm_checked(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
    gb300_throw_if_error("cblas_ctrmm");
}
static inline void cblas_ztrmm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG
                              diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A,
                              gb300_blas_int lda, void* B, gb300_blas_int ldb) {
    gb300_cblas_ztrmm_checked(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
    gb300_throw_if_error("cblas_ztrmm");
}
static inline void cblas_strmv(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                              gb300_blas_int n, const float* A, gb300_blas_int lda, float* x, gb300_blas_int incX) {
    gb300_cblas_strmv_checked(order, uplo, transA, diag, n, A, lda, x, incX);
    gb300_throw_if_error("cblas_strmv");
}
static inline void cblas_dtrmv(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                              gb300_blas_int n, const double* A, gb300_blas_int lda, double* x, gb300_blas_int incX) {
    gb300_cblas_dtrmv_checked(order, uplo, transA, diag, n, A, lda, x, incX);
    gb300_throw_if_error("cblas_dtrmv");
}
static inline void cblas_ctrmv(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                              gb300_blas_int n, const void* A, gb300_blas_int lda, void* x, gb300_blas_int incX) {
    gb300_cblas_ctrmv_checked(order, uplo, transA, diag, n, A, lda, x, incX);
    gb300_throw_if_error("cblas_ctrmv");
}
static inline void cblas_ztrmv(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                              gb300_blas_int n, const void* A, gb300_blas_int lda, void* x, gb300_blas_int incX) {
    gb300_cblas_ztrmv_checked(order, uplo, transA, diag, n, A, lda, x, incX);
    gb300_throw_if_error("cblas_ztrmv");
}
static inline void cblas_strsm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
    CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, float alpha, const float* A, gb300_blas_int lda, float* B,
    gb300_blas_int ldb) {
    gb300_cblas_strsm_checked(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
    gb300_throw_if_error("cblas_strsm");
}
static inline void cblas_saxpy(gb300_blas_int n, float alpha, const float* x, gb300_blas_int incX, float* y,
    gb300_blas_int incY) {
    gb300_cblas_saxpy_checked(n, alpha, x, incX, y, incY);
    gb300_throw_if_error("cblas_saxpy");
}
static inline void cblas_dtrsm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
    CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, double alpha, const double* A, gb300_blas_int lda,
    double* B, gb300_blas_int ldb) {
    gb300_cblas_dtrsm_checked(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
    gb300_throw_if_error("cblas_dtrsm");
}
static inline void cblas_daxpy(gb300_blas_int n, double alpha, const double* x, gb300_blas_int incX, double* y,
    gb300_blas_int incY) {
    gb300_cblas_daxpy_checked(n, alpha, x, incX, y, incY);
    gb300_throw_if_error("cblas_daxpy");
}
static inline void cblas_ctrsm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
    CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda,
    void* B, gb300_blas_int ldb) {
    gb300_cblas_ctrsm_checked(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
    gb300_throw_if_error("cblas_ctrsm");
}
static inline void cblas_caxpy(gb300_blas_int n, const void* alpha, const void* x, gb300_blas_int incX, void* y,
    gb300_blas_int incY) {
    gb300_cblas_caxpy_checked(n, alpha, x, incX, y, incY);
    gb300_throw_if_error("cblas_caxpy");
}
static inline void cblas_ztrsm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
    CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A, gb300_blas_int lda,
    void* B, gb300_blas_int ldb) {
    gb300_cblas_ztrsm_checked(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
    gb300_throw_if_error("cblas_ztrsm");
}
static inline void cblas_zaxpy(gb300_blas_int n, const void* alpha, const void* x, gb300_blas_int incX, void* y,
    gb300_blas_int incY) {
    gb300_cblas_zaxpy_checked(n, alpha, x, incX, y, incY);
    gb300_throw_if_error("cblas_zaxpy");
}
static inline float cblas_sdot(gb300_blas_int n, const float* x, gb300_blas_int incX, const float* y,
    gb300_blas_int incY) {
    const float r = gb300_cblas_sdot_checked(n, x, incX, y, incY);
    gb300_throw_if_error("cblas_sdot");
    return r;
}
static inline double cblas_ddot(gb300_blas_int n, const double* x, gb300_blas_int incX, const double* y,
    gb300_blas_int incY) {
    const double r = gb300_cblas_ddot_checked(n, x, incX, y, incY);
    gb300_throw_if_error("cblas_ddot");
    return r;
}
static inline void cblas_cdotu_sub(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotu) {
    gb300_cblas_cdotu_sub_checked(n, x, incX, y, incY, dotu);
    gb300_throw_if_error("cblas_cdotu_sub");
}
static inline void cblas_cdotu(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotu) {
    gb300_cblas_cdotu_checked(n, x, incX, y, incY, dotu);
    gb300_throw_if_error("cblas_cdotu");
}
static inline void cblas_cdotc_sub(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotc) {
    gb300_cblas_cdotc_sub_checked(n, x, incX, y, incY, dotc);
    gb300_throw_if_error("cblas_cdotc_sub");
}
static inline void cblas_cdotc(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotc) {
    gb300_cblas_cdotc_checked(n, x, incX, y, incY, dotc);
    gb300_throw_if_error("cblas_cdotc");
}
static inline void cblas_zdotu_sub(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotu) {
    gb300_cblas_zdotu_sub_checked(n, x, incX, y, incY, dotu);
    gb300_throw_if_error("cblas_zdotu_sub");
}
static inline void cblas_zdotu(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotu) {
    gb300_cblas_zdotu_checked(n, x, incX, y, incY, dotu);
    gb300_throw_if_error("cblas_zdotu");
}
static inline void cblas_zdotc_sub(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotc) {
    gb300_cblas_zdotc_sub_checked(n, x, incX, y, incY, dotc);
    gb300_throw_if_error("cblas_zdotc_sub");
}
static inline void cblas_zdotc(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
    gb300_blas_int incY, void* dotc) {
    gb300_cblas_zdotc_checked(n, x, incX, y, incY, dotc);
    gb300_throw_if_error("cblas_zdotc");
}
}
#endif

#endif /* GB300_CBLAS_H */
