// stub_cblas.cpp — TEST-ONLY stand-in for libgb300blas used to check the Blaze seam on a host
// without a GPU: it implements the gb300_cblas.h routines Blaze calls on the CPU (plain loops), and
// logs each call's CBLAS arguments to the file named by GB300_STUB_LOG, so the test can compare
// them with what Blaze must pass (blaze/math/blas/gemm.h:115-131 and the gemv / trmv / trmm /
// trsm / axpy / dot wrappers next to it) and replay them through the real library.
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "gb300_cblas.h"

namespace {
thread_local int t_status = 0;
thread_local char t_msg[256] = "";

// With GB300_STUB_LOG_PTRS set, a ?gemm line also carries the addresses of A, B and C (hex), from
// which a test recovers where each call's operands lie inside the caller's matrices.
void log_call(const char* name, int order, int ta, int tb, long m, long n, long k, double alpha, long lda, long ldb,
              double beta, long ldc, const void* A = nullptr, const void* B = nullptr, const void* C = nullptr) {
    const char* path = std::getenv("GB300_STUB_LOG");
    if (!path) return;
    char line[512];
    int len = std::snprintf(line, sizeof line, "%s %d %d %d %ld %ld %ld %.17g %ld %ld %.17g %ld", name, order, ta, tb,
                            m, n, k, alpha, lda, ldb, beta, ldc);
    if (std::getenv("GB300_STUB_LOG_PTRS"))
        len += std::snprintf(line + len, sizeof line - size_t(len), " %p %p %p", A, B, C);
    line[len++] = '\n';
    // one write per line: concurrent callers (Blaze's OpenMP tiles) append whole lines
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fwrite(line, 1, size_t(len), f);
    std::fclose(f);
}

void log_line(const char* fmt, ...) {
    const char* path = std::getenv("GB300_STUB_LOG");
    if (!path) return;
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    va_list ap;
    va_start(ap, fmt);
    std::vfprintf(f, fmt, ap);
    va_end(ap);
    std::fclose(f);
}

template <typename T>
struct is_cplx : std::false_type {};
template <typename T>
struct is_cplx<std::complex<T>> : std::true_type {};

template <typename T>
T conj_if(T a, bool c) {
    if constexpr (is_cplx<T>::value) return c ? std::conj(a) : a;
    else return a;
}

// element (i, j) of the CBLAS-stored matrix (leading dimension ld)
template <typename T>
T& at(T* A, long ld, int order, long i, long j) {
    return order == CblasRowMajor ? A[i * ld + j] : A[j * ld + i];
}

// element (r, c) of op(A), A stored m x n in CBLAS order
template <typename T>
T op_at(const T* A, long ld, int order, int trans, long r, long c) {
    T* a = const_cast<T*>(A);
    return trans == CblasNoTrans ? at(a, ld, order, r, c) : conj_if(at(a, ld, order, c, r), trans == CblasConjTrans);
}

template <typename T>
T& vec(T* x, long inc, long len, long k) {
    return inc > 0 ? x[k * inc] : x[(len - 1 - k) * -inc];
}

template <typename T>
void gemv(int order, int trans, long m, long n, T alpha, const T* A, long lda, const T* x, long incx, T beta, T* y,
          long incy) {
    const long yl = trans == CblasNoTrans ? m : n, xl = trans == CblasNoTrans ? n : m;
    for (long r = 0; r < yl; ++r) {
        T s = T(0);
        for (long c = 0; c < xl; ++c) s += op_at(A, lda, order, trans, r, c) * vec(const_cast<T*>(x), incx, xl, c);
        T& yr = vec(y, incy, yl, r);
        yr = (beta == T(0)) ? alpha * s : alpha * s + beta * yr;
    }
}

// the triangular matrix: zero outside the uplo triangle, one on a unit diagonal
template <typename T>
T tri_at(const T* A, long lda, int order, int uplo, int diag, long i, long j) {
    const bool in = uplo == CblasLower ? j <= i : j >= i;
    if (!in) return T(0);
    if (diag == CblasUnit && i == j) return T(1);
    return at(const_cast<T*>(A), lda, order, i, j);
}
template <typename T>
T op_tri(const T* A, long lda, int order, int uplo, int trans, int diag, long r, long c) {
    return trans == CblasNoTrans ? tri_at(A, lda, order, uplo, diag, r, c)
                                 : conj_if(tri_at(A, lda, order, uplo, diag, c, r), trans == CblasConjTrans);
}

template <typename T>
void trmv(int order, int uplo, int trans, int diag, long n, const T* A, long lda, T* x, long incx) {
    std::vector<T> t(n);
    for (long r = 0; r < n; ++r) {
        T s = T(0);
        for (long c = 0; c < n; ++c) s += op_tri(A, lda, order, uplo, trans, diag, r, c) * vec(x, incx, n, c);
        t[r] = s;
    }
    for (long r = 0; r < n; ++r) vec(x, incx, n, r) = t[r];
}

template <typename T>
void trmm(int order, int side, int uplo, int trans, int diag, long m, long n, T alpha, const T* A, long lda, T* B,
          long ldb) {
    std::vector<T> t(m * n);
    for (long i = 0; i < m; ++i)
        for (long j = 0; j < n; ++j) {
            T s = T(0);
            if (side == CblasLeft)
                for (long p = 0; p < m; ++p) s += op_tri(A, lda, order, uplo, trans, diag, i, p) * at(B, ldb, order, p, j);
            else
                for (long p = 0; p < n; ++p) s += at(B, ldb, order, i, p) * op_tri(A, lda, order, uplo, trans, diag, p, j);
            t[i * n + j] = alpha * s;
        }
    for (long i = 0; i < m; ++i)
        for (long j = 0; j < n; ++j) at(B, ldb, order, i, j) = t[i * n + j];
}

template <typename T>
void cgemm(int order, int ta, int tb, long m, long n, long k, T alpha, const T* A, long lda, const T* B, long ldb,
           T beta, T* C, long ldc) {
    for (long i = 0; i < m; ++i)
        for (long j = 0; j < n; ++j) {
            T s = T(0);
            for (long p = 0; p < k; ++p) s += op_at(A, lda, order, ta, i, p) * op_at(B, ldb, order, tb, p, j);
            T& c = at(C, ldc, order, i, j);
            c = (beta == T(0)) ? alpha * s : alpha * s + beta * c;
        }
}

template <typename T>
void gemm(int order, int ta, int tb, long m, long n, long k, T alpha, const T* A, long lda, const T* B, long ldb,
          T beta, T* C, long ldc) {
    auto a = [&](long i, long p) -> T {
        const bool t = ta != CblasNoTrans;
        if (order == CblasRowMajor) return t ? A[p * lda + i] : A[i * lda + p];
        return t ? A[i * lda + p] : A[p * lda + i];
    };
    auto b = [&](long p, long j) -> T {
        const bool t = tb != CblasNoTrans;
        if (order == CblasRowMajor) return t ? B[j * ldb + p] : B[p * ldb + j];
        return t ? B[p * ldb + j] : B[j * ldb + p];
    };
    for (long i = 0; i < m; ++i)
        for (long j = 0; j < n; ++j) {
            T s = 0;
            for (long p = 0; p < k; ++p) s += a(i, p) * b(p, j);
            T& c = (order == CblasRowMajor) ? C[i * ldc + j] : C[j * ldc + i];
            c = (beta == T(0)) ? alpha * s : alpha * s + beta * c;
        }
}
// B = alpha op(A)^-1 B (left) or alpha B op(A)^-1 (right) by substitution on the logical matrices
template <typename T>
void trsm(int order, int side, int uplo, int trans, int diag, long m, long n, T alpha, const T* A, long lda, T* B,
          long ldb) {
    const bool left = side == CblasLeft;
    const long ka = left ? m : n;
    const bool lower = (uplo == CblasLower) == (trans == CblasNoTrans);  // op(A) lower triangular
    std::vector<T> X(m * n);
    for (long i = 0; i < m; ++i)
        for (long j = 0; j < n; ++j) X[i * n + j] = alpha * at(B, ldb, order, i, j);
    auto t = [&](long r, long c) { return op_tri(A, lda, order, uplo, trans, diag, r, c); };
    for (long s = 0; s < ka; ++s) {
        // left: rows of X in the order op(A) allows; right: columns (X op(A) = B, op(A)^T X^T = B^T)
        const bool forward = left ? lower : !lower;
        const long i = forward ? s : ka - 1 - s;
        const long k0 = forward ? 0 : i + 1, k1 = forward ? i : ka;
        if (left) {
            for (long j = 0; j < n; ++j) {
                T v = X[i * n + j];
                for (long k = k0; k < k1; ++k) v -= t(i, k) * X[k * n + j];
                X[i * n + j] = v / t(i, i);
            }
        } else {
            for (long r = 0; r < m; ++r) {
                T v = X[r * n + i];
                for (long k = k0; k < k1; ++k) v -= X[r * n + k] * t(k, i);
                X[r * n + i] = v / t(i, i);
            }
        }
    }
    for (long i = 0; i < m; ++i)
        for (long j = 0; j < n; ++j) at(B, ldb, order, i, j) = X[i * n + j];
}

template <typename T>
void axpy(long n, T alpha, const T* x, long incx, T* y, long incy) {
    for (long k = 0; k < n; ++k) vec(y, incy, n, k) += alpha * vec(const_cast<T*>(x), incx, n, k);
}

template <typename T>
T dot(long n, const T* x, long incx, const T* y, long incy, bool conj) {
    T s = T(0);
    for (long k = 0; k < n; ++k)
        s += conj_if(vec(const_cast<T*>(x), incx, n, k), conj) * vec(const_cast<T*>(y), incy, n, k);
    return s;
}
}  // namespace

extern "C" {
int gb300_last_error(void) { return t_status; }
const char* gb300_last_error_message(void) { return t_msg; }
void gb300_clear_error(void) { t_status = 0; t_msg[0] = 0; }

void gb300_cblas_dgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                               gb300_blas_int n, gb300_blas_int k, double alpha, const double* A, gb300_blas_int lda,
                               const double* B, gb300_blas_int ldb, double beta, double* C, gb300_blas_int ldc) {
    log_call("dgemm", order, transA, transB, m, n, k, alpha, lda, ldb, beta, ldc, A, B, C);
    if (std::getenv("GB300_STUB_FAIL")) {
        t_status = 2;
        std::strcpy(t_msg, "injected failure");
        return;
    }
    gemm<double>(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

void gb300_cblas_sgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                               gb300_blas_int n, gb300_blas_int k, float alpha, const float* A, gb300_blas_int lda,
                               const float* B, gb300_blas_int ldb, float beta, float* C, gb300_blas_int ldc) {
    log_call("sgemm", order, transA, transB, m, n, k, alpha, lda, ldb, beta, ldc, A, B, C);
    gemm<float>(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

// ---- the routines next to ?gemm (logged as: name, then the CBLAS arguments in order, with complex
// scalars as re,im and the pointers left out) ------------------------------------------------------
using CF = std::complex<float>;
using CD = std::complex<double>;

void gb300_cblas_sgemv_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n,
                               float alpha, const float* A, gb300_blas_int lda, const float* x, gb300_blas_int incX,
                               float beta, float* y, gb300_blas_int incY) {
    log_line("sgemv %d %d %ld %ld %.9g %ld %ld %.9g %ld\n", order, transA, long(m), long(n), alpha, long(lda),
             long(incX), beta, long(incY));
    gemv<float>(order, transA, m, n, alpha, A, lda, x, incX, beta, y, incY);
}
void gb300_cblas_dgemv_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n,
                               double alpha, const double* A, gb300_blas_int lda, const double* x,
                               gb300_blas_int incX, double beta, double* y, gb300_blas_int incY) {
    log_line("dgemv %d %d %ld %ld %.17g %ld %ld %.17g %ld\n", order, transA, long(m), long(n), alpha, long(lda),
             long(incX), beta, long(incY));
    gemv<double>(order, transA, m, n, alpha, A, lda, x, incX, beta, y, incY);
}
void gb300_cblas_zgemv_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n,
                               const void* alpha, const void* A, gb300_blas_int lda, const void* x,
                               gb300_blas_int incX, const void* beta, void* y, gb300_blas_int incY) {
    const CD al = *static_cast<const CD*>(alpha), be = *static_cast<const CD*>(beta);
    log_line("zgemv %d %d %ld %ld %.17g,%.17g %ld %ld %.17g,%.17g %ld\n", order, transA, long(m), long(n), al.real(),
             al.imag(), long(lda), long(incX), be.real(), be.imag(), long(incY));
    gemv<CD>(order, transA, m, n, al, static_cast<const CD*>(A), lda, static_cast<const CD*>(x), incX, be,
             static_cast<CD*>(y), incY);
}
void gb300_cblas_cgemv_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, gb300_blas_int m, gb300_blas_int n,
                               const void* alpha, const void* A, gb300_blas_int lda, const void* x,
                               gb300_blas_int incX, const void* beta, void* y, gb300_blas_int incY) {
    const CF al = *static_cast<const CF*>(alpha), be = *static_cast<const CF*>(beta);
    log_line("cgemv %d %d %ld %ld %.9g,%.9g %ld %ld %.9g,%.9g %ld\n", order, transA, long(m), long(n), al.real(),
             al.imag(), long(lda), long(incX), be.real(), be.imag(), long(incY));
    gemv<CF>(order, transA, m, n, al, static_cast<const CF*>(A), lda, static_cast<const CF*>(x), incX, be,
             static_cast<CF*>(y), incY);
}
void gb300_cblas_dtrmv_checked(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                               gb300_blas_int n, const double* A, gb300_blas_int lda, double* x,
                               gb300_blas_int incX) {
    log_line("dtrmv %d %d %d %d %ld %ld %ld\n", order, uplo, transA, diag, long(n), long(lda), long(incX));
    trmv<double>(order, uplo, transA, diag, n, A, lda, x, incX);
}
void gb300_cblas_strmv_checked(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                               gb300_blas_int n, const float* A, gb300_blas_int lda, float* x, gb300_blas_int incX) {
    log_line("strmv %d %d %d %d %ld %ld %ld\n", order, uplo, transA, diag, long(n), long(lda), long(incX));
    trmv<float>(order, uplo, transA, diag, n, A, lda, x, incX);
}
void gb300_cblas_ztrmv_checked(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                               gb300_blas_int n, const void* A, gb300_blas_int lda, void* x, gb300_blas_int incX) {
    log_line("ztrmv %d %d %d %d %ld %ld %ld\n", order, uplo, transA, diag, long(n), long(lda), long(incX));
    trmv<CD>(order, uplo, transA, diag, n, static_cast<const CD*>(A), lda, static_cast<CD*>(x), incX);
}
void gb300_cblas_ctrmv_checked(CBLAS_ORDER order, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA, CBLAS_DIAG diag,
                               gb300_blas_int n, const void* A, gb300_blas_int lda, void* x, gb300_blas_int incX) {
    log_line("ctrmv %d %d %d %d %ld %ld %ld\n", order, uplo, transA, diag, long(n), long(lda), long(incX));
    trmv<CF>(order, uplo, transA, diag, n, static_cast<const CF*>(A), lda, static_cast<CF*>(x), incX);
}
void gb300_cblas_dtrmm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
                               CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, double alpha, const double* A,
                               gb300_blas_int lda, double* B, gb300_blas_int ldb) {
    log_line("dtrmm %d %d %d %d %d %ld %ld %.17g %ld %ld\n", order, side, uplo, transA, diag, long(m), long(n), alpha,
             long(lda), long(ldb));
    trmm<double>(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
void gb300_cblas_strmm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
                               CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, float alpha, const float* A,
                               gb300_blas_int lda, float* B, gb300_blas_int ldb) {
    log_line("strmm %d %d %d %d %d %ld %ld %.9g %ld %ld\n", order, side, uplo, transA, diag, long(m), long(n), alpha,
             long(lda), long(ldb));
    trmm<float>(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
void gb300_cblas_ztrmm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
                               CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A,
                               gb300_blas_int lda, void* B, gb300_blas_int ldb) {
    const CD al = *static_cast<const CD*>(alpha);
    log_line("ztrmm %d %d %d %d %d %ld %ld %.17g,%.17g %ld %ld\n", order, side, uplo, transA, diag, long(m), long(n),
             al.real(), al.imag(), long(lda), long(ldb));
    trmm<CD>(order, side, uplo, transA, diag, m, n, al, static_cast<const CD*>(A), lda, static_cast<CD*>(B), ldb);
}
void gb300_cblas_ctrmm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
                               CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A,
                               gb300_blas_int lda, void* B, gb300_blas_int ldb) {
    const CF al = *static_cast<const CF*>(alpha);
    log_line("ctrmm %d %d %d %d %d %ld %ld %.9g,%.9g %ld %ld\n", order, side, uplo, transA, diag, long(m), long(n),
             al.real(), al.imag(), long(lda), long(ldb));
    trmm<CF>(order, side, uplo, transA, diag, m, n, al, static_cast<const CF*>(A), lda, static_cast<CF*>(B), ldb);
}
void gb300_cblas_zgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                               gb300_blas_int n, gb300_blas_int k, const void* alpha, const void* A,
                               gb300_blas_int lda, const void* B, gb300_blas_int ldb, const void* beta, void* C,
                               gb300_blas_int ldc) {
    const CD al = *static_cast<const CD*>(alpha), be = *static_cast<const CD*>(beta);
    log_line("zgemm %d %d %d %ld %ld %ld %.17g,%.17g %ld %ld %.17g,%.17g %ld\n", order, transA, transB, long(m),
             long(n), long(k), al.real(), al.imag(), long(lda), long(ldb), be.real(), be.imag(), long(ldc));
    cgemm<CD>(order, transA, transB, m, n, k, al, static_cast<const CD*>(A), lda, static_cast<const CD*>(B), ldb, be,
              static_cast<CD*>(C), ldc);
}
void gb300_cblas_cgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                               gb300_blas_int n, gb300_blas_int k, const void* alpha, const void* A,
                               gb300_blas_int lda, const void* B, gb300_blas_int ldb, const void* beta, void* C,
                               gb300_blas_int ldc) {
    const CF al = *static_cast<const CF*>(alpha), be = *static_cast<const CF*>(beta);
    log_line("cgemm %d %d %d %ld %ld %ld %.9g,%.9g %ld %ld %.9g,%.9g %ld\n", order, transA, transB, long(m), long(n),
             long(k), al.real(), al.imag(), long(lda), long(ldb), be.real(), be.imag(), long(ldc));
    cgemm<CF>(order, transA, transB, m, n, k, al, static_cast<const CF*>(A), lda, static_cast<const CF*>(B), ldb, be,
              static_cast<CF*>(C), ldc);
}
void gb300_cblas_dtrsm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
                               CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, double alpha, const double* A,
                               gb300_blas_int lda, double* B, gb300_blas_int ldb) {
    log_line("dtrsm %d %d %d %d %d %ld %ld %.17g %ld %ld\n", order, side, uplo, transA, diag, long(m), long(n), alpha,
             long(lda), long(ldb));
    trsm<double>(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
void gb300_cblas_strsm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
                               CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, float alpha, const float* A,
                               gb300_blas_int lda, float* B, gb300_blas_int ldb) {
    log_line("strsm %d %d %d %d %d %ld %ld %.9g %ld %ld\n", order, side, uplo, transA, diag, long(m), long(n), alpha,
             long(lda), long(ldb));
    trsm<float>(order, side, uplo, transA, diag, m, n, alpha, A, lda, B, ldb);
}
void gb300_cblas_ztrsm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
                               CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A,
                               gb300_blas_int lda, void* B, gb300_blas_int ldb) {
    const CD al = *static_cast<const CD*>(alpha);
    log_line("ztrsm %d %d %d %d %d %ld %ld %.17g,%.17g %ld %ld\n", order, side, uplo, transA, diag, long(m), long(n),
             al.real(), al.imag(), long(lda), long(ldb));
    trsm<CD>(order, side, uplo, transA, diag, m, n, al, static_cast<const CD*>(A), lda, static_cast<CD*>(B), ldb);
}
void gb300_cblas_ctrsm_checked(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transA,
                               CBLAS_DIAG diag, gb300_blas_int m, gb300_blas_int n, const void* alpha, const void* A,
                               gb300_blas_int lda, void* B, gb300_blas_int ldb) {
    const CF al = *static_cast<const CF*>(alpha);
    log_line("ctrsm %d %d %d %d %d %ld %ld %.9g,%.9g %ld %ld\n", order, side, uplo, transA, diag, long(m), long(n),
             al.real(), al.imag(), long(lda), long(ldb));
    trsm<CF>(order, side, uplo, transA, diag, m, n, al, static_cast<const CF*>(A), lda, static_cast<CF*>(B), ldb);
}
void gb300_cblas_daxpy_checked(gb300_blas_int n, double alpha, const double* x, gb300_blas_int incX, double* y,
                               gb300_blas_int incY) {
    log_line("daxpy %ld %.17g %ld %ld\n", long(n), alpha, long(incX), long(incY));
    axpy<double>(n, alpha, x, incX, y, incY);
}
void gb300_cblas_saxpy_checked(gb300_blas_int n, float alpha, const float* x, gb300_blas_int incX, float* y,
                               gb300_blas_int incY) {
    log_line("saxpy %ld %.9g %ld %ld\n", long(n), alpha, long(incX), long(incY));
    axpy<float>(n, alpha, x, incX, y, incY);
}
void gb300_cblas_zaxpy_checked(gb300_blas_int n, const void* alpha, const void* x, gb300_blas_int incX, void* y,
                               gb300_blas_int incY) {
    const CD al = *static_cast<const CD*>(alpha);
    log_line("zaxpy %ld %.17g,%.17g %ld %ld\n", long(n), al.real(), al.imag(), long(incX), long(incY));
    axpy<CD>(n, al, static_cast<const CD*>(x), incX, static_cast<CD*>(y), incY);
}
void gb300_cblas_caxpy_checked(gb300_blas_int n, const void* alpha, const void* x, gb300_blas_int incX, void* y,
                               gb300_blas_int incY) {
    const CF al = *static_cast<const CF*>(alpha);
    log_line("caxpy %ld %.9g,%.9g %ld %ld\n", long(n), al.real(), al.imag(), long(incX), long(incY));
    axpy<CF>(n, al, static_cast<const CF*>(x), incX, static_cast<CF*>(y), incY);
}
double gb300_cblas_ddot_checked(gb300_blas_int n, const double* x, gb300_blas_int incX, const double* y,
                                gb300_blas_int incY) {
    log_line("ddot %ld %ld %ld\n", long(n), long(incX), long(incY));
    return dot<double>(n, x, incX, y, incY, false);
}
float gb300_cblas_sdot_checked(gb300_blas_int n, const float* x, gb300_blas_int incX, const float* y,
                               gb300_blas_int incY) {
    log_line("sdot %ld %ld %ld\n", long(n), long(incX), long(incY));
    return dot<float>(n, x, incX, y, incY, false);
}
void gb300_cblas_zdotu_sub_checked(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
                                   gb300_blas_int incY, void* dotu) {
    log_line("zdotu_sub %ld %ld %ld\n", long(n), long(incX), long(incY));
    *static_cast<CD*>(dotu) = dot<CD>(n, static_cast<const CD*>(x), incX, static_cast<const CD*>(y), incY, false);
}
void gb300_cblas_zdotc_sub_checked(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
                                   gb300_blas_int incY, void* dotc) {
    log_line("zdotc_sub %ld %ld %ld\n", long(n), long(incX), long(incY));
    *static_cast<CD*>(dotc) = dot<CD>(n, static_cast<const CD*>(x), incX, static_cast<const CD*>(y), incY, true);
}
void gb300_cblas_cdotu_sub_checked(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
                                   gb300_blas_int incY, void* dotu) {
    log_line("cdotu_sub %ld %ld %ld\n", long(n), long(incX), long(incY));
    *static_cast<CF*>(dotu) = dot<CF>(n, static_cast<const CF*>(x), incX, static_cast<const CF*>(y), incY, false);
}
void gb300_cblas_cdotc_sub_checked(gb300_blas_int n, const void* x, gb300_blas_int incX, const void* y,
                                   gb300_blas_int incY, void* dotc) {
    log_line("cdotc_sub %ld %ld %ld\n", long(n), long(incX), long(incY));
    *static_cast<CF*>(dotc) = dot<CF>(n, static_cast<const CF*>(x), incX, static_cast<const CF*>(y), incY, true);
}
}
