// stub_cblas.cpp — TEST-ONLY stand-in for libgb300blas used to check the Blaze seam on a host
// without a GPU: it implements the gb300_cblas.h surface on the CPU (a plain triple loop), and
// logs each call's CBLAS arguments to the file named by GB300_STUB_LOG, so the test can compare
// them with what blaze::gemm() must pass (blaze/math/blas/gemm.h:115-131).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "gb300_cblas.h"

namespace {
thread_local int t_status = 0;
thread_local char t_msg[256] = "";

void log_call(const char* name, int order, int ta, int tb, long m, long n, long k, double alpha, long lda, long ldb,
              double beta, long ldc) {
    const char* path = std::getenv("GB300_STUB_LOG");
    if (!path) return;
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%s %d %d %d %ld %ld %ld %.17g %ld %ld %.17g %ld\n", name, order, ta, tb, m, n, k, alpha, lda, ldb,
                 beta, ldc);
    std::fclose(f);
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
}  // namespace

extern "C" {
int gb300_last_error(void) { return t_status; }
const char* gb300_last_error_message(void) { return t_msg; }
void gb300_clear_error(void) { t_status = 0; t_msg[0] = 0; }

void gb300_cblas_dgemm_checked(CBLAS_ORDER order, CBLAS_TRANSPOSE transA, CBLAS_TRANSPOSE transB, gb300_blas_int m,
                               gb300_blas_int n, gb300_blas_int k, double alpha, const double* A, gb300_blas_int lda,
                               const double* B, gb300_blas_int ldb, double beta, double* C, gb300_blas_int ldc) {
    log_call("dgemm", order, transA, transB, m, n, k, alpha, lda, ldb, beta, ldc);
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
    log_call("sgemm", order, transA, transB, m, n, k, alpha, lda, ldb, beta, ldc);
    gemm<float>(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
}
