// dropin_smp.cpp — Blaze's OpenMP evaluation of C = A*B in BLAS mode with BLAZE_BLAS_IS_PARALLEL=0:
// smpAssign (blaze/math/smp/openmp/DenseMatrix.h:97-160) splits C into one block per thread, and
// each thread evaluates its block's product through submatrix views
// (blaze/math/views/submatrix/Dense.h), so cblas_dgemm is called concurrently on tiles whose
// pointers lie inside the operands and whose leading dimensions are the whole matrices'.
//
// Built with -fopenmp -DBLAZE_BLAS_IS_PARALLEL=0 and run with OMP_NUM_THREADS > 1.  Before each
// product the program appends "product <label> <M> <N> <K> <A> <B> <C>" (base addresses) to the
// stub's log, so that the logged tile calls (GB300_STUB_LOG_PTRS=1) can be placed inside the
// whole matrices.  One line per product on stdout: <label> status=<ok|exception> maxdiff=<..>.
#include <blaze/Math.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>

using blaze::columnMajor;
using blaze::rowMajor;

template <typename MT>
void fill(MT& M, unsigned seed) {
    unsigned s = seed;
    for (size_t i = 0; i < M.rows(); ++i)
        for (size_t j = 0; j < M.columns(); ++j) {
            s = s * 1664525u + 1013904223u;
            M(i, j) = (double((s >> 8) & 0xffff) / 32768.0) - 1.0;
        }
}

template <typename MC, typename M1, typename M2>
double maxdiff(const MC& C, const M1& A, const M2& B, double scale, const MC* C0) {
    double d = 0.0;
    for (size_t i = 0; i < C.rows(); ++i)
        for (size_t j = 0; j < C.columns(); ++j) {
            double r = 0.0;
            for (size_t p = 0; p < A.columns(); ++p) r += A(i, p) * B(p, j);
            r *= scale;
            if (C0) r += (*C0)(i, j);
            d = std::max(d, std::fabs(C(i, j) - r));
        }
    return d;
}

void mark(const char* label, size_t m, size_t n, size_t k, const void* a, const void* b, const void* c) {
    const char* path = std::getenv("GB300_STUB_LOG");
    if (!path) return;
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "product %s %zu %zu %zu %p %p %p\n", label, m, n, k, a, b, c);
    std::fclose(f);
}

template <bool SOC, bool SOA, bool SOB>
void run(const char* label, size_t m, size_t k, size_t n, bool add = false) {
    blaze::DynamicMatrix<double, SOA> A(m, k);
    blaze::DynamicMatrix<double, SOB> B(k, n);
    blaze::DynamicMatrix<double, SOC> C(m, n), C0;
    fill(A, 1);
    fill(B, 2);
    fill(C, 3);
    C0 = C;
    mark(label, m, n, k, A.data(), B.data(), C.data());
    try {
        if (add) C += A * B;
        else C = A * B;
        std::printf("%s status=ok maxdiff=%.3e\n", label, maxdiff(C, A, B, 1.0, add ? &C0 : nullptr));
    } catch (const std::exception& e) {
        std::printf("%s status=exception what=\"%s\"\n", label, e.what());
    }
}

int main() {
    run<rowMajor, rowMajor, rowMajor>("smp_rr", 400, 350, 300);
    run<rowMajor, rowMajor, rowMajor>("smp_rr_add", 400, 350, 300, true);
    run<rowMajor, rowMajor, columnMajor>("smp_rc", 320, 300, 280);
    run<columnMajor, columnMajor, columnMajor>("smp_cc", 300, 250, 410);
    run<columnMajor, rowMajor, columnMajor>("smp_c_rc", 260, 330, 300);
    return 0;
}
