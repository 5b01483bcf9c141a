// dropin_main.cpp — Blaze program built in BLAS mode against gb300_cblas.h (test of the seam).
//
// Compiled with -DBLAZE_BLAS_MODE=1 -DBLAZE_BLAS_IS_PARALLEL=1
//               -DBLAZE_BLAS_INCLUDE_FILE="<gb300_cblas.h>" -DGB300_BLAS_THROW
// and linked either against a recording stub (stub_cblas.cpp: checks how Blaze calls cblas_dgemm)
// or against libgb300blas.so itself (checks that a library error surfaces as an exception).
// It exercises the four multiplication expression classes (row/column-major operands and result:
// DMatDMatMultExpr, DMatTDMatMultExpr, TDMatDMatMultExpr, TDMatTDMatMultExpr), CustomMatrix,
// `C = A*B`, `C += A*B`, `C -= A*B` and `C = s*(A*B)`, and prints one line per product:
//   <label> status=<ok|exception> maxdiff=<|C - reference|>
// where the reference is Blaze's own default kernel on the same operands (BLAS bypassed by
// evaluating the product element by element).
#include <blaze/Math.h>

#include <cmath>
#include <cstdio>
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

template <typename M1, typename M2>
double reference_entry(const M1& A, const M2& B, size_t i, size_t j) {
    double s = 0.0;
    for (size_t p = 0; p < A.columns(); ++p) s += A(i, p) * B(p, j);
    return s;
}

template <typename MC, typename M1, typename M2>
double maxdiff(const MC& C, const M1& A, const M2& B, double scale, const MC* C0, double c0scale) {
    double d = 0.0;
    for (size_t i = 0; i < C.rows(); ++i)
        for (size_t j = 0; j < C.columns(); ++j) {
            double r = scale * reference_entry(A, B, i, j);
            if (C0) r += c0scale * (*C0)(i, j);
            d = std::max(d, std::fabs(C(i, j) - r));
        }
    return d;
}

template <bool SOC, bool SOA, bool SOB>
void run(const char* label, size_t m, size_t n, size_t k) {
    blaze::DynamicMatrix<double, SOA> A(m, k);
    blaze::DynamicMatrix<double, SOB> B(k, n);
    blaze::DynamicMatrix<double, SOC> C(m, n), C0;
    fill(A, 1);
    fill(B, 2);
    const std::string base(label);
    auto report = [&](const std::string& what, auto&& body, double scale, bool with_c0, double c0scale) {
        try {
            fill(C, 3);
            C0 = C;
            body();
            std::printf("%s/%s status=ok maxdiff=%.3e\n", base.c_str(), what.c_str(),
                        maxdiff(C, A, B, scale, with_c0 ? &C0 : nullptr, c0scale));
        } catch (const std::exception& e) {
            std::printf("%s/%s status=exception what=\"%s\"\n", base.c_str(), what.c_str(), e.what());
        }
    };
    report("assign", [&] { C = A * B; }, 1.0, false, 0.0);
    report("add", [&] { C += A * B; }, 1.0, true, 1.0);
    report("sub", [&] { C -= A * B; }, -1.0, true, 1.0);
    report("scaled", [&] { C = 2.5 * (A * B); }, 2.5, false, 0.0);
}

int main() {
    // 100 x 96 x 90: M*N >= 4900 and N > 10*SIMDSIZE, so every storage-order class takes the BLAS kernel
    run<rowMajor, rowMajor, rowMajor>("rr_r", 100, 96, 90);
    run<rowMajor, rowMajor, columnMajor>("rc_r", 100, 96, 90);
    run<rowMajor, columnMajor, rowMajor>("cr_r", 100, 96, 90);
    run<rowMajor, columnMajor, columnMajor>("cc_r", 100, 96, 90);
    run<columnMajor, rowMajor, rowMajor>("rr_c", 100, 96, 90);
    run<columnMajor, columnMajor, columnMajor>("cc_c", 100, 96, 90);
    // CustomMatrix over caller memory (unpadded, odd leading dimension)
    {
        std::vector<double> a(101 * 97), b(97 * 99), c(101 * 99);
        blaze::CustomMatrix<double, blaze::unaligned, blaze::unpadded, rowMajor> A(a.data(), 101, 97);
        blaze::CustomMatrix<double, blaze::unaligned, blaze::unpadded, rowMajor> B(b.data(), 97, 99);
        blaze::CustomMatrix<double, blaze::unaligned, blaze::unpadded, rowMajor> C(c.data(), 101, 99);
        fill(A, 4);
        fill(B, 5);
        try {
            C = A * B;
            double d = 0.0;
            for (size_t i = 0; i < 101; ++i)
                for (size_t j = 0; j < 99; ++j) d = std::max(d, std::fabs(C(i, j) - reference_entry(A, B, i, j)));
            std::printf("custom/assign status=ok maxdiff=%.3e\n", d);
        } catch (const std::exception& e) {
            std::printf("custom/assign status=exception what=\"%s\"\n", e.what());
        }
    }
    return 0;
}
