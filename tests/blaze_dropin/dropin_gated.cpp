// dropin_gated.cpp — products that Blaze's kernel selection keeps on the CPU even in BLAS mode
// (blaze/math/expressions/DMatDMatMultExpr.h:561-569 and its three siblings: a result of fewer
// than 4900 elements, or a skinny operand of at most 10 SIMD widths), built in BLAS mode against
// gb300_cblas.h, with (-DGB300_INTERCEPT: include/gb300_blaze.h included) and without the
// interception header.
//
// One line per product:
//   <label> status=<ok|exception> maxdiff=<|C - reference| on checked rows> gated=<0|1> m= n= k=
// gated=1: Blaze's own selection would use its small CPU kernel for this product.  The reference
// is a plain loop over the same operands (every row of small results, every 61st row of large ones).
#include <blaze/Math.h>
#ifdef GB300_INTERCEPT
#include <gb300_blaze.h>
#endif

#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

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
double maxdiff(const MC& C, const M1& A, const M2& B, double scale, const MC* C0, double c0scale) {
    const size_t step = C.rows() > 256 ? 61 : 1;
    double d = 0.0;
    for (size_t i = 0; i < C.rows(); i += step)
        for (size_t j = 0; j < C.columns(); ++j) {
            double r = 0.0;
            for (size_t p = 0; p < A.columns(); ++p) r += double(A(i, p)) * double(B(p, j));
            r *= scale;
            if (C0) r += c0scale * double((*C0)(i, j));
            d = std::max(d, std::fabs(double(C(i, j)) - r));
        }
    return d;
}

constexpr size_t kGate = blaze::SIMDTrait<double>::size * 10UL;  // Blaze's skinny-operand gate

template <typename T, bool SOC, bool SOA, bool SOB>
void run(const char* label, size_t m, size_t k, size_t n, bool gated, bool forms = false) {
    blaze::DynamicMatrix<T, SOA> A(m, k);
    blaze::DynamicMatrix<T, SOB> B(k, n);
    blaze::DynamicMatrix<T, SOC> C(m, n), C0;
    fill(A, 1);
    fill(B, 2);
    const std::string base(label);
    auto report = [&](const char* what, auto&& body, double scale, bool with_c0) {
        try {
            fill(C, 3);
            C0 = C;
            body();
            std::printf("%s%s status=ok maxdiff=%.3e gated=%d m=%zu n=%zu k=%zu\n", base.c_str(), what,
                        maxdiff(C, A, B, scale, with_c0 ? &C0 : nullptr, 1.0), gated ? 1 : 0, m, n, k);
        } catch (const std::exception& e) {
            std::printf("%s%s status=exception what=\"%s\"\n", base.c_str(), what, e.what());
        }
    };
    report("", [&] { C = A * B; }, 1.0, false);
    if (forms) {
        report("/add", [&] { C += A * B; }, 1.0, true);
        report("/sub", [&] { C -= A * B; }, -1.0, true);
        report("/scaled", [&] { C = 2.5 * (A * B); }, 2.5, false);
    }
}

int main() {
    // skinny operands: B with kGate columns (row-major result of row-major operands, or of a
    // column-major A), A with kGate rows (column-major operands and result)
    run<double, rowMajor, rowMajor, rowMajor>("skinny_rr", 4096, 4096, kGate, true);
    run<double, rowMajor, columnMajor, rowMajor>("skinny_cr", 4096, 4096, kGate, true);
    run<double, columnMajor, columnMajor, columnMajor>("skinny_cc", kGate, 4096, 4096, true);
    // small results (fewer than 4900 elements): every storage-order class, the other assignment
    // forms, float
    run<double, rowMajor, rowMajor, rowMajor>("small_rr", 30, 50, 40, true, true);
    run<double, rowMajor, rowMajor, columnMajor>("small_rc", 30, 50, 40, true);
    run<double, rowMajor, columnMajor, rowMajor>("small_cr", 30, 50, 40, true);
    run<double, columnMajor, columnMajor, columnMajor>("small_cc", 30, 50, 40, true);
    run<float, rowMajor, rowMajor, rowMajor>("small_float", 24, 33, 17, true);
    // a product Blaze already sends to BLAS: the same single call either way
    run<double, rowMajor, rowMajor, rowMajor>("large_rr", 100, 90, 96, false);
    // a CustomMatrix target over caller memory
    {
        std::vector<double> c(20 * 30);
        blaze::DynamicMatrix<double, rowMajor> A(20, 25), B(25, 30);
        fill(A, 4);
        fill(B, 5);
        blaze::CustomMatrix<double, blaze::unaligned, blaze::unpadded, rowMajor> C(c.data(), 20, 30);
        try {
            C = A * B;
            std::printf("custom_small status=ok maxdiff=%.3e gated=1 m=20 n=30 k=25\n",
                        maxdiff(C, A, B, 1.0, static_cast<decltype(&C)>(nullptr), 0.0));
        } catch (const std::exception& e) {
            std::printf("custom_small status=exception what=\"%s\"\n", e.what());
        }
    }
    // an operand that is itself an expression: Blaze evaluates it into a temporary first, and the
    // product of the evaluated operands is then intercepted like the others
    {
        blaze::DynamicMatrix<double, rowMajor> A(20, 25), B(25, 30), C(20, 30), A2;
        fill(A, 6);
        fill(B, 7);
        try {
            C = (A + A) * B;
            A2 = A + A;
            std::printf("expr_operand status=ok maxdiff=%.3e gated=1 m=20 n=30 k=25\n",
                        maxdiff(C, A2, B, 1.0, static_cast<decltype(&C)>(nullptr), 0.0));
        } catch (const std::exception& e) {
            std::printf("expr_operand status=exception what=\"%s\"\n", e.what());
        }
    }
    return 0;
}
