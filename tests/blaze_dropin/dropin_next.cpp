// dropin_next.cpp — Blaze program built in BLAS mode against gb300_cblas.h that reaches the BLAS
// routines next to ?gemm through Blaze's own expressions (test of the seam).
//
// Compiled like dropin_main.cpp plus -DBLAZE_USE_BLAS_MATRIX_VECTOR_MULTIPLICATION=1 and lowered
// matrix x vector thresholds (blaze/config/Thresholds.h), so that modest sizes take the BLAS kernels:
//   y = A*x, y += A*x, y^T = x^T*A (dense, row- and column-major)  -> cblas_dgemv / cblas_sgemv
//   y = L*x, L a LowerMatrix / UpperMatrix adaptor                 -> cblas_dtrmv / cblas_ztrmv
//       (blaze/math/expressions/DMatDVecMultExpr.h:1166-1172)
//   complex y = A*x, C = A*B                                       -> cblas_zgemv, cblas_zgemm
//   C = L*B, L triangular (DMatDMatMultExpr.h:2026-2033)          -> cblas_dtrmm / cblas_ztrmm
//   C = A*B of a small area, with -DBLAZE_DMATDMATMULT_THRESHOLD=1 -> cblas_dgemm
//   C = A*B with B of at most 10 SIMD widths of columns            -> Blaze's own small kernel
//   blaze::dotu / dotc / axpy / trsm                               -> cblas_?dot / ?dot?_sub /
//                                                                     ?axpy / ?trsm
// and prints one line per product:  <label> status=<ok|exception> maxdiff=<|result - reference|>
// where the reference is a plain loop over the same operands (BLAS bypassed).
#include <blaze/Math.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <stdexcept>
#include <string>

using blaze::columnMajor;
using blaze::rowMajor;
using CD = std::complex<double>;

unsigned lcg(unsigned& s) {
    s = s * 1664525u + 1013904223u;
    return s;
}
double val(unsigned& s) { return (double((lcg(s) >> 8) & 0xffff) / 32768.0) - 1.0; }
template <typename T>
T make(unsigned& s) {
    if constexpr (std::is_same_v<T, CD>) {
        const double re = val(s);
        return CD(re, val(s));
    } else {
        return T(val(s));
    }
}

template <typename MT>
void fill(MT& M, unsigned seed) {  // the whole matrix (for an adaptor: its triangle only)
    unsigned s = seed;
    using T = blaze::ElementType_t<MT>;
    for (size_t i = 0; i < M.rows(); ++i)
        for (size_t j = 0; j < M.columns(); ++j) {
            const T v = make<T>(s);
            if constexpr (blaze::IsLower_v<MT>) { if (j <= i) M(i, j) = v; }
            else if constexpr (blaze::IsUpper_v<MT>) { if (j >= i) M(i, j) = v; }
            else M(i, j) = v;
        }
}
template <typename VT>
void fillv(VT& v, unsigned seed) {
    unsigned s = seed;
    for (size_t i = 0; i < v.size(); ++i) v[i] = make<blaze::ElementType_t<VT>>(s);
}

template <typename F>
void report(const char* label, F&& body) {
    try {
        const double d = body();
        std::printf("%s status=ok maxdiff=%.3e\n", label, d);
    } catch (const std::exception& e) {
        std::printf("%s status=exception what=\"%s\"\n", label, e.what());
    }
}

// max |y - (alpha * M v + beta * y0)| with M read element by element (no BLAS)
template <typename MT, typename VT, typename YT, typename S>
double mv_diff(const MT& M, const VT& v, const YT& y, S alpha, const YT* y0, S beta) {
    double d = 0.0;
    for (size_t i = 0; i < M.rows(); ++i) {
        S r = S(0);
        for (size_t j = 0; j < M.columns(); ++j) r += M(i, j) * v[j];
        r = alpha * r + (y0 ? beta * (*y0)[i] : S(0));
        d = std::max(d, double(std::abs(y[i] - r)));
    }
    return d;
}
template <typename M1, typename M2, typename MC>
double mm_diff(const M1& A, const M2& B, const MC& C) {
    double d = 0.0;
    using T = blaze::ElementType_t<MC>;
    for (size_t i = 0; i < C.rows(); ++i)
        for (size_t j = 0; j < C.columns(); ++j) {
            T r = T(0);
            for (size_t p = 0; p < A.columns(); ++p) r += A(i, p) * B(p, j);
            d = std::max(d, double(std::abs(C(i, j) - r)));
        }
    return d;
}

int main() {
    report("gemv_r", [] {
        blaze::DynamicMatrix<double, rowMajor> A(300, 200);
        blaze::DynamicVector<double> x(200), y;
        fill(A, 1); fillv(x, 2);
        y = A * x;
        return mv_diff(A, x, y, 1.0, (decltype(y)*)nullptr, 0.0);
    });
    report("gemv_c_add", [] {
        blaze::DynamicMatrix<double, columnMajor> A(300, 200);
        blaze::DynamicVector<double> x(200), y(300), y0;
        fill(A, 3); fillv(x, 4); fillv(y, 5);
        y0 = y;
        y += A * x;
        return mv_diff(A, x, y, 1.0, &y0, 1.0);
    });
    report("gemv_t", [] {
        blaze::DynamicMatrix<double, rowMajor> A(300, 200);
        blaze::DynamicVector<double, blaze::rowVector> x(300), y;
        fill(A, 6); fillv(x, 7);
        y = x * A;
        const blaze::DynamicMatrix<double, rowMajor> At(trans(A));
        return mv_diff(At, x, y, 1.0, (decltype(y)*)nullptr, 0.0);
    });
    report("sgemv_r", [] {
        blaze::DynamicMatrix<float, rowMajor> A(300, 200);
        blaze::DynamicVector<float> x(200), y;
        fill(A, 8); fillv(x, 9);
        y = A * x;
        return mv_diff(A, x, y, 1.0f, (decltype(y)*)nullptr, 0.0f);
    });
    report("trmv_lower_r", [] {
        blaze::LowerMatrix<blaze::DynamicMatrix<double, rowMajor>> L(200);
        blaze::DynamicVector<double> x(200), y;
        fill(L, 10); fillv(x, 11);
        y = L * x;
        return mv_diff(L, x, y, 1.0, (decltype(y)*)nullptr, 0.0);
    });
    report("trmv_upper_c", [] {
        blaze::UpperMatrix<blaze::DynamicMatrix<double, columnMajor>> U(200);
        blaze::DynamicVector<double> x(200), y;
        fill(U, 12); fillv(x, 13);
        y = U * x;
        return mv_diff(U, x, y, 1.0, (decltype(y)*)nullptr, 0.0);
    });
    report("ztrmv_lower_r", [] {
        blaze::LowerMatrix<blaze::DynamicMatrix<CD, rowMajor>> L(200);
        blaze::DynamicVector<CD> x(200), y;
        fill(L, 14); fillv(x, 15);
        y = L * x;
        return mv_diff(L, x, y, CD(1.0), (decltype(y)*)nullptr, CD(0.0));
    });
    report("zgemv_r", [] {
        blaze::DynamicMatrix<CD, rowMajor> A(300, 200);
        blaze::DynamicVector<CD> x(200), y;
        fill(A, 16); fillv(x, 17);
        y = A * x;
        return mv_diff(A, x, y, CD(1.0), (decltype(y)*)nullptr, CD(0.0));
    });
    report("zgemm_rr", [] {
        blaze::DynamicMatrix<CD, rowMajor> A(100, 90), C;
        blaze::DynamicMatrix<CD, columnMajor> B(90, 96);
        fill(A, 18); fill(B, 19);
        C = A * B;
        return mm_diff(A, B, C);
    });
    report("dtrmm_lower", [] {
        blaze::LowerMatrix<blaze::DynamicMatrix<double, rowMajor>> L(100);
        blaze::DynamicMatrix<double, rowMajor> B(100, 96), C;
        fill(L, 20); fill(B, 21);
        C = L * B;
        return mm_diff(L, B, C);
    });
    report("ztrmm_upper", [] {
        blaze::UpperMatrix<blaze::DynamicMatrix<CD, columnMajor>> U(100);
        blaze::DynamicMatrix<CD, columnMajor> B(100, 96), C;
        fill(U, 22); fill(B, 23);
        C = U * B;
        return mm_diff(U, B, C);
    });
    // Blaze's size gates (DMatDMatMultExpr.h:561-569): with the area threshold lowered
    // (-DBLAZE_DMATDMATMULT_THRESHOLD), a small product (M*N = 3840 < 4900) takes the BLAS kernel;
    // a product with B.columns() <= 10 SIMD widths stays in Blaze's small kernel (that gate is fixed).
    report("small_area", [] {
        blaze::DynamicMatrix<double, rowMajor> A(40, 30), B(30, 96), C;
        fill(A, 24); fill(B, 25);
        C = A * B;
        return mm_diff(A, B, C);
    });
    report("skinny_cpu", [] {
        blaze::DynamicMatrix<double, rowMajor> A(300, 30), B(30, 16), C;
        fill(A, 26); fill(B, 27);
        C = A * B;
        return mm_diff(A, B, C);
    });
    // blaze::dotu / dotc / axpy / trsm (blaze/math/blas/), the calls blazetest's BLAS operation
    // test makes (blazetest/mathtest/blas/OperationTest.h): 7-element vectors, 3 x 3 triangular
    // systems with one and with several right-hand sides, plus larger systems; a storage order of
    // B that differs from A's makes Blaze pass the transposed triangle (blaze/math/blas/trsm.h:195-199)
    report("dotu_d", [] {
        blaze::StaticVector<double, 7, blaze::rowVector> x;
        blaze::StaticVector<double, 7> y;
        fillv(x, 28); fillv(y, 29);
        const double r = blaze::dotu(x, y);
        double s = 0.0;
        for (size_t i = 0; i < 7; ++i) s += x[i] * y[i];
        return std::abs(r - s);
    });
    report("dotu_z", [] {
        blaze::StaticVector<CD, 7, blaze::rowVector> x;
        blaze::StaticVector<CD, 7> y;
        fillv(x, 30); fillv(y, 31);
        const CD r = blaze::dotu(x, y);
        CD s(0.0);
        for (size_t i = 0; i < 7; ++i) s += x[i] * y[i];
        return std::abs(r - s);
    });
    report("dotc_z", [] {
        blaze::StaticVector<CD, 7, blaze::rowVector> x;
        blaze::StaticVector<CD, 7> y;
        fillv(x, 32); fillv(y, 33);
        const CD r = blaze::dotc(x, y);
        CD s(0.0);
        for (size_t i = 0; i < 7; ++i) s += std::conj(x[i]) * y[i];
        return std::abs(r - s);
    });
    report("axpy_d", [] {
        blaze::StaticVector<double, 7, blaze::rowVector> x, y, y0;
        fillv(x, 34); fillv(y, 35);
        y0 = y;
        blaze::axpy(y, x, 0.75);
        double d = 0.0;
        for (size_t i = 0; i < 7; ++i) d = std::max(d, std::abs(y[i] - (y0[i] + 0.75 * x[i])));
        return d;
    });
    report("axpy_z", [] {
        blaze::DynamicVector<CD> x(500), y(500), y0;
        fillv(x, 36); fillv(y, 37);
        y0 = y;
        const CD al(0.5, -2.0);
        blaze::axpy(y, x, al);
        double d = 0.0;
        for (size_t i = 0; i < 500; ++i) d = std::max(d, std::abs(y[i] - (y0[i] + al * x[i])));
        return d;
    });
    report("trsm_lower_vec", [] {
        blaze::LowerMatrix<blaze::StaticMatrix<double, 3, 3, rowMajor>> A;
        fill(A, 38);
        for (size_t i = 0; i < 3; ++i) A(i, i) += 4.0;
        blaze::StaticVector<double, 3> b, x;
        fillv(b, 39);
        x = b;
        blaze::trsm(A, x, CblasLeft, CblasLower, 1.0);
        return mv_diff(A, x, b, 1.0, (decltype(b)*)nullptr, 0.0);
    });
    report("trsm_upper_right", [] {
        blaze::UpperMatrix<blaze::StaticMatrix<double, 3, 3, columnMajor>> A;
        fill(A, 40);
        for (size_t i = 0; i < 3; ++i) A(i, i) += 4.0;
        blaze::StaticMatrix<double, 3, 3, columnMajor> B, X;
        fill(B, 41);
        X = B;
        blaze::trsm(A, X, CblasRight, CblasUpper, 1.0);
        return mm_diff(X, A, B);
    });
    report("trsm_mixed", [] {  // A row-major, B column-major: the transposed triangle
        blaze::LowerMatrix<blaze::DynamicMatrix<double, rowMajor>> A(300);
        fill(A, 42);
        for (size_t i = 0; i < 300; ++i) A(i, i) += 300.0;
        blaze::DynamicMatrix<double, columnMajor> B(300, 24), X, B2;
        fill(B, 43);
        X = B;
        blaze::trsm(A, X, CblasLeft, CblasLower, 2.0);
        B2 = 2.0 * B;
        return mm_diff(A, X, B2);
    });
    report("ztrsm_lower", [] {
        blaze::LowerMatrix<blaze::DynamicMatrix<CD, rowMajor>> A(100);
        fill(A, 44);
        for (size_t i = 0; i < 100; ++i) A(i, i) += 100.0;
        blaze::DynamicMatrix<CD, rowMajor> B(100, 16), X, B2;
        fill(B, 45);
        X = B;
        const CD al(0.5, -1.0);
        blaze::trsm(A, X, CblasLeft, CblasLower, al);
        B2 = al * B;
        return mm_diff(A, X, B2);
    });
    return 0;
}
