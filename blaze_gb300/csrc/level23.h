// level23.h — launchers of the kernels of the BLAS routines next to ?gemm: ?gemv / ?trmv, complex
// ?gemm and ?trmm (level23.cu), ?axpy and the dot products (level1.cu), ?trsm (trsm.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace gb {

// How a matrix x vector launch reads its operand S (rows x cols, row-major storage, pitch ld).
struct MvForm {
    bool cols_form = false;  // y = op(S)^T x (threads over columns, partial sums over row slices)
                             // instead of y = op(S) x (a warp per row)
    int tri = 0;             // 0: all of S; 1: lower triangle (j <= i); 2: upper triangle (j >= i)
    bool unit = false;       // the diagonal reads as one (S's diagonal is not read)
    bool conj = false;       // S's elements conjugated (complex only)
};

// y = alpha * S x + beta * y (rows form) or y = alpha * S^T x + beta * y (cols form: `slices`
// partial sums of row slices in `part`, slices * cols elements, then a fixed-order sum).  CPLX:
// elements are interleaved complex pairs of T, alpha / beta point at (re, im), ld / inc count
// complex elements and the complex pointers are 2 * sizeof(T)-aligned.  beta == 0: y is not read.
// Row slices of the cols form for an operand of rows x cols (enough blocks for two full waves);
// `part` then holds slices * cols elements.
template <typename T, bool CPLX>
int mv_cols_slices(int64_t rows, int64_t cols);

template <typename T, bool CPLX>
cudaError_t launch_mv(const MvForm& f, int64_t rows, int64_t cols, const T* alpha, const T* S, int64_t ld, const T* x,
                      int64_t incx, const T* beta, T* y, int64_t incy, T* part, int slices, cudaStream_t st);

// Interleaved complex rows x cols (pitch ld in complex elements) -> real planes re and im, each with
// pitch out_ld (side by side: im = re + cols, out_ld = 2 cols; one below the other: im = re +
// rows cols, out_ld = cols).
template <typename T>
cudaError_t launch_split_complex(int64_t rows, int64_t cols, const T* Z, int64_t ld, T* re, T* im, int64_t out_ld,
                                 cudaStream_t st);

// C (rows x cols, interleaved, pitch ldc) = alpha op(A) op(B) + beta C from the real product
// P = [op(Ar); op(Ai)] [op(Br), op(Bi)] (2 rows x 2 cols, pitch 2 cols) of the planes with the
// conjugations (conj_a, conj_b) not yet applied; alpha = (ar, ai), beta = (br, bi).
template <typename T>
cudaError_t launch_complex_quadrants(int64_t rows, int64_t cols, const T* P, bool conj_a, bool conj_b, T ar, T ai,
                                     T br, T bi, T* C, int64_t ldc, cudaStream_t st);

// Dense copy of the lower (or upper) triangle of the n x n row-major A, zeros elsewhere, ones on
// the diagonal when `unit` (CPLX: interleaved complex elements).
template <typename T, bool CPLX>
cudaError_t launch_triangle(int64_t n, const T* A, int64_t lda, bool lower, bool unit, T* out, cudaStream_t st);

// ---- level1.cu ---------------------------------------------------------------------------------
// y[i incy] += alpha x[i incx] for i < n (CPLX: interleaved complex, alpha points at (re, im)); the
// pointers address logical element 0.  incy == 0 applies the n updates to y[0] in order.
template <typename T, bool CPLX>
cudaError_t launch_axpy(int64_t n, const T* alpha, const T* x, int64_t incx, T* y, int64_t incy, cudaStream_t st);

// Block sums of a dot product of length n (the size of `part` in sums).
int dot_parts(int64_t n);

// out = sum_i op(x_i) y_i in double precision (one double, or re / im for CPLX), op = conjugation
// when CONJ, summed in a fixed order; `part` holds dot_parts(n) sums (two doubles each for CPLX).
template <typename T, bool CPLX, bool CONJ>
cudaError_t launch_dot(int64_t n, const T* x, int64_t incx, const T* y, int64_t incy, double* part, double* out,
                       cudaStream_t st);

// ---- trsm.cu -----------------------------------------------------------------------------------
// Rows of the diagonal blocks that a triangular solve inverts (its recursion's leaves) for elements
// of `elem` bytes: 512 for every element type; the inverse kernel's shared memory, (9 nb + 64)
// elements, stays below 75 KB even for complex double.  Larger leaves mean fewer, larger products
// for the same work: 512 rows instead of 256 made ztrsm 4096 5 % faster and halved its error.
constexpr int solve_block(size_t /*elem*/) { return 512; }

// X (rows x cols, pitch ld) = alpha X.
template <typename T, bool CPLX>
cudaError_t launch_scale(int64_t rows, int64_t cols, const T* alpha, T* X, int64_t ld, cudaStream_t st);

// Dense inverses of the diagonal blocks (nb x nb, nb a multiple of 32 up to solve_block(); the last
// block may be smaller) of the triangular op(SA): SA ka x ka in row-major storage, op = transpose
// (trans) and conjugation (conj), `upper` when op(SA) is upper triangular, `unit` for a unit
// diagonal (not read).  Block b's inverse goes to inv + b nb nb (pitch nb).
template <typename T, bool CPLX>
cudaError_t launch_tri_inverse(int64_t ka, int nb, const T* SA, int64_t lda, bool trans, bool conj, bool upper,
                               bool unit, T* inv, cudaStream_t st);

}  // namespace gb
