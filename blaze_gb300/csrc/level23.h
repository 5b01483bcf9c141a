// level23.h — launchers of the ?gemv / ?trmv, complex ?gemm and ?trmm kernels (level23.cu).
#pragma once

#include <cuda_runtime.h>

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

// Interleaved complex rows x cols (pitch ld in complex elements) -> dense real planes.
template <typename T>
cudaError_t launch_split_complex(int64_t rows, int64_t cols, const T* Z, int64_t ld, T* re, T* im, cudaStream_t st);

// C (interleaved, pitch ldc) = (ar + i ai) (Pr + i Pi) + (br + i bi) C.
template <typename T>
cudaError_t launch_complex_epilogue(int64_t rows, int64_t cols, const T* Pr, const T* Pi, T ar, T ai, T br, T bi, T* C,
                                   int64_t ldc, cudaStream_t st);

// Dense copy of the lower (or upper) triangle of the n x n row-major A, zeros elsewhere, ones on
// the diagonal when `unit` (CPLX: interleaved complex elements).
template <typename T, bool CPLX>
cudaError_t launch_triangle(int64_t n, const T* A, int64_t lda, bool lower, bool unit, T* out, cudaStream_t st);

}  // namespace gb
