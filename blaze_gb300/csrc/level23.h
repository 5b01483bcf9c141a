// level23.h — launchers of the ?gemv, complex ?gemm and ?trmm kernels (level23.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace gb {

// y = alpha * S x + beta * y (rows form, S rows x cols) or y = alpha * S^T x + beta * y (cols form:
// `slices` partial sums of row slices in `part`, slices * cols elements, then a fixed-order sum).
template <typename T>
cudaError_t launch_gemv(bool cols_form, int64_t rows, int64_t cols, T alpha, const T* S, int64_t ld, const T* x,
                        int64_t incx, T beta, T* y, int64_t incy, T* part, int slices, cudaStream_t st);

// Interleaved complex rows x cols (pitch ld in complex elements) -> dense real planes.
template <typename T>
cudaError_t launch_split_complex(int64_t rows, int64_t cols, const T* Z, int64_t ld, T* re, T* im, cudaStream_t st);

// C (interleaved, pitch ldc) = (ar + i ai) (Pr + i Pi) + (br + i bi) C.
template <typename T>
cudaError_t launch_complex_epilogue(int64_t rows, int64_t cols, const T* Pr, const T* Pi, T ar, T ai, T br, T bi, T* C,
                                   int64_t ldc, cudaStream_t st);

// Dense copy of the lower (or upper) triangle of the n x n row-major A, zeros elsewhere, ones on
// the diagonal when `unit`.
template <typename T>
cudaError_t launch_triangle(int64_t n, const T* A, int64_t lda, bool lower, bool unit, T* out, cudaStream_t st);

}  // namespace gb
