// level23.cu — kernels of the BLAS routines next to ?gemm on Blaze's seam: ?gemv (matrix x vector),
// complex ?gemm (four real products over split real / imaginary planes) and ?trmm (triangular
// product through a masked copy of the triangle).  The host entries are in api_next.cpp.
//
// Matrix operands are described in row-major storage (rows x cols, pitch ld); a column-major
// CBLAS operand is the transpose of its row-major storage, which the host folds into the
// transposition flags.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "gb300_internal.h"
#include "level23.h"
#include "runtime.h"

namespace gb {
namespace {

// ---- gemv ------------------------------------------------------------------------------------
// y[i] = alpha * sum_j S[i][j] x[j] + beta * y[i] for i < rows: one warp per row, lanes stride over
// the row (coalesced), a shuffle reduction, FP64 (or FP32) accumulation in the element type.
template <typename T>
__global__ void gemv_rows_kernel(int64_t rows, int64_t cols, T alpha, const T* __restrict__ S, int64_t ld,
                                 const T* __restrict__ x, int64_t incx, T beta, T* __restrict__ y, int64_t incy) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; i < rows; i += warps) {
        const T* row = S + i * ld;
        T acc = T(0);
        for (int64_t j = lane; j < cols; j += 32) acc = fma(row[j], x[j * incx], acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            T* yi = y + i * incy;
            *yi = (beta == T(0)) ? alpha * acc : fma(beta, *yi, alpha * acc);
        }
    }
}

// Partial column sums: part[s][j] = sum_{i in slice s} S[i][j] x[i] for j < cols, threads over j
// (coalesced), slice s of the rows per blockIdx.y.
template <typename T>
__global__ void gemv_cols_partial_kernel(int64_t rows, int64_t cols, const T* __restrict__ S, int64_t ld,
                                         const T* __restrict__ x, int64_t incx, int64_t rows_per_slice,
                                         T* __restrict__ part) {
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    const int64_t i0 = int64_t(blockIdx.y) * rows_per_slice, i1 = min(rows, i0 + rows_per_slice);
    T acc = T(0);
    for (int64_t i = i0; i < i1; ++i) acc = fma(S[i * ld + j], x[i * incx], acc);
    part[int64_t(blockIdx.y) * cols + j] = acc;
}

// y[j] = alpha * sum_s part[s][j] + beta * y[j] (slices summed in a fixed order: deterministic).
template <typename T>
__global__ void gemv_cols_reduce_kernel(int64_t cols, int slices, const T* __restrict__ part, T alpha, T beta,
                                        T* __restrict__ y, int64_t incy) {
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    T acc = T(0);
    for (int s = 0; s < slices; ++s) acc += part[int64_t(s) * cols + j];
    T* yj = y + j * incy;
    *yj = (beta == T(0)) ? alpha * acc : fma(beta, *yj, alpha * acc);
}

// ---- complex planes --------------------------------------------------------------------------
// Interleaved complex rows x cols (pitch ld, in complex elements) -> dense real planes re, im.
template <typename T>
__global__ void split_complex_kernel(int64_t rows, int64_t cols, const T* __restrict__ Z, int64_t ld,
                                     T* __restrict__ re, T* __restrict__ im) {
    const int64_t total = rows * cols;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t r = e / cols, c = e - r * cols;
        const T* z = Z + 2 * (r * ld + c);
        re[e] = z[0];
        im[e] = z[1];
    }
}

// C (interleaved, pitch ldc) = alpha * (Pr + i Pi) + beta * C for rows x cols (P dense).
template <typename T>
__global__ void complex_epilogue_kernel(int64_t rows, int64_t cols, const T* __restrict__ Pr, const T* __restrict__ Pi,
                                       T ar, T ai, T br, T bi, T* __restrict__ C, int64_t ldc) {
    const int64_t total = rows * cols;
    const bool beta0 = (br == T(0) && bi == T(0));
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t r = e / cols, c = e - r * cols;
        T* z = C + 2 * (r * ldc + c);
        const T pr = Pr[e], pi = Pi[e];
        T cr = ar * pr - ai * pi, ci = ar * pi + ai * pr;
        if (!beta0) {
            const T zr = z[0], zi = z[1];
            cr += br * zr - bi * zi;
            ci += br * zi + bi * zr;
        }
        z[0] = cr;
        z[1] = ci;
    }
}

// ---- triangle --------------------------------------------------------------------------------
// T (dense n x n, pitch n) = the `lower` (or upper) triangle of A (n x n, pitch lda, row-major
// storage) with zeros elsewhere and ones on the diagonal when `unit`.
template <typename T>
__global__ void triangle_kernel(int64_t n, const T* __restrict__ A, int64_t lda, int lower, int unit,
                                T* __restrict__ out) {
    const int64_t total = n * n;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i = e / n, j = e - i * n;
        const bool in = lower ? (j <= i) : (j >= i);
        out[e] = !in ? T(0) : ((unit && i == j) ? T(1) : A[i * lda + j]);
    }
}

unsigned grid_for(int64_t work, int threads, int num_sms) {
    const int64_t b = (work + threads - 1) / threads;
    return unsigned(std::max<int64_t>(1, std::min<int64_t>(b, int64_t(num_sms) * 16)));
}

}  // namespace

template <typename T>
cudaError_t launch_gemv(bool cols_form, int64_t rows, int64_t cols, T alpha, const T* S, int64_t ld, const T* x,
                        int64_t incx, T beta, T* y, int64_t incy, T* part, int slices, cudaStream_t st) {
    Runtime& r = runtime();
    if (!cols_form) {
        gemv_rows_kernel<T><<<grid_for(rows * 32, 256, r.num_sms), 256, 0, st>>>(rows, cols, alpha, S, ld, x, incx,
                                                                                beta, y, incy);
        count_launches(1);
    } else {
        const int64_t per = (rows + slices - 1) / slices;
        gemv_cols_partial_kernel<T><<<dim3(unsigned((cols + 255) / 256), unsigned(slices)), 256, 0, st>>>(
            rows, cols, S, ld, x, incx, per, part);
        gemv_cols_reduce_kernel<T><<<unsigned((cols + 255) / 256), 256, 0, st>>>(cols, slices, part, alpha, beta, y,
                                                                                   incy);
        count_launches(2);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_split_complex(int64_t rows, int64_t cols, const T* Z, int64_t ld, T* re, T* im, cudaStream_t st) {
    split_complex_kernel<T><<<grid_for(rows * cols, 256, runtime().num_sms), 256, 0, st>>>(rows, cols, Z, ld, re, im);
    count_launches(1);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_complex_epilogue(int64_t rows, int64_t cols, const T* Pr, const T* Pi, T ar, T ai, T br, T bi, T* C,
                                   int64_t ldc, cudaStream_t st) {
    complex_epilogue_kernel<T><<<grid_for(rows * cols, 256, runtime().num_sms), 256, 0, st>>>(rows, cols, Pr, Pi, ar,
                                                                                             ai, br, bi, C, ldc);
    count_launches(1);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_triangle(int64_t n, const T* A, int64_t lda, bool lower, bool unit, T* out, cudaStream_t st) {
    triangle_kernel<T><<<grid_for(n * n, 256, runtime().num_sms), 256, 0, st>>>(n, A, lda, lower ? 1 : 0, unit ? 1 : 0,
                                                                               out);
    count_launches(1);
    return cudaGetLastError();
}

template cudaError_t launch_gemv<double>(bool, int64_t, int64_t, double, const double*, int64_t, const double*,
                                         int64_t, double, double*, int64_t, double*, int, cudaStream_t);
template cudaError_t launch_gemv<float>(bool, int64_t, int64_t, float, const float*, int64_t, const float*, int64_t,
                                        float, float*, int64_t, float*, int, cudaStream_t);
template cudaError_t launch_split_complex<double>(int64_t, int64_t, const double*, int64_t, double*, double*,
                                                  cudaStream_t);
template cudaError_t launch_split_complex<float>(int64_t, int64_t, const float*, int64_t, float*, float*,
                                                 cudaStream_t);
template cudaError_t launch_complex_epilogue<double>(int64_t, int64_t, const double*, const double*, double, double,
                                                     double, double, double*, int64_t, cudaStream_t);
template cudaError_t launch_complex_epilogue<float>(int64_t, int64_t, const float*, const float*, float, float, float,
                                                    float, float*, int64_t, cudaStream_t);
template cudaError_t launch_triangle<double>(int64_t, const double*, int64_t, bool, bool, double*, cudaStream_t);
template cudaError_t launch_triangle<float>(int64_t, const float*, int64_t, bool, bool, float*, cudaStream_t);

}  // namespace gb
