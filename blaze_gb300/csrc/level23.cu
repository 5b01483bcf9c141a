// level23.cu — kernels of the BLAS routines next to ?gemm on Blaze's seam: ?gemv and ?trmv (matrix x
// vector, real or complex, a triangle optionally masked), complex ?gemm (one real product of the
// stacked real / imaginary planes, recombined from its quadrants) and ?trmm (triangular product
// through a masked copy of the triangle).  The host entries are in api_next.cpp.
//
// Matrix operands are described in row-major storage (rows x cols, pitch ld); a column-major
// CBLAS operand is the transpose of its row-major storage, which the host folds into the
// transposition flags.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "gb300_internal.h"
#include "cplx.cuh"
#include "level23.h"
#include "runtime.h"

namespace gb {
namespace {

// ---- matrix x vector (gemv, trmv) ------------------------------------------------------------
// acc + op(S[i][j]) * xv for the element at p: one on a unit diagonal (the diagonal's value is not
// used), conjugated for a conjugate transpose.
template <typename V, bool CONJ>
__device__ __forceinline__ V mv_step(const V* __restrict__ p, bool diag_one, V xv, V acc) {
    // select the operand, then one FMA: a branch between an add and an FMA would have both
    // evaluated, doubling the FP64 instructions
    const V a = diag_one ? Ar<V>::one() : *p;
    return CONJ ? Ar<V>::fmadd_conj(a, xv, acc) : Ar<V>::fmadd(a, xv, acc);
}

// y[i] = alpha * sum_j S[i][j] x[j] + beta * y[i] for i < rows: one warp per row, lanes stride over
// the row (coalesced; pointers step, no index products per element), a shuffle reduction.
// tri = 1 (lower) keeps j <= i, tri = 2 (upper) j >= i.  FP64 data is bound by the FP64 pipe here
// (one FMA per 8-byte element, four per 16-byte complex element), not by HBM; a single
// accumulator per lane keeps the registers low and the occupancy high, which measured faster than
// unrolled partial sums or several warps per row.
template <typename V, bool CONJ>
__global__ void __launch_bounds__(256) mv_rows_kernel(int64_t rows, int64_t cols, V alpha, const V* __restrict__ S,
                                                      int64_t ld, const V* __restrict__ x, int64_t incx, V beta,
                                                      V* __restrict__ y, int64_t incy, int tri, int unit) {
    using A = Ar<V>;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    const int64_t xstep = 32 * incx;
    for (int64_t i = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; i < rows; i += warps) {
        const int64_t j0 = tri == 2 ? i : 0, j1 = tri == 1 ? min(cols, i + 1) : cols;
        V acc = A::zero();
        const V* sp = S + i * ld + j0 + lane;
        const V* xp = x + (j0 + lane) * incx;
        // unrolled (still one chain per lane, summed in order) so that the next steps' loads issue
        // ahead of this step's FMA: 2 % faster at 16384 x 8192
#pragma unroll 4
        for (int64_t j = j0 + lane; j < j1; j += 32, sp += 32, xp += xstep)
            acc = mv_step<V, CONJ>(sp, unit && j == i, *xp, acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc = A::add(acc, A::shfl_xor(acc, o));
        if (lane == 0) {
            V* yi = y + i * incy;
            *yi = A::axpby(alpha, acc, beta, yi);
        }
    }
}

// Partial column sums: part[s][j] = sum_{i in slice s} S[i][j] x[i] for j < cols, threads over j
// (coalesced), slice s of the rows per blockIdx.y; tri = 1 (lower) keeps i >= j, tri = 2 (upper)
// i <= j.
template <typename V, bool CONJ>
__global__ void __launch_bounds__(256) mv_cols_partial_kernel(int64_t rows, int64_t cols, const V* __restrict__ S,
                                                              int64_t ld, const V* __restrict__ x, int64_t incx,
                                                              int64_t rows_per_slice, V* __restrict__ part, int tri,
                                                              int unit) {
    using A = Ar<V>;
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    int64_t i0 = int64_t(blockIdx.y) * rows_per_slice, i1 = min(rows, i0 + rows_per_slice);
    if (tri == 1) i0 = max(i0, j);
    if (tri == 2) i1 = min(i1, j + 1);
    V acc = A::zero();
    const V* sp = S + i0 * ld + j;
    const V* xp = x + i0 * incx;
#pragma unroll 4
    for (int64_t i = i0; i < i1; ++i, sp += ld, xp += incx) acc = mv_step<V, CONJ>(sp, unit && i == j, *xp, acc);
    part[int64_t(blockIdx.y) * cols + j] = acc;
}

// y[j] = alpha * sum_s part[s][j] + beta * y[j]: 32 columns per block, eight threads per column
// each summing every eighth slice, then the eight sums in a fixed order (deterministic).
template <typename V>
__global__ void __launch_bounds__(256) mv_cols_reduce_kernel(int64_t cols, int slices, const V* __restrict__ part,
                                                             V alpha, V beta, V* __restrict__ y, int64_t incy) {
    using A = Ar<V>;
    __shared__ V red[8][32];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int64_t j = int64_t(blockIdx.x) * 32 + tx;
    V acc = A::zero();
    if (j < cols)
        for (int s = ty; s < slices; s += 8) acc = A::add(acc, part[int64_t(s) * cols + j]);
    red[ty][tx] = acc;
    __syncthreads();
    if (ty == 0 && j < cols) {
        V t = red[0][tx];
#pragma unroll
        for (int w = 1; w < 8; ++w) t = A::add(t, red[w][tx]);
        V* yj = y + j * incy;
        *yj = A::axpby(alpha, t, beta, yj);
    }
}

// ---- complex planes --------------------------------------------------------------------------
// The element-wise kernels below take rows on blockIdx.y (striding by gridDim.y) and columns on
// threads (striding by the grid's x extent): no index division per element.

// Interleaved complex rows x cols (pitch ld, in complex elements) -> real planes re, im (pitch
// out_ld each; the caller places them side by side or one below the other).
template <typename T>
__global__ void split_complex_kernel(int64_t rows, int64_t cols, const T* __restrict__ Z, int64_t ld,
                                     T* __restrict__ re, T* __restrict__ im, int64_t out_ld) {
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y)
        for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < cols; c += int64_t(gridDim.x) * blockDim.x) {
            const T* z = Z + 2 * (r * ld + c);
            re[r * out_ld + c] = z[0];
            im[r * out_ld + c] = z[1];
        }
}

// C (rows x cols interleaved, pitch ldc) = alpha (Re + i Im) + beta C from the quadrants of the real
// product P = [op(Ar); op(Ai)] [op(Br), op(Bi)] (2 rows x 2 cols, pitch 2 cols):
// Re = P00 - SAB P11 and Im = SB (P01 + SAB P10), where SB = -1 conjugates B and SAB = -1 when
// exactly one operand is conjugated.  The signs are template arguments, so each combination is one
// FP64 add; with alpha = 1 and beta = 0 (what Blaze passes) nothing else is computed.
template <typename T, int SAB, int SB>
__global__ void complex_quadrant_kernel(int64_t rows, int64_t cols, const T* __restrict__ P, T ar, T ai, T br, T bi,
                                        T* __restrict__ C, int64_t ldc) {
    const bool plain = ar == T(1) && ai == T(0) && br == T(0) && bi == T(0);
    const bool beta0 = br == T(0) && bi == T(0);
    const int64_t ldp = 2 * cols, cstep = int64_t(gridDim.x) * blockDim.x;
    const int64_t c0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y) {
        const T* p0 = P + r * ldp;           // P00 | P01
        const T* p1 = P + (r + rows) * ldp;  // P10 | P11
        for (int64_t c = c0; c < cols; c += cstep) {
            const T re = SAB > 0 ? p0[c] - p1[cols + c] : p0[c] + p1[cols + c];
            const T s = SAB > 0 ? p0[cols + c] + p1[c] : p0[cols + c] - p1[c];
            const T im = SB > 0 ? s : -s;
            T* z = C + 2 * (r * ldc + c);
            if (plain) {
                z[0] = re;
                z[1] = im;
                continue;
            }
            T cr = ar * re - ai * im, ci = ar * im + ai * re;
            if (!beta0) {
                const T zr = z[0], zi = z[1];
                cr += br * zr - bi * zi;
                ci += br * zi + bi * zr;
            }
            z[0] = cr;
            z[1] = ci;
        }
    }
}

// ---- triangle --------------------------------------------------------------------------------
// T (dense n x n, pitch n) = the `lower` (or upper) triangle of A (n x n, pitch lda, row-major
// storage) with zeros elsewhere and ones on the diagonal when `unit`.
template <typename V>
__global__ void triangle_kernel(int64_t n, const V* __restrict__ A, int64_t lda, int lower, int unit,
                                V* __restrict__ out) {
    for (int64_t i = blockIdx.y; i < n; i += gridDim.y)
        for (int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += int64_t(gridDim.x) * blockDim.x) {
            const bool in = lower ? (j <= i) : (j >= i);
            out[i * n + j] = !in ? Ar<V>::zero() : ((unit && i == j) ? Ar<V>::one() : A[i * lda + j]);
        }
}

// Grid of the element-wise kernels: 256-thread blocks over the columns, rows on y, about 16 blocks
// per SM in all (each block strides over many rows).
dim3 grid_2d(int64_t rows, int64_t cols) {
    const int64_t x = std::max<int64_t>(1, std::min<int64_t>((cols + 255) / 256, 64));
    const int64_t y = std::max<int64_t>(1, std::min<int64_t>(rows, int64_t(runtime().num_sms) * 16 / x));
    return dim3(unsigned(x), unsigned(y));
}

// Blocks for `work` threads of `threads` per block, at most `per_sm` blocks per SM (grid-stride
// loops take the rest).
unsigned grid_for(int64_t work, int threads, int num_sms, int per_sm = 16) {
    const int64_t b = (work + threads - 1) / threads;
    return unsigned(std::max<int64_t>(1, std::min<int64_t>(b, int64_t(num_sms) * per_sm)));
}

}  // namespace

template <typename T, bool CPLX>
int mv_cols_slices(int64_t rows, int64_t) {
    // slices of at least 64 rows, at most 128 of them (measured on 8192- and 16384-row operands:
    // 128 slices beat 32 or 64 by 5 %, 256 gained nothing more)
    return int(std::max<int64_t>(1, std::min<int64_t>(128, rows / 64)));
}

template <typename T, bool CPLX>
cudaError_t launch_mv(const MvForm& f, int64_t rows, int64_t cols, const T* alpha, const T* S, int64_t ld, const T* x,
                      int64_t incx, const T* beta, T* y, int64_t incy, T* part, int slices, cudaStream_t st) {
    using V = typename std::conditional<CPLX, Cx<T>, T>::type;
    Runtime& r = runtime();
    V al, be;
    std::memcpy(&al, alpha, sizeof(V));
    std::memcpy(&be, beta, sizeof(V));
    const V* vS = reinterpret_cast<const V*>(S);
    const V* vx = reinterpret_cast<const V*>(x);
    V* vy = reinterpret_cast<V*>(y);
    const int tri = f.tri, unit = f.unit ? 1 : 0;
    const bool conj = CPLX && f.conj;
    if (!f.cols_form) {
        auto kern = conj ? mv_rows_kernel<V, CPLX> : mv_rows_kernel<V, false>;
        kern<<<grid_for(rows * 32, 256, r.num_sms, 8), 256, 0, st>>>(rows, cols, al, vS, ld, vx, incx, be, vy, incy, tri,
                                                                      unit);
        count_launches(1);
    } else {
        V* vp = reinterpret_cast<V*>(part);
        const int64_t per = (rows + slices - 1) / slices;
        auto kern = conj ? mv_cols_partial_kernel<V, CPLX> : mv_cols_partial_kernel<V, false>;
        kern<<<dim3(unsigned((cols + 255) / 256), unsigned(slices)), 256, 0, st>>>(rows, cols, vS, ld, vx, incx, per, vp,
                                                                                  tri, unit);
        mv_cols_reduce_kernel<V><<<unsigned((cols + 31) / 32), 256, 0, st>>>(cols, slices, vp, al, be, vy, incy);
        count_launches(2);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_split_complex(int64_t rows, int64_t cols, const T* Z, int64_t ld, T* re, T* im, int64_t out_ld,
                                 cudaStream_t st) {
    split_complex_kernel<T><<<grid_2d(rows, cols), 256, 0, st>>>(rows, cols, Z, ld, re, im, out_ld);
    count_launches(1);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_complex_quadrants(int64_t rows, int64_t cols, const T* P, bool conj_a, bool conj_b, T ar, T ai,
                                     T br, T bi, T* C, int64_t ldc, cudaStream_t st) {
    const dim3 grid = grid_2d(rows, cols);
    const bool sab_pos = conj_a == conj_b;
    if (sab_pos && !conj_b)
        complex_quadrant_kernel<T, 1, 1><<<grid, 256, 0, st>>>(rows, cols, P, ar, ai, br, bi, C, ldc);
    else if (sab_pos)
        complex_quadrant_kernel<T, 1, -1><<<grid, 256, 0, st>>>(rows, cols, P, ar, ai, br, bi, C, ldc);
    else if (!conj_b)
        complex_quadrant_kernel<T, -1, 1><<<grid, 256, 0, st>>>(rows, cols, P, ar, ai, br, bi, C, ldc);
    else
        complex_quadrant_kernel<T, -1, -1><<<grid, 256, 0, st>>>(rows, cols, P, ar, ai, br, bi, C, ldc);
    count_launches(1);
    return cudaGetLastError();
}

template <typename T, bool CPLX>
cudaError_t launch_triangle(int64_t n, const T* A, int64_t lda, bool lower, bool unit, T* out, cudaStream_t st) {
    using V = typename std::conditional<CPLX, Cx<T>, T>::type;
    triangle_kernel<V><<<grid_2d(n, n), 256, 0, st>>>(n, reinterpret_cast<const V*>(A), lda, lower ? 1 : 0,
                                                        unit ? 1 : 0, reinterpret_cast<V*>(out));
    count_launches(1);
    return cudaGetLastError();
}

#define GB_MV(T, C)                                                                                          \
    template cudaError_t launch_mv<T, C>(const MvForm&, int64_t, int64_t, const T*, const T*, int64_t, const T*, \
                                         int64_t, const T*, T*, int64_t, T*, int, cudaStream_t);                \
    template cudaError_t launch_triangle<T, C>(int64_t, const T*, int64_t, bool, bool, T*, cudaStream_t);         \
    template int mv_cols_slices<T, C>(int64_t, int64_t);
GB_MV(double, false)
GB_MV(double, true)
GB_MV(float, false)
GB_MV(float, true)
#undef GB_MV
template cudaError_t launch_split_complex<double>(int64_t, int64_t, const double*, int64_t, double*, double*, int64_t,
                                                  cudaStream_t);
template cudaError_t launch_split_complex<float>(int64_t, int64_t, const float*, int64_t, float*, float*, int64_t,
                                                 cudaStream_t);
template cudaError_t launch_complex_quadrants<double>(int64_t, int64_t, const double*, bool, bool, double, double,
                                                     double, double, double*, int64_t, cudaStream_t);
template cudaError_t launch_complex_quadrants<float>(int64_t, int64_t, const float*, bool, bool, float, float, float,
                                                    float, float*, int64_t, cudaStream_t);

}  // namespace gb
