// level1.cu — kernels of the vector routines on Blaze's seam: ?axpy (y += alpha x) and the dot
// products (?dot, ?dotu, ?dotc).  The host entries are in api_next.cpp.
//
// Vectors are given by the address of their logical element 0 and a stride in elements (negative
// strides were already folded into that address by the host, as CBLAS defines them).
//
// Both routines move every byte once: they are bound by HBM.  A double dot product does one FMA
// per 16 bytes read, and a complex double one does four per 32 bytes.  The GB300 FP64 pipe
// (measured 1.25 TFLOP/s) sustains that at about 10 TB/s and 5 TB/s, above the HBM rate.  Dot
// products reduce in a fixed order.  The grid is fixed by the length and the SM count, each block
// sums a contiguous chunk, and one block adds the block sums.  The same inputs therefore give the
// same bits on every call.  Float dot products are compensated (Dot2: T. Ogita, S. M. Rump,
// S. Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26(6), 2005).  Each product's
// rounding error comes from an FMA and each sum's from TwoSum, so the per-thread result is as
// accurate as one in twice the working precision.  The partial sums are then added in double.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "cplx.cuh"
#include "gb300_internal.h"
#include "level23.h"
#include "runtime.h"

namespace gb {
namespace {

// ---- axpy --------------------------------------------------------------------------------------
template <typename V>
__global__ void __launch_bounds__(256) axpy_kernel(int64_t n, V alpha, const V* __restrict__ x, int64_t incx,
                                                   V* __restrict__ y, int64_t incy) {
    const int64_t step = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += step) {
        V* yi = y + i * incy;
        *yi = Ar<V>::fmadd(alpha, x[i * incx], *yi);
    }
}

// incy == 0: every update lands on y[0], in order (as the reference loop does it).
template <typename V>
__global__ void axpy_serial_kernel(int64_t n, V alpha, const V* __restrict__ x, int64_t incx, V* __restrict__ y) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    V acc = *y;
    for (int64_t i = 0; i < n; ++i) acc = Ar<V>::fmadd(alpha, x[i * incx], acc);
    *y = acc;
}

// ---- dot products ------------------------------------------------------------------------------
// s + c += a * b, exactly up to the final rounding of c (Dot2's step).  The _rn intrinsics keep
// the compiler from contracting the error terms into FMAs, which would lose them.
__device__ __forceinline__ void dot2_step(float& s, float& c, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = fmaf(a, b, -p);  // a * b = p + e
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float q = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));  // s + p = t + q
    s = t;
    c = __fadd_rn(c, __fadd_rn(q, e));
}

// Per-thread accumulator of sum_i op(x_i) y_i (op = conjugation when CONJ); out() is the sum in
// double precision: double or Cx<double>.
template <typename V, bool CONJ>
struct DotAcc;
template <bool CONJ>
struct DotAcc<double, CONJ> {
    using W = double;
    double s = 0.0;
    __device__ void add(double a, double b) { s = fma(a, b, s); }
    __device__ W out() const { return s; }
};
template <bool CONJ>
struct DotAcc<float, CONJ> {
    using W = double;
    float s = 0.f, c = 0.f;
    __device__ void add(float a, float b) { dot2_step(s, c, a, b); }
    __device__ W out() const { return double(s) + double(c); }
};
template <bool CONJ>
struct DotAcc<Cx<double>, CONJ> {
    using W = Cx<double>;
    W s{0.0, 0.0};
    __device__ void add(W a, W b) { s = CONJ ? Ar<W>::fmadd_conj(a, b, s) : Ar<W>::fmadd(a, b, s); }
    __device__ W out() const { return s; }
};
template <bool CONJ>
struct DotAcc<Cx<float>, CONJ> {
    using W = Cx<double>;
    float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
    // op(a) b with op(a) = conj(a) when CONJ:  re = ar br -+ ai bi,  im = ar bi +- ai br
    __device__ void add(Cx<float> a, Cx<float> b) {
        dot2_step(sr, cr, a.re, b.re);
        dot2_step(sr, cr, CONJ ? a.im : -a.im, b.im);
        dot2_step(si, ci, a.re, b.im);
        dot2_step(si, ci, CONJ ? -a.im : a.im, b.re);
    }
    __device__ W out() const { return W{double(sr) + double(cr), double(si) + double(ci)}; }
};

// Sum of v over the 256 threads of the block in a fixed order (shuffle tree per warp, then the
// eight warp sums by warp 0); the result is valid in thread 0.
template <typename W>
__device__ W block_sum_256(W v) {
    __shared__ W warp_sums[8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = Ar<W>::add(v, Ar<W>::shfl_xor(v, o));
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < 8 ? warp_sums[threadIdx.x] : Ar<W>::zero();
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) v = Ar<W>::add(v, Ar<W>::shfl_xor(v, o));
    }
    return v;
}

// Elements per 16-byte group of a contiguous vector.
template <typename V>
__host__ __device__ constexpr int dot_group() { return sizeof(V) >= 16 ? 1 : int(16 / sizeof(V)); }

// part[b] = sum over i in [b chunk, (b + 1) chunk) of op(x_i) y_i.  Contiguous vectors go in groups
// of G = 16 / sizeof(V) elements: thread t takes groups t, t + 256, ... of its block's chunk (chunk
// a multiple of G), loaded as one 16-byte vector each when both vectors are 16-byte aligned (VEC)
// and element by element otherwise, in the same order, so the sum's bits do not depend on the
// alignment.
template <typename V, bool CONJ, bool VEC>
__global__ void __launch_bounds__(256) dot_partial_kernel(int64_t n, const V* __restrict__ x, int64_t incx,
                                                          const V* __restrict__ y, int64_t incy, int64_t chunk,
                                                          typename DotAcc<V, CONJ>::W* __restrict__ part) {
    constexpr int G = dot_group<V>();
    struct alignas(16) Group {
        V v[G];
    };
    DotAcc<V, CONJ> acc;
    const int64_t i0 = int64_t(blockIdx.x) * chunk, i1 = min(n, i0 + chunk);
    if (incx == 1 && incy == 1) {
        int64_t i = i0 + int64_t(threadIdx.x) * G;
        for (; i + G <= i1; i += 256 * G) {
            if (VEC) {
                const Group a = *reinterpret_cast<const Group*>(x + i), b = *reinterpret_cast<const Group*>(y + i);
#pragma unroll
                for (int w = 0; w < G; ++w) acc.add(a.v[w], b.v[w]);
            } else {
#pragma unroll
                for (int w = 0; w < G; ++w) acc.add(x[i + w], y[i + w]);
            }
        }
        for (; i < i1; ++i) acc.add(x[i], y[i]);  // the ragged end of the last group
    } else {
        for (int64_t i = i0 + threadIdx.x; i < i1; i += 256) acc.add(x[i * incx], y[i * incy]);
    }
    const auto s = block_sum_256(acc.out());
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// out[0] = sum of part[0 .. nparts) in a fixed order.
template <typename W>
__global__ void __launch_bounds__(256) dot_final_kernel(int nparts, const W* __restrict__ part, W* __restrict__ out) {
    W v = Ar<W>::zero();
    for (int i = threadIdx.x; i < nparts; i += 256) v = Ar<W>::add(v, part[i]);
    v = block_sum_256(v);
    if (threadIdx.x == 0) out[0] = v;
}

}  // namespace

template <typename T, bool CPLX>
cudaError_t launch_axpy(int64_t n, const T* alpha, const T* x, int64_t incx, T* y, int64_t incy, cudaStream_t st) {
    using V = typename std::conditional<CPLX, Cx<T>, T>::type;
    V al;
    std::memcpy(&al, alpha, sizeof(V));
    const V* vx = reinterpret_cast<const V*>(x);
    V* vy = reinterpret_cast<V*>(y);
    if (incy == 0) {
        axpy_serial_kernel<V><<<1, 32, 0, st>>>(n, al, vx, incx, vy);
    } else {
        const int64_t blocks = std::min<int64_t>((n + 255) / 256, int64_t(runtime().num_sms) * 16);
        axpy_kernel<V><<<unsigned(std::max<int64_t>(1, blocks)), 256, 0, st>>>(n, al, vx, incx, vy, incy);
    }
    count_launches(1);
    return cudaGetLastError();
}

int dot_parts(int64_t n) {
    // at least 2048 elements per block, at most eight blocks per SM
    const int64_t b = (n + 2047) / 2048;
    return int(std::max<int64_t>(1, std::min<int64_t>(b, int64_t(runtime().num_sms) * 8)));
}

template <typename T, bool CPLX, bool CONJ>
cudaError_t launch_dot(int64_t n, const T* x, int64_t incx, const T* y, int64_t incy, double* part, double* out,
                       cudaStream_t st) {
    using V = typename std::conditional<CPLX, Cx<T>, T>::type;
    using W = typename DotAcc<V, CONJ>::W;
    constexpr int G = dot_group<V>();
    const int parts = dot_parts(n);
    const int64_t chunk = ((n + parts - 1) / parts + G - 1) / G * G;
    const bool vec = incx == 1 && incy == 1 && (reinterpret_cast<uintptr_t>(x) % 16) == 0 &&
                     (reinterpret_cast<uintptr_t>(y) % 16) == 0;
    auto kern = vec ? dot_partial_kernel<V, CONJ, true> : dot_partial_kernel<V, CONJ, false>;
    const int blocks = int((n + chunk - 1) / chunk);
    kern<<<unsigned(blocks), 256, 0, st>>>(n, reinterpret_cast<const V*>(x), incx, reinterpret_cast<const V*>(y), incy,
                                           chunk, reinterpret_cast<W*>(part));
    dot_final_kernel<W><<<1, 256, 0, st>>>(blocks, reinterpret_cast<const W*>(part), reinterpret_cast<W*>(out));
    count_launches(2);
    return cudaGetLastError();
}

template cudaError_t launch_axpy<double, false>(int64_t, const double*, const double*, int64_t, double*, int64_t,
                                                cudaStream_t);
template cudaError_t launch_axpy<float, false>(int64_t, const float*, const float*, int64_t, float*, int64_t,
                                               cudaStream_t);
template cudaError_t launch_axpy<double, true>(int64_t, const double*, const double*, int64_t, double*, int64_t,
                                               cudaStream_t);
template cudaError_t launch_axpy<float, true>(int64_t, const float*, const float*, int64_t, float*, int64_t,
                                              cudaStream_t);
#define GB_DOT(T, C, J)                                                                                        \
    template cudaError_t launch_dot<T, C, J>(int64_t, const T*, int64_t, const T*, int64_t, double*, double*, \
                                             cudaStream_t);
GB_DOT(double, false, false)
GB_DOT(float, false, false)
GB_DOT(double, true, false)
GB_DOT(double, true, true)
GB_DOT(float, true, false)
GB_DOT(float, true, true)
#undef GB_DOT

}  // namespace gb
