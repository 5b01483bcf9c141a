// cplx.cuh — element arithmetic shared by the BLAS-routine kernels (level23.cu, level1.cu,
// trsm.cu): V = T (real) or Cx<T> (complex, interleaved re / im as CBLAS stores it).
#pragma once

#include <cuda_runtime.h>

namespace gb {

// Element arithmetic: V = T (real) or Cx<T> (complex, interleaved re / im).
template <typename T>
struct alignas(2 * sizeof(T)) Cx {
    T re, im;
};

template <typename V>
struct Ar {  // real
    __device__ static V zero() { return V(0); }
    __device__ static V one() { return V(1); }
    __device__ static V conj(V a) { return a; }
    __device__ static V fmadd(V a, V b, V c) { return fma(a, b, c); }
    __device__ static V fmadd_conj(V a, V b, V c) { return fma(a, b, c); }
    __device__ static V fnmadd(V a, V b, V c) { return fma(-a, b, c); }  // c - a * b
    __device__ static V div(V a, V b) { return a / b; }
    __device__ static V mul(V a, V b) { return a * b; }
    __device__ static V add(V a, V b) { return a + b; }
    __device__ static bool is_zero(V a) { return a == V(0); }
    __device__ static V shfl_xor(V a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
    // alpha * acc + beta * y, y not read when beta == 0
    __device__ static V axpby(V alpha, V acc, V beta, const V* y) {
        return is_zero(beta) ? alpha * acc : fma(beta, *y, alpha * acc);
    }
};

template <typename T>
struct Ar<Cx<T>> {  // complex
    using V = Cx<T>;
    __device__ static V zero() { return V{T(0), T(0)}; }
    __device__ static V one() { return V{T(1), T(0)}; }
    __device__ static V conj(V a) { return V{a.re, -a.im}; }
    __device__ static V fmadd(V a, V b, V c) {
        return V{fma(a.re, b.re, fma(-a.im, b.im, c.re)), fma(a.re, b.im, fma(a.im, b.re, c.im))};
    }
    // conj(a) * b + c with the sign folded into the FMAs (a negation would be one more FP64
    // instruction per element)
    __device__ static V fmadd_conj(V a, V b, V c) {
        return V{fma(a.re, b.re, fma(a.im, b.im, c.re)), fma(a.re, b.im, fma(-a.im, b.re, c.im))};
    }
    // c - a * b
    __device__ static V fnmadd(V a, V b, V c) {
        return V{fma(-a.re, b.re, fma(a.im, b.im, c.re)), fma(-a.re, b.im, fma(-a.im, b.re, c.im))};
    }
    // a / b by Smith's method (R. L. Smith, Algorithm 116, CACM 5(8), 1962): the ratio of the
    // smaller to the larger part of b keeps the intermediate products from overflowing
    __device__ static V div(V a, V b) {
        if (fabs(b.re) >= fabs(b.im)) {
            const T r = b.im / b.re, d = b.re + b.im * r;
            return V{(a.re + a.im * r) / d, (a.im - a.re * r) / d};
        }
        const T r = b.re / b.im, d = b.re * r + b.im;
        return V{(a.re * r + a.im) / d, (a.im * r - a.re) / d};
    }
    __device__ static V mul(V a, V b) { return V{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
    __device__ static V add(V a, V b) { return V{a.re + b.re, a.im + b.im}; }
    __device__ static bool is_zero(V a) { return a.re == T(0) && a.im == T(0); }
    __device__ static V shfl_xor(V a, int o) {
        return V{__shfl_xor_sync(0xffffffffu, a.re, o), __shfl_xor_sync(0xffffffffu, a.im, o)};
    }
    __device__ static V axpby(V alpha, V acc, V beta, const V* y) {
        const V t = mul(alpha, acc);
        return is_zero(beta) ? t : fmadd(beta, *y, t);
    }
};

}  // namespace gb
