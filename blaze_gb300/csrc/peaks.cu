// peaks.cu — arithmetic-rate probes used by the dispatcher and reported beside results.
//
// gb300_measure_fp64_peak runs independent DFMA chains on every SM and returns the sustained
// FP64 rate in TFLOP/s.  The automatic method choice (split-precision vs native FP64) compares
// predicted times with this measured rate instead of a datasheet figure.  gb300_measure_fp32_peak
// does the same with FFMA chains: the roofline of the native and grouped FP32 kernels.
#include <cuda_runtime.h>

#include <string>

#include "../../include/gb300_blas.h"
#include "runtime.h"

namespace gb {
namespace {

// independent multiply-add chains per thread: enough to cover the pipe latency with the warps an
// SM holds (the FP32 pipe retires four times the FP64 pipe's operations per clock)
template <typename T>
__host__ __device__ constexpr int chains() { return sizeof(T) == 8 ? 8 : 16; }

template <typename T>
__global__ void fma_chains(T* out, int iters, T y, T z) {
    constexpr int kChains = chains<T>();
    T x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = T(1) + T(1e-3) * T(threadIdx.x + c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], y, z);
    }
    T s = T(0);
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == T(12345.678)) out[blockIdx.x] = s;  // keeps the chains alive; never true in practice
}

template <typename T>
int measure_peak(double* tflops, const char* routine) {
    gb::Runtime& r = gb::runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = gb::ensure_init(&err);
    if (st != GB300_OK) {
        gb::set_error(st, std::string(routine) + ": " + err);
        return st;
    }
    T* d = static_cast<T*>(gb::pool_get(gb::kSlotMisc, 4096 * sizeof(double), &err));
    if (!d) {
        gb::set_error(GB300_ERR_NO_MEMORY, err);
        return GB300_ERR_NO_MEMORY;
    }
    const int blocks = r.num_sms * 8, threads = 256, iters = 4096;
    const T y = T(0.9999999), z = T(1e-7);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<T><<<blocks, threads, 0, r.stream>>>(d, 64, y, z);  // warm-up
    cudaEventRecord(e0, r.stream);
    fma_chains<T><<<blocks, threads, 0, r.stream>>>(d, iters, y, z);
    cudaEventRecord(e1, r.stream);
    gb::count_launches(2);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        gb::set_error(GB300_ERR_CUDA, std::string(routine) + ": " + cudaGetErrorString(e));
        return GB300_ERR_CUDA;
    }
    const double flops = 2.0 * double(blocks) * threads * iters * chains<T>();
    if (tflops) *tflops = flops / (double(ms) * 1e-3) / 1e12;
    return GB300_OK;
}

}  // namespace
}  // namespace gb

extern "C" int gb300_measure_fp32_peak(double* tflops) { return gb::measure_peak<float>(tflops, "gb300_measure_fp32_peak"); }

extern "C" int gb300_measure_fp64_peak(double* tflops) { return gb::measure_peak<double>(tflops, "gb300_measure_fp64_peak"); }
