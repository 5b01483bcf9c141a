// peaks.cu — arithmetic-rate probes used by the dispatcher and reported beside results.
//
// gb300_measure_fp64_peak runs independent DFMA chains on every SM and returns the sustained
// FP64 rate in TFLOP/s.  The automatic method choice (split-precision vs native FP64) compares
// predicted times with this measured rate instead of a datasheet figure.
#include <cuda_runtime.h>

#include <string>

#include "../../include/gb300_blas.h"
#include "runtime.h"

namespace gb {
namespace {

constexpr int kChains = 8;

__global__ void dfma_chains(double* out, int iters, double y, double z) {
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = 1.0 + 1e-3 * (threadIdx.x + c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], y, z);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.678) out[blockIdx.x] = s;  // keeps the chains alive; never true in practice
}

}  // namespace
}  // namespace gb

extern "C" int gb300_measure_fp64_peak(double* tflops) {
    gb::Runtime& r = gb::runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = gb::ensure_init(&err);
    if (st != GB300_OK) {
        gb::set_error(st, "gb300_measure_fp64_peak: " + err);
        return st;
    }
    double* d = static_cast<double*>(gb::pool_get(gb::kSlotMisc, 4096 * sizeof(double), &err));
    if (!d) {
        gb::set_error(GB300_ERR_NO_MEMORY, err);
        return GB300_ERR_NO_MEMORY;
    }
    const int blocks = r.num_sms * 4, threads = 256, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    gb::dfma_chains<<<blocks, threads, 0, r.stream>>>(d, 64, 0.9999999, 1e-7);  // warm-up
    cudaEventRecord(e0, r.stream);
    gb::dfma_chains<<<blocks, threads, 0, r.stream>>>(d, iters, 0.9999999, 1e-7);
    cudaEventRecord(e1, r.stream);
    gb::count_launches(2);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        gb::set_error(GB300_ERR_CUDA, std::string("gb300_measure_fp64_peak: ") + cudaGetErrorString(e));
        return GB300_ERR_CUDA;
    }
    const double flops = 2.0 * double(blocks) * threads * iters * gb::kChains;
    if (tflops) *tflops = flops / (double(ms) * 1e-3) / 1e12;
    return GB300_OK;
}
