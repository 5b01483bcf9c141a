// profile.h — optional CUDA-event timing of the library's dominant kernels (benchmarks).
#pragma once

#include <cuda_runtime.h>

namespace gb {

// Scope that records an event pair on `stream` around the kernel launched inside it when
// profiling is enabled (gb300_profile_enable); a no-op otherwise.
class KernelTimer {
  public:
    KernelTimer(const char* name, cudaStream_t stream);
    ~KernelTimer();

  private:
    int slot_ = -1;
    cudaStream_t stream_;
};

}  // namespace gb
