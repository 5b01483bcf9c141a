// profile.cpp — CUDA-event timing of the dominant kernels, read back by gb300_profile_read.
#include "profile.h"

#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gb300_blas.h"
#include "runtime.h"

namespace gb {
namespace {

struct Record {
    cudaEvent_t start = nullptr, stop = nullptr;
    std::string name;
    bool used = false;
};

std::atomic<bool> g_on{false};
std::mutex g_mu;
std::vector<Record> g_recs;

}  // namespace

KernelTimer::KernelTimer(const char* name, cudaStream_t stream) : stream_(stream) {
    if (!g_on.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lock(g_mu);
    for (size_t i = 0; i < g_recs.size(); ++i)
        if (!g_recs[i].used) { slot_ = int(i); break; }
    if (slot_ < 0) {
        if (g_recs.size() >= 65536) return;
        Record r;
        if (cudaEventCreate(&r.start) != cudaSuccess || cudaEventCreate(&r.stop) != cudaSuccess) return;
        g_recs.push_back(r);
        slot_ = int(g_recs.size() - 1);
    }
    g_recs[slot_].used = true;
    g_recs[slot_].name = name;
    cudaEventRecord(g_recs[slot_].start, stream_);
}

KernelTimer::~KernelTimer() {
    if (slot_ < 0) return;
    std::lock_guard<std::mutex> lock(g_mu);
    cudaEventRecord(g_recs[slot_].stop, stream_);
}

}  // namespace gb

extern "C" void gb300_profile_enable(int on) { gb::g_on.store(on != 0); }

extern "C" int gb300_profile_read(const char* prefix, double* total_ms, int64_t* launches) {
    std::lock_guard<std::mutex> lock(gb::g_mu);
    double tot = 0.0;
    int64_t cnt = 0;
    for (auto& r : gb::g_recs) {
        if (!r.used) continue;
        if (cudaEventSynchronize(r.stop) != cudaSuccess) {
            gb::set_error(GB300_ERR_CUDA, "gb300_profile_read: event wait failed");
            return GB300_ERR_CUDA;
        }
        if (!prefix || std::strncmp(r.name.c_str(), prefix, std::strlen(prefix)) == 0) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, r.start, r.stop);
            tot += ms;
            ++cnt;
        }
        r.used = false;
    }
    if (total_ms) *total_ms = tot;
    if (launches) *launches = cnt;
    return GB300_OK;
}
