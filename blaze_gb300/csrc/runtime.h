// runtime.h — process-wide state of libgb300blas: the device, the library stream, grow-only
// device buffers, the device status word, the thread-local last error and launch accounting.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

namespace gb {

// Buffer slots of the grow-only device pool.  A slot keeps its high-water allocation for the
// life of the process, so repeated calls of similar size allocate nothing.
enum Slot : int {
    kSlotA = 0,        // staged / realigned A
    kSlotB,            // staged / realigned B
    kSlotC,            // staged / realigned C
    kSlotWork,         // split-k partials
    kSlotSliceA,       // split-precision digit planes of A
    kSlotSliceB,       // split-precision digit planes of B
    kSlotScaleA,       // per-row exponents of A
    kSlotScaleB,       // per-column exponents of B
    kSlotLevels,       // split-precision per-level integer sums
    kSlotMisc,         // small reductions (norms, bounds)
    kSlotExtra,        // unused by the products; the eleventh buffer of the neighbouring routines
    kSlotCount
};

// Grow-only device buffers of one execution context (the library's default context, or one slot
// of a server), used on that context's stream.  A slot keeps its high-water allocation, so
// repeated calls of similar size allocate nothing.
struct Workspace {
    cudaStream_t stream = nullptr;
    // Stream-ordered buffers (cudaMallocAsync / cudaFreeAsync on `stream`): growing or releasing
    // them never waits for other streams.  For contexts whose buffers only `stream` uses (the
    // server's slots); cudaFree would wait for the whole device.
    bool stream_ordered = false;
    int* d_status = nullptr;       // device status word written by kernels (DeviceStatus)
    void* ptr[kSlotCount] = {};
    size_t bytes[kSlotCount] = {};
    // Buffer of at least `n` bytes in slot `s`; nullptr (and *err) on allocation failure.
    void* get(int s, size_t n, std::string* err);
    size_t total() const;
    void release();                // frees every buffer (after the stream drained)
};

struct Runtime {
    std::mutex mu;                 // one queue: GPU work submitted through the library is serialized
    bool inited = false;
    int device = -1;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    int* d_status = nullptr;       // device status word of the default context
    Workspace ws;                  // default context (stream = `stream`)
    Workspace aux;                 // operands and intermediates of ?gemv, complex ?gemm, ?trmm
                                   // (their real products use `ws`)
    std::atomic<int64_t> launches{0};
    int inject_stall_count = 0;
    uint64_t inject_limit_ns = 0;
    // copy streams and events of the panel pipeline for host operands (created on first use)
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    static constexpr int kPipeEvents = 64;
    cudaEvent_t pipe_ev[kPipeEvents] = {};
    bool pipe_ready = false;
    // events ordering a split product's two column parts across its two streams (created on
    // first use, reused)
    std::mutex part_mu;
    std::vector<cudaEvent_t> part_events;
};

Runtime& runtime();

// Bytes held by every Workspace of the process (the default context, the neighbouring routines'
// buffers and the server slots), as allocated by Workspace::get and returned by release().
extern std::atomic<int64_t> g_pool_bytes;

// Initialise the device state once (thread-safe).  Returns a gb300_status.
int ensure_init(std::string* err);

// Device buffer of at least `bytes` in slot `s` of the default context (caller holds
// runtime().mu).  nullptr on failure.
void* pool_get(int s, size_t bytes, std::string* err);

// Thread-local last error.
void set_error(int status, const std::string& msg);
void clear_error();

// One C-ABI call: an NVTX range named after the routine around the whole call (shown by Nsight
// tools; close to free when none is attached) and, with GB300_BLAS_TRACE=1 in the environment, an
// enter and a leave line on stderr with the thread, the shape, the call's status and its wall time
// (the counterpart of Blaze's BLAZE_FUNCTION_TRACE).
class CallTrace {
  public:
    CallTrace(const char* routine, int64_t m, int64_t n, int64_t k);
    ~CallTrace();
    CallTrace(const CallTrace&) = delete;
    CallTrace& operator=(const CallTrace&) = delete;

  private:
    const char* routine_;
    double t0_ = 0.0;
    bool trace_ = false;
};
int last_error();
const char* last_error_message();

// Count kernel launches issued by the library.
inline void count_launches(int n) { runtime().launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace gb
