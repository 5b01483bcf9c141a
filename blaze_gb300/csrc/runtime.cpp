// runtime.cpp — device state, tensor-map encoding, device buffer pool and error bookkeeping.
#include "runtime.h"

#include <nvtx3/nvToolsExt.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <thread>

#include "../../include/gb300_blas.h"
#include "gb300_internal.h"

namespace gb {

namespace {

struct ThreadError {
    int status = 0;
    std::string msg;
};
thread_local ThreadError t_err;

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn g_encode = nullptr;
std::once_flag g_encode_once;

EncodeTiledFn encode_fn() {
    std::call_once(g_encode_once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        // The library links the CUDA runtime statically and reaches the driver's tensor-map
        // encoder through the runtime, so loading the library needs no driver.
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<EncodeTiledFn>(fn);
    });
    return g_encode;
}

}  // namespace

Runtime& runtime() {
    static Runtime* r = new Runtime();  // never destroyed: safe at process exit
    return *r;
}

namespace {
bool trace_enabled() {
    static const bool on = [] {
        const char* v = std::getenv("GB300_BLAS_TRACE");
        return v && *v && *v != '0';
    }();
    return on;
}

double wall_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

unsigned long long thread_tag() { return (unsigned long long)std::hash<std::thread::id>()(std::this_thread::get_id()); }
}  // namespace

CallTrace::CallTrace(const char* routine, int64_t m, int64_t n, int64_t k) : routine_(routine) {
    nvtxRangePushA(routine);
    trace_ = trace_enabled();
    if (trace_) {
        std::fprintf(stderr, "libgb300blas: enter %s m=%lld n=%lld k=%lld thread=%llx\n", routine, (long long)m,
                     (long long)n, (long long)k, thread_tag());
        t0_ = wall_ms();
    }
}

CallTrace::~CallTrace() {
    if (trace_)
        std::fprintf(stderr, "libgb300blas: leave %s status=%d ms=%.3f thread=%llx\n", routine_, t_err.status,
                     wall_ms() - t0_, thread_tag());
    nvtxRangePop();
}

void set_error(int status, const std::string& msg) {
    t_err.status = status;
    t_err.msg = msg;
    if (status != 0) {
        static const bool verbose = [] {
            const char* v = std::getenv("GB300_BLAS_VERBOSE");
            return v && *v && *v != '0';
        }();
        static const bool abort_on = [] {
            const char* v = std::getenv("GB300_BLAS_ABORT_ON_ERROR");
            return v && *v && *v != '0';
        }();
        if (verbose || abort_on) std::fprintf(stderr, "libgb300blas: %s\n", msg.c_str());
        if (abort_on) std::abort();
    }
}

void clear_error() {
    t_err.status = 0;
    t_err.msg.clear();
}

int last_error() { return t_err.status; }

const char* last_error_message() { return t_err.msg.c_str(); }

int ensure_init(std::string* err) {
    Runtime& r = runtime();
    if (r.inited) return GB300_OK;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        if (err) *err = std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "count is 0");
        return GB300_ERR_NO_DEVICE;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, dev)) != cudaSuccess) {
        if (err) *err = std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    if (prop.major < 10) {
        if (err) *err = "libgb300blas needs an sm_103a (Blackwell Ultra) device; found sm_" +
                        std::to_string(prop.major) + std::to_string(prop.minor);
        return GB300_ERR_NO_DEVICE;
    }
    if ((e = cudaStreamCreateWithFlags(&r.stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc(&r.d_status, 64)) != cudaSuccess || (e = cudaMemset(r.d_status, 0, 64)) != cudaSuccess) {
        if (err) *err = std::string("device set-up: ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    if (!encode_fn()) {
        if (err) *err = "the driver does not provide cuTensorMapEncodeTiled";
        return GB300_ERR_CUDA;
    }
    r.device = dev;
    r.num_sms = prop.multiProcessorCount;
    r.ws.stream = r.stream;
    r.ws.d_status = r.d_status;
    r.aux.stream = r.stream;
    r.aux.d_status = r.d_status;
    r.inited = true;
    return GB300_OK;
}

std::atomic<int64_t> g_pool_bytes{0};

void* Workspace::get(int s, size_t n, std::string* err) {
    if (n == 0) n = 256;
    if (bytes[s] >= n) return ptr[s];
    if (ptr[s]) {
        if (stream_ordered) {
            cudaFreeAsync(ptr[s], stream);
        } else {
            cudaStreamSynchronize(stream);
            cudaFree(ptr[s]);
        }
        g_pool_bytes.fetch_sub(int64_t(bytes[s]));
        ptr[s] = nullptr;
        bytes[s] = 0;
    }
    // round up to 2 MiB so that slowly growing sizes do not reallocate every call
    const size_t rounded = (n + (size_t(2) << 20) - 1) & ~((size_t(2) << 20) - 1);
    void* p = nullptr;
    cudaError_t e = stream_ordered ? cudaMallocAsync(&p, rounded, stream) : cudaMalloc(&p, rounded);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (err) *err = "device allocation of " + std::to_string(rounded) + " bytes failed: " + cudaGetErrorString(e);
        return nullptr;
    }
    ptr[s] = p;
    bytes[s] = rounded;
    g_pool_bytes.fetch_add(int64_t(rounded));
    return p;
}

size_t Workspace::total() const {
    size_t t = 0;
    for (int s = 0; s < kSlotCount; ++s) t += bytes[s];
    return t;
}

void Workspace::release() {
    if (stream && !stream_ordered) cudaStreamSynchronize(stream);
    for (int s = 0; s < kSlotCount; ++s) {
        if (ptr[s]) {
            if (stream_ordered) cudaFreeAsync(ptr[s], stream);
            else cudaFree(ptr[s]);
            g_pool_bytes.fetch_sub(int64_t(bytes[s]));
        }
        ptr[s] = nullptr;
        bytes[s] = 0;
    }
}

void* pool_get(int s, size_t bytes, std::string* err) { return runtime().ws.get(s, bytes, err); }

bool encode_tmap_2d(CUtensorMap* map, CUtensorMapDataType dtype, size_t elem_bytes, const void* base,
                    uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows, uint32_t box_cols,
                    CUtensorMapSwizzle swizzle, std::string* err) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) {
        if (err) *err = "cuTensorMapEncodeTiled unavailable";
        return false;
    }
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {ld * elem_bytes};
    cuuint32_t box[2] = {box_cols, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, dtype, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        if (err)
            *err = "cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ") for " + std::to_string(rows) + "x" +
                   std::to_string(cols) + " ld=" + std::to_string(ld) + " box " + std::to_string(box_rows) + "x" +
                   std::to_string(box_cols);
        return false;
    }
    return true;
}

bool encode_tmap_3d(CUtensorMap* map, CUtensorMapDataType dtype, size_t elem_bytes, const void* base,
                    uint64_t planes, uint64_t rows, uint64_t cols, uint64_t ld, uint64_t plane_stride,
                    uint32_t box_rows, uint32_t box_cols, CUtensorMapSwizzle swizzle, std::string* err) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) {
        if (err) *err = "cuTensorMapEncodeTiled unavailable";
        return false;
    }
    cuuint64_t dims[3] = {cols, rows, planes};
    cuuint64_t strides[2] = {ld * elem_bytes, plane_stride * elem_bytes};
    cuuint32_t box[3] = {box_cols, box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, dtype, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        if (err) *err = "cuTensorMapEncodeTiled (3-D) failed (" + std::to_string(int(r)) + ")";
        return false;
    }
    return true;
}

}  // namespace gb
