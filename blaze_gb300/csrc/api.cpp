// api.cpp — the C-ABI of libgb300blas: CBLAS dgemm/sgemm (the call Blaze's BLAS mode makes),
// the extended gb300_*gemm_ex entry points, and error reporting.
//
// Call path replaced:  blaze::gemm(C,A,B,alpha,beta)        blaze/math/blas/gemm.h:105-131
//                      -> gemm(CBLAS_ORDER, ...)             blaze/math/blas/cblas/gemm.h:116-162
//                      -> cblas_dgemm / cblas_sgemm          (this file)
// Semantics follow CBLAS: C = alpha*op(A)*op(B) + beta*C; beta == 0 does not read C; quick return
// when m == 0, n == 0, or (alpha == 0 or k == 0) and beta == 1; argument errors name the
// 1-based parameter position like xerbla.  Operands may be host memory (pageable or pinned) —
// staged through the device inside the call — or device/managed memory, used in place.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/gb300_blas.h"
#include "../../include/gb300_cblas.h"
#include "gb300_internal.h"
#include "ptx.cuh"
#include "runtime.h"
#include "split_api.h"

namespace gb {
namespace {

int g_default_method = -1;

int default_method() {
    if (g_default_method < 0) {
        g_default_method = GB300_METHOD_AUTO;
        if (const char* v = std::getenv("GB300_DGEMM_METHOD")) {
            const std::string s(v);
            if (s == "native") g_default_method = GB300_METHOD_NATIVE;
            else if (s == "split") g_default_method = GB300_METHOD_SPLIT;
            else if (s == "split_crt") g_default_method = GB300_METHOD_SPLIT_CRT;
            else if (s == "bf16x3") g_default_method = GB300_METHOD_BF16X3;
            else if (s == "bf16") g_default_method = GB300_METHOD_BF16;
        }
    }
    return g_default_method;
}

bool is_device_ptr(const void* p) {
    if (p == nullptr) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Stored (row-major) shape of an operand of the logical problem.
struct Stored {
    const void* ptr;
    int64_t rows, cols, ld;
};

template <typename T>
bool aligned_for_tma(const Stored& s) {
    return (reinterpret_cast<uintptr_t>(s.ptr) % 16 == 0) && ((s.ld * int64_t(sizeof(T))) % 16 == 0);
}

int64_t padded_ld(int64_t cols, size_t elem) {
    const int64_t q = int64_t(16 / elem);
    return std::max<int64_t>((cols + q - 1) / q * q, q);
}

// Copy `s` into device slot `slot` with a TMA-compatible pitch; returns the new Stored.
template <typename T>
bool stage_in(const Stored& s, int slot, bool from_host, cudaStream_t st, Stored* out, std::string* err) {
    const int64_t ldp = padded_ld(s.cols, sizeof(T));
    void* d = pool_get(slot, size_t(ldp) * size_t(s.rows) * sizeof(T), err);
    if (!d) return false;
    cudaError_t e = cudaMemcpy2DAsync(d, size_t(ldp) * sizeof(T), s.ptr, size_t(s.ld) * sizeof(T),
                                      size_t(s.cols) * sizeof(T), size_t(s.rows),
                                      from_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
        if (err) *err = std::string("operand copy: ") + cudaGetErrorString(e);
        return false;
    }
    *out = Stored{d, s.rows, s.cols, ldp};
    return true;
}

const char* method_name(int m) {
    switch (m) {
        case GB300_METHOD_NATIVE: return "native";
        case GB300_METHOD_SPLIT: return "split";
        case GB300_METHOD_BF16X3: return "bf16x3";
        case GB300_METHOD_BF16: return "bf16";
        case GB300_METHOD_SPLIT_CRT: return "split_crt";
        default: return "auto";
    }
}

}  // namespace

int library_default_method() { return default_method(); }

template <typename T>
int gemm_entry(int order, int transA, int transB, int64_t m, int64_t n, int64_t k, T alpha, const T* A, int64_t lda,
              const T* B, int64_t ldb, T beta, T* C, int64_t ldc, gb300_gemm_opts* opts, const char* routine) {
    const bool is_double = sizeof(T) == 8;
    const CallTrace trace(routine, m, n, k);
    auto fail = [&](int st, const std::string& msg) {
        set_error(st, std::string(routine) + ": " + msg);
        return st;
    };
    // ---- argument checks (CBLAS contract; positions as in xerbla) ----
    if (order != CblasRowMajor && order != CblasColMajor) return fail(GB300_ERR_INVALID_ARG, "parameter 1 (order) is invalid");
    auto valid_trans = [](int t) { return t == CblasNoTrans || t == CblasTrans || t == CblasConjTrans; };
    if (!valid_trans(transA)) return fail(GB300_ERR_INVALID_ARG, "parameter 2 (transA) is invalid");
    if (!valid_trans(transB)) return fail(GB300_ERR_INVALID_ARG, "parameter 3 (transB) is invalid");
    if (m < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 4 (m) is negative");
    if (n < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 5 (n) is negative");
    if (k < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 6 (k) is negative");
    const bool tA = transA != CblasNoTrans, tB = transB != CblasNoTrans;
    const bool rm = order == CblasRowMajor;
    // minimum leading dimensions: row length of the stored matrix
    const int64_t minlda = std::max<int64_t>(1, rm ? (tA ? m : k) : (tA ? k : m));
    const int64_t minldb = std::max<int64_t>(1, rm ? (tB ? k : n) : (tB ? n : k));
    const int64_t minldc = std::max<int64_t>(1, rm ? n : m);
    if (lda < minlda) return fail(GB300_ERR_INVALID_ARG, "parameter 9 (lda) is too small");
    if (ldb < minldb) return fail(GB300_ERR_INVALID_ARG, "parameter 11 (ldb) is too small");
    if (ldc < minldc) return fail(GB300_ERR_INVALID_ARG, "parameter 14 (ldc) is too small");
    int method = opts ? opts->method : GB300_METHOD_AUTO;
    if (method == GB300_METHOD_AUTO && opts == nullptr) method = default_method();
    if (method < GB300_METHOD_AUTO || method > GB300_METHOD_SPLIT_CRT)
        return fail(GB300_ERR_INVALID_ARG, "unknown method " + std::to_string(method));
    clear_error();
    if (opts) {
        opts->method_used = GB300_METHOD_NATIVE;
        opts->slices_used = 0;
        opts->error_bound = 0.0;
    }
    // ---- quick returns ----
    if (m == 0 || n == 0) return GB300_OK;
    if ((alpha == T(0) || k == 0) && beta == T(1)) return GB300_OK;
    if (A == nullptr && alpha != T(0) && k > 0) return fail(GB300_ERR_INVALID_ARG, "parameter 8 (A) is NULL");
    if (B == nullptr && alpha != T(0) && k > 0) return fail(GB300_ERR_INVALID_ARG, "parameter 10 (B) is NULL");
    if (C == nullptr) return fail(GB300_ERR_INVALID_ARG, "parameter 13 (C) is NULL");

    Runtime& r = runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = ensure_init(&err);
    if (st != GB300_OK) return fail(st, err);

    // ---- logical row-major form ----
    Gemm g;
    if (rm) {
        g.m = m; g.n = n; g.k = k; g.ta = tA; g.tb = tB;
        g.A = A; g.lda = lda; g.B = B; g.ldb = ldb;
    } else {  // C^T = op(B)^T op(A)^T
        g.m = n; g.n = m; g.k = k; g.ta = tB; g.tb = tA;
        g.A = B; g.lda = ldb; g.B = A; g.ldb = lda;
    }
    g.C = C; g.ldc = ldc;
    const bool product = (alpha != T(0)) && k > 0;
    if (!product) g.k = 0;  // C = beta*C only
    g.alpha = double(alpha);
    g.beta = double(beta);

    // ---- residency ----
    const int res = opts ? opts->residency : GB300_PTR_DETECT;
    auto on_device = [&](const void* p) {
        if (res == GB300_PTR_DEVICE) return true;
        if (res == GB300_PTR_HOST) return false;
        return is_device_ptr(p);
    };
    const bool devC = on_device(C);
    const bool devA = product ? on_device(g.A) : true;
    const bool devB = product ? on_device(g.B) : true;
    const bool any_host = !(devA && devB && devC);
    cudaStream_t s = (opts && opts->stream) ? static_cast<cudaStream_t>(opts->stream) : r.stream;
    const bool sync = any_host || !opts || opts->synchronous;

    LaunchCtl ctl;
    ctl.status = r.d_status;
    if (r.inject_stall_count > 0) {
        --r.inject_stall_count;
        ctl.inject_stall = 1;
        ctl.wait_limit_ns = r.inject_limit_ns;
    }
    cudaMemsetAsync(r.d_status, 0, sizeof(int), s);
    int used = method;
    const void* info_dev = nullptr;
    cudaError_t e = cudaSuccess;

    // Host operands of a large FP64-accurate product: row panels of A whose copies in and out
    // overlap the computation (falls through to staging when the method or shape does not qualify).
    bool done = false;
    if (is_double && product && !devA && !devB && !devC && method != GB300_METHOD_NATIVE) {
        SplitRequest req;
        req.method = method;
        req.slices = opts ? opts->slices : 0;
        req.target_error = opts ? opts->target_error : 0.0;
        SplitResult pres;
        const int pst = device_product_host_panels(g, req, ctl, s, r.ws, &pres, &err);
        if (pst == GB300_OK) {
            done = true;
            used = pres.method_used;
            info_dev = pres.info_dev;
        } else if (pst != GB300_ERR_NOT_SUPPORTED) {
            return fail(pst, err);
        } else {
            err.clear();
        }
    }

    Stored sa{g.A, g.ta ? g.k : g.m, g.ta ? g.m : g.k, g.lda};
    Stored sb{g.B, g.tb ? g.n : g.k, g.tb ? g.k : g.n, g.ldb};
    Stored sc{g.C, g.m, g.n, g.ldc};
    Stored da = sa, db = sb, dc = sc;
    bool c_staged = false;
    if (!done) {
    if (product) {
        if (!devA || !aligned_for_tma<T>(sa))
            if (!stage_in<T>(sa, kSlotA, !devA, s, &da, &err)) return fail(GB300_ERR_NO_MEMORY, err);
        if (!devB || !aligned_for_tma<T>(sb))
            if (!stage_in<T>(sb, kSlotB, !devB, s, &db, &err)) return fail(GB300_ERR_NO_MEMORY, err);
    }
    if (!devC) {
        c_staged = true;
        const int64_t ldp = padded_ld(sc.cols, sizeof(T));
        void* d = pool_get(kSlotC, size_t(ldp) * size_t(sc.rows) * sizeof(T), &err);
        if (!d) return fail(GB300_ERR_NO_MEMORY, err);
        dc = Stored{d, sc.rows, sc.cols, ldp};
        if (beta != T(0)) {
            cudaError_t e = cudaMemcpy2DAsync(d, size_t(ldp) * sizeof(T), C, size_t(ldc) * sizeof(T),
                                              size_t(sc.cols) * sizeof(T), size_t(sc.rows), cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("copy of C: ") + cudaGetErrorString(e));
        }
    }
    g.A = da.ptr; g.lda = da.ld;
    g.B = db.ptr; g.ldb = db.ld;
    g.C = const_cast<void*>(dc.ptr); g.ldc = dc.ld;

    // ---- run ----
    // float: the split forms run on double copies at the float target (device_product_float); small
    // products under `auto` stay on the native kernel, as for double
    const bool split_path = product && method != GB300_METHOD_NATIVE &&
                            (is_double || !(method == GB300_METHOD_AUTO && split_auto_uses_native(g)));
    if (split_path) {
        SplitRequest req;
        req.method = method;
        req.slices = opts ? opts->slices : 0;
        req.target_error = opts ? opts->target_error : 0.0;
        SplitResult res_out;
        st = is_double ? device_product(g, req, ctl, s, r.ws, &res_out, &err)
                       : device_product_float(g, req, ctl, s, r.ws, r.aux, &res_out, &err);
        if (st != GB300_OK) return fail(st, err);
        used = res_out.method_used;
        info_dev = res_out.info_dev;
        if (opts) {
            opts->slices_used = res_out.slices;
            opts->error_bound = res_out.error_bound;
        }
    } else {
        used = GB300_METHOD_NATIVE;
        int splits = 1;
        T* ws = nullptr;
        if (g.k > 0) {
            splits = native_choose_splits(g.m, g.n, g.k, int(sizeof(T)), r.num_sms);
            if (splits > 1) {
                ws = static_cast<T*>(pool_get(kSlotWork, size_t(splits) * size_t(g.m) * size_t(g.n) * sizeof(T), &err));
                if (!ws) return fail(GB300_ERR_NO_MEMORY, err);
            }
        }
        e = native_gemm<T>(g, splits, ws, ctl, s, &err);
        if (e != cudaSuccess) return fail(GB300_ERR_CUDA, err.empty() ? cudaGetErrorString(e) : err);
        if (opts) opts->error_bound = double(g.k) * (is_double ? 0x1p-53 : 0x1p-24);
    }
    if (opts) opts->method_used = used;

    if (c_staged) {
        e = copy_to_host(C, size_t(ldc) * sizeof(T), dc.ptr, size_t(dc.ld) * sizeof(T), size_t(sc.cols) * sizeof(T),
                         size_t(sc.rows), s);
        if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("copy of C back: ") + cudaGetErrorString(e));
    }
    }  // !done
    if (opts) opts->method_used = used;
    if (sync) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("kernel failed: ") + cudaGetErrorString(e));
        int status = 0;
        cudaMemcpy(&status, r.d_status, sizeof(int), cudaMemcpyDeviceToHost);
        if (status != kDevOk)
            return fail(GB300_ERR_DEVICE_TIMEOUT, std::string("a device-side wait ran out (code ") +
                                                      std::to_string(status) + ", method " + method_name(used) +
                                                      "); the result is incomplete");
        if (opts && info_dev) {
            int sl = 0;
            double bd = 0;
            if (split_read_info(info_dev, &sl, &bd)) {
                opts->slices_used = sl;
                opts->error_bound = is_double ? bd : bd + 0x1p-24;  // float: the final rounding
            }
        }
    }
    return GB300_OK;
}

template int gemm_entry<double>(int, int, int, int64_t, int64_t, int64_t, double, const double*, int64_t,
                                const double*, int64_t, double, double*, int64_t, gb300_gemm_opts*, const char*);
template int gemm_entry<float>(int, int, int, int64_t, int64_t, int64_t, float, const float*, int64_t, const float*,
                               int64_t, float, float*, int64_t, gb300_gemm_opts*, const char*);

}  // namespace gb

// ============================================================================================
//  C-ABI
// ============================================================================================
extern "C" {

void gb300_gemm_opts_init(gb300_gemm_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->method = gb::default_method();
    o->slices = 0;
    o->target_error = 0.0;
    o->residency = GB300_PTR_DETECT;
    o->stream = nullptr;
    o->synchronous = 1;
}

int gb300_dgemm_ex(int order, int transA, int transB, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                   int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                   gb300_gemm_opts* opts) {
    return gb::gemm_entry<double>(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, opts,
                                 "gb300_dgemm_ex");
}

int gb300_sgemm_ex(int order, int transA, int transB, int64_t m, int64_t n, int64_t k, float alpha, const float* A,
                   int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc, gb300_gemm_opts* opts) {
    return gb::gemm_entry<float>(order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, opts,
                                "gb300_sgemm_ex");
}

int gb300_set_default_method(int method) {
    const int prev = gb::default_method();
    if (method >= GB300_METHOD_AUTO && method <= GB300_METHOD_SPLIT_CRT) gb::g_default_method = method;
    return prev;
}

int gb300_last_error(void) { return gb::last_error(); }

const char* gb300_last_error_message(void) { return gb::last_error_message(); }

void gb300_clear_error(void) { gb::clear_error(); }

int gb300_device_info(int* num_sms, int64_t* free_bytes, int64_t* total_bytes) {
    gb::Runtime& r = gb::runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    const int st = gb::ensure_init(&err);
    if (st != GB300_OK) {
        gb::set_error(st, "gb300_device_info: " + err);
        return st;
    }
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    if (num_sms) *num_sms = r.num_sms;
    if (free_bytes) *free_bytes = int64_t(fr);
    if (total_bytes) *total_bytes = int64_t(tot);
    return GB300_OK;
}

int64_t gb300_launch_count(void) { return gb::runtime().launches.load(); }

int64_t gb300_pool_bytes(void) { return gb::g_pool_bytes.load(); }

int gb300_select_device(int ordinal) {
    gb::Runtime& r = gb::runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    if (r.inited) {
        if (r.device == ordinal) return GB300_OK;
        gb::set_error(GB300_ERR_INVALID_ARG, "gb300_select_device: the library already runs on device " +
                                                 std::to_string(r.device));
        return GB300_ERR_INVALID_ARG;
    }
    cudaError_t e = cudaSetDevice(ordinal);
    if (e != cudaSuccess) {
        gb::set_error(GB300_ERR_NO_DEVICE, std::string("gb300_select_device: ") + cudaGetErrorString(e));
        return GB300_ERR_NO_DEVICE;
    }
    return GB300_OK;
}

int gb300_synchronize(void) {
    gb::Runtime& r = gb::runtime();
    if (!r.inited) return GB300_OK;
    cudaError_t e = cudaStreamSynchronize(r.stream);
    if (e != cudaSuccess) {
        gb::set_error(GB300_ERR_CUDA, std::string("gb300_synchronize: ") + cudaGetErrorString(e));
        return GB300_ERR_CUDA;
    }
    int status = 0;
    cudaMemcpy(&status, r.d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (status != 0) {
        gb::set_error(GB300_ERR_DEVICE_TIMEOUT, "gb300_synchronize: a device-side wait ran out");
        return GB300_ERR_DEVICE_TIMEOUT;
    }
    return GB300_OK;
}

void gb300_debug_inject_stall(int count, uint64_t limit_ns) {
    gb::Runtime& r = gb::runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    r.inject_stall_count = count > 0 ? count : 0;
    r.inject_limit_ns = limit_ns > 0 ? limit_ns : 20000000ull;
}

}  // extern "C"
