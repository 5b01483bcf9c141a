// api_next.cpp — the BLAS routines next to ?gemm on Blaze's seam, on the GPU:
//
//   cblas_?gemv   y = alpha op(A) x + beta y          blaze/math/blas/cblas/gemv.h:116-235
//   cblas_zgemm / cblas_cgemm  complex C = alpha op(A) op(B) + beta C
//                                                     blaze/math/blas/cblas/gemm.h:196-256
//   cblas_?trmm   B = alpha op(A) B or alpha B op(A), A triangular
//                                                     blaze/math/blas/cblas/trmm.h:116-235
//
// Semantics follow CBLAS (argument positions as in xerbla, quick returns, beta == 0 does not read
// the output, alpha == 0 does not read the inputs).  Complex products are four real products of
// the real and imaginary parts (conjugate-transpose flips the sign of an imaginary part), each
// through the library's real product: FP64-accurate split precision for double by default, the
// native kernel for float.  A triangular product runs on a dense copy of the triangle (zeros
// elsewhere, ones on a unit diagonal).  Host operands are staged through device buffers;
// device or managed operands are used in place.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/gb300_blas.h"
#include "../../include/gb300_cblas.h"
#include "gb300_internal.h"
#include "level23.h"
#include "ptx.cuh"
#include "runtime.h"
#include "split_api.h"

namespace gb {
namespace {

bool on_device(const void* p) {
    if (p == nullptr) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// aux workspace slots of these routines
enum AuxSlot : int { kAuxA = 0, kAuxB, kAuxC, kAuxX, kAuxY, kAuxAr, kAuxAi, kAuxBr, kAuxBi, kAuxP };

// Device copy of `rows` x `cols` elements (pitch ld, elem bytes each) of a host or device buffer into
// aux slot `slot` with the same pitch; returns the device pointer (or the buffer itself when it is
// already on the device).
void* stage(const void* p, int64_t rows, int64_t cols, int64_t ld, size_t elem, int slot, bool dev, cudaStream_t st,
            std::string* err) {
    if (dev || rows == 0 || cols == 0) return const_cast<void*>(p);
    const size_t bytes = (size_t(std::max<int64_t>(rows - 1, 0)) * size_t(ld) + size_t(cols)) * elem;
    void* d = runtime().aux.get(slot, bytes, err);
    if (!d) return nullptr;
    const cudaError_t e = cudaMemcpy2DAsync(d, size_t(ld) * elem, p, size_t(ld) * elem, size_t(cols) * elem,
                                            size_t(rows), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        if (err) *err = std::string("operand copy: ") + cudaGetErrorString(e);
        return nullptr;
    }
    return d;
}

cudaError_t unstage(void* host, const void* dev, int64_t rows, int64_t cols, int64_t ld, size_t elem, cudaStream_t st) {
    if (rows == 0 || cols == 0) return cudaSuccess;
    return copy_to_host(host, size_t(ld) * elem, dev, size_t(ld) * elem, size_t(cols) * elem, size_t(rows), st);
}

// Finish a call: wait for the stream and read the device status word.
int finish(cudaStream_t st, std::string* err) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        if (err) *err = std::string("kernel failed: ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    int status = 0;
    cudaMemcpy(&status, runtime().d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (status != kDevOk) {
        if (err) *err = "a device-side wait ran out (code " + std::to_string(status) + "); the result is incomplete";
        return GB300_ERR_DEVICE_TIMEOUT;
    }
    return GB300_OK;
}

// One real product C = alpha op(A) op(B) + beta C of device operands in the logical row-major form:
// the default method for double (FP64-accurate split precision, or the native kernel for small
// products and when native is the default), the native kernel for float.
template <typename T>
int real_product(const Gemm& g, const LaunchCtl& ctl, cudaStream_t st, std::string* err) {
    Runtime& r = runtime();
    const int method = library_default_method();
    if (sizeof(T) == 8 && method != GB300_METHOD_NATIVE) {
        SplitRequest req;
        req.method = method;
        SplitResult out;
        return device_product(g, req, ctl, st, r.ws, &out, err);
    }
    // the native kernel reads A and B through TMA: 16-byte aligned bases and pitches, else a copy
    Gemm gn = g;
    auto realign = [&](const void*& p, int64_t& ld, int64_t rows, int64_t cols, int slot) {
        if (reinterpret_cast<uintptr_t>(p) % 16 == 0 && (ld * int64_t(sizeof(T))) % 16 == 0) return true;
        const int64_t q = int64_t(16 / sizeof(T)), ldp = (cols + q - 1) / q * q;
        void* d = r.ws.get(slot, size_t(rows) * size_t(ldp) * sizeof(T), err);
        if (!d) return false;
        if (cudaMemcpy2DAsync(d, size_t(ldp) * sizeof(T), p, size_t(ld) * sizeof(T), size_t(cols) * sizeof(T),
                              size_t(rows), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            return false;
        p = d;
        ld = ldp;
        return true;
    };
    if (g.k > 0 && (!realign(gn.A, gn.lda, g.ta ? g.k : g.m, g.ta ? g.m : g.k, kSlotA) ||
                    !realign(gn.B, gn.ldb, g.tb ? g.n : g.k, g.tb ? g.k : g.n, kSlotB)))
        return GB300_ERR_NO_MEMORY;
    int splits = 1;
    T* w = nullptr;
    if (g.k > 0) {
        splits = native_choose_splits(g.m, g.n, g.k, int(sizeof(T)), r.num_sms);
        if (splits > 1) {
            w = static_cast<T*>(r.ws.get(kSlotWork, size_t(splits) * size_t(g.m) * size_t(g.n) * sizeof(T), err));
            if (!w) return GB300_ERR_NO_MEMORY;
        }
    }
    const cudaError_t e = native_gemm<T>(gn, splits, w, ctl, st, err);
    return e == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

LaunchCtl fresh_ctl(cudaStream_t st) {
    Runtime& r = runtime();
    LaunchCtl ctl;
    ctl.status = r.d_status;
    cudaMemsetAsync(r.d_status, 0, sizeof(int), st);
    return ctl;
}

}  // namespace

// ---- gemv --------------------------------------------------------------------------------------
template <typename T>
int gemv_entry(int order, int transA, int64_t m, int64_t n, T alpha, const T* A, int64_t lda, const T* x,
               int64_t incx, T beta, T* y, int64_t incy, const char* routine) {
    auto fail = [&](int st, const std::string& msg) {
        set_error(st, std::string(routine) + ": " + msg);
        return st;
    };
    if (order != CblasRowMajor && order != CblasColMajor) return fail(GB300_ERR_INVALID_ARG, "parameter 1 (order) is invalid");
    if (transA != CblasNoTrans && transA != CblasTrans && transA != CblasConjTrans)
        return fail(GB300_ERR_INVALID_ARG, "parameter 2 (transA) is invalid");
    if (m < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 3 (m) is negative");
    if (n < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 4 (n) is negative");
    const bool rm = order == CblasRowMajor, ta = transA != CblasNoTrans;
    if (lda < std::max<int64_t>(1, rm ? n : m)) return fail(GB300_ERR_INVALID_ARG, "parameter 7 (lda) is too small");
    if (incx == 0) return fail(GB300_ERR_INVALID_ARG, "parameter 9 (incx) is zero");
    if (incy == 0) return fail(GB300_ERR_INVALID_ARG, "parameter 12 (incy) is zero");
    clear_error();
    if (m == 0 || n == 0 || (alpha == T(0) && beta == T(1))) return GB300_OK;
    if (y == nullptr) return fail(GB300_ERR_INVALID_ARG, "parameter 11 (y) is NULL");
    if (alpha != T(0) && (A == nullptr || x == nullptr)) return fail(GB300_ERR_INVALID_ARG, "A or x is NULL");

    Runtime& r = runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = ensure_init(&err);
    if (st != GB300_OK) return fail(st, err);
    cudaStream_t s = r.stream;
    const LaunchCtl ctl = fresh_ctl(s);
    (void)ctl;

    // stored row-major S: A itself (row-major, m x n) or A^T (column-major, n x m)
    const int64_t srows = rm ? m : n, scols = rm ? n : m;
    // y = S x (rows form) or y = S^T x (cols form)
    const bool cols_form = rm ? ta : !ta;
    const int64_t xl = ta ? m : n, yl = ta ? n : m;
    const bool use_a = alpha != T(0);
    const T* dS = A;
    if (use_a) {
        dS = static_cast<const T*>(stage(A, srows, scols, lda, sizeof(T), kAuxA, on_device(A), s, &err));
        if (!dS) return fail(GB300_ERR_NO_MEMORY, err);
    }
    const int64_t ax = incx < 0 ? -incx : incx, ay = incy < 0 ? -incy : incy;
    const T* dx = x;
    if (use_a) {
        dx = static_cast<const T*>(stage(x, 1, 1 + (xl - 1) * ax, 1 + (xl - 1) * ax, sizeof(T), kAuxX, on_device(x), s, &err));
        if (!dx) return fail(GB300_ERR_NO_MEMORY, err);
    }
    const bool ydev = on_device(y);
    T* dy = static_cast<T*>(stage(y, 1, 1 + (yl - 1) * ay, 1 + (yl - 1) * ay, sizeof(T), kAuxY, ydev, s, &err));
    if (!dy) return fail(GB300_ERR_NO_MEMORY, err);
    // logical element j of a strided vector: base + j * inc, the base at the far end for inc < 0
    const T* xb = dx + (incx < 0 ? (xl - 1) * ax : 0);
    T* yb = dy + (incy < 0 ? (yl - 1) * ay : 0);
    const int64_t rows = cols_form ? srows : yl, cols = cols_form ? yl : (use_a ? scols : 0);
    int slices = 1;
    T* part = nullptr;
    if (cols_form && use_a) {
        slices = int(std::max<int64_t>(1, std::min<int64_t>(64, srows / 256)));
        part = static_cast<T*>(r.aux.get(kAuxP, size_t(slices) * size_t(yl) * sizeof(T), &err));
        if (!part) return fail(GB300_ERR_NO_MEMORY, err);
    }
    cudaError_t e = cols_form && use_a
                        ? launch_gemv<T>(true, srows, yl, alpha, dS, lda, xb, incx, beta, yb, incy, part, slices, s)
                        : launch_gemv<T>(false, rows, cols, alpha, dS, lda, xb, incx, beta, yb, incy, nullptr, 1, s);
    if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("gemv launch: ") + cudaGetErrorString(e));
    if (!ydev && (e = unstage(y, dy, 1, 1 + (yl - 1) * ay, 1 + (yl - 1) * ay, sizeof(T), s)) != cudaSuccess)
        return fail(GB300_ERR_CUDA, std::string("copy of y back: ") + cudaGetErrorString(e));
    st = finish(s, &err);
    return st == GB300_OK ? GB300_OK : fail(st, err);
}

// ---- complex gemm ------------------------------------------------------------------------------
template <typename T>
int cgemm_entry(int order, int transA, int transB, int64_t m, int64_t n, int64_t k, const T* alpha, const T* A,
                int64_t lda, const T* B, int64_t ldb, const T* beta, T* C, int64_t ldc, const char* routine) {
    auto fail = [&](int st, const std::string& msg) {
        set_error(st, std::string(routine) + ": " + msg);
        return st;
    };
    if (order != CblasRowMajor && order != CblasColMajor) return fail(GB300_ERR_INVALID_ARG, "parameter 1 (order) is invalid");
    auto valid_trans = [](int t) { return t == CblasNoTrans || t == CblasTrans || t == CblasConjTrans; };
    if (!valid_trans(transA)) return fail(GB300_ERR_INVALID_ARG, "parameter 2 (transA) is invalid");
    if (!valid_trans(transB)) return fail(GB300_ERR_INVALID_ARG, "parameter 3 (transB) is invalid");
    if (m < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 4 (m) is negative");
    if (n < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 5 (n) is negative");
    if (k < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 6 (k) is negative");
    const bool tA = transA != CblasNoTrans, tB = transB != CblasNoTrans, rm = order == CblasRowMajor;
    if (lda < std::max<int64_t>(1, rm ? (tA ? m : k) : (tA ? k : m))) return fail(GB300_ERR_INVALID_ARG, "parameter 9 (lda) is too small");
    if (ldb < std::max<int64_t>(1, rm ? (tB ? k : n) : (tB ? n : k))) return fail(GB300_ERR_INVALID_ARG, "parameter 11 (ldb) is too small");
    if (ldc < std::max<int64_t>(1, rm ? n : m)) return fail(GB300_ERR_INVALID_ARG, "parameter 14 (ldc) is too small");
    if (alpha == nullptr || beta == nullptr) return fail(GB300_ERR_INVALID_ARG, "alpha or beta is NULL");
    const T ar = alpha[0], ai = alpha[1], br = beta[0], bi = beta[1];
    clear_error();
    const bool alpha0 = ar == T(0) && ai == T(0), beta1 = br == T(1) && bi == T(0);
    if (m == 0 || n == 0 || ((alpha0 || k == 0) && beta1)) return GB300_OK;
    if (C == nullptr) return fail(GB300_ERR_INVALID_ARG, "parameter 13 (C) is NULL");
    const bool product = !alpha0 && k > 0;
    if (product && (A == nullptr || B == nullptr)) return fail(GB300_ERR_INVALID_ARG, "A or B is NULL");

    Runtime& r = runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = ensure_init(&err);
    if (st != GB300_OK) return fail(st, err);
    cudaStream_t s = r.stream;
    const LaunchCtl ctl = fresh_ctl(s);

    // logical row-major form (C^T = op(B)^T op(A)^T for column-major; conjugation moves along)
    int64_t M = m, N = n;
    bool ta = tA, tb = tB, ca = transA == CblasConjTrans, cb = transB == CblasConjTrans;
    const T* pA = A;
    const T* pB = B;
    int64_t la = lda, lb = ldb;
    if (!rm) {
        M = n; N = m;
        ta = tB; tb = tA; ca = transB == CblasConjTrans; cb = transA == CblasConjTrans;
        pA = B; pB = A; la = ldb; lb = lda;
    }
    const int64_t ra = ta ? k : M, cA = ta ? M : k;  // stored shape of the first operand
    const int64_t rb = tb ? N : k, cB = tb ? k : N;
    // C: row-major M x N (pitch ldc) in either case
    const bool cdev = on_device(C);
    T* dC = static_cast<T*>(stage(C, M, N, ldc, 2 * sizeof(T), kAuxC, cdev, s, &err));
    if (!dC) return fail(GB300_ERR_NO_MEMORY, err);
    T* Pr = static_cast<T*>(r.aux.get(kAuxP, size_t(2) * size_t(M) * size_t(N) * sizeof(T), &err));
    if (!Pr) return fail(GB300_ERR_NO_MEMORY, err);
    T* Pi = Pr + M * N;
    if (product) {
        const T* dA = static_cast<const T*>(stage(pA, ra, cA, la, 2 * sizeof(T), kAuxA, on_device(pA), s, &err));
        const T* dB = static_cast<const T*>(stage(pB, rb, cB, lb, 2 * sizeof(T), kAuxB, on_device(pB), s, &err));
        T* Ar = static_cast<T*>(r.aux.get(kAuxAr, size_t(ra) * size_t(cA) * sizeof(T), &err));
        T* Ai = static_cast<T*>(r.aux.get(kAuxAi, size_t(ra) * size_t(cA) * sizeof(T), &err));
        T* Br = static_cast<T*>(r.aux.get(kAuxBr, size_t(rb) * size_t(cB) * sizeof(T), &err));
        T* Bi = static_cast<T*>(r.aux.get(kAuxBi, size_t(rb) * size_t(cB) * sizeof(T), &err));
        if (!dA || !dB || !Ar || !Ai || !Br || !Bi) return fail(GB300_ERR_NO_MEMORY, err);
        cudaError_t e = launch_split_complex<T>(ra, cA, dA, la, Ar, Ai, s);
        if (e == cudaSuccess) e = launch_split_complex<T>(rb, cB, dB, lb, Br, Bi, s);
        if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("complex split: ") + cudaGetErrorString(e));
        // op(A) = Ar' + i sa Ai', op(B) = Br' + i sb Bi' (sa = -1 for the conjugate transpose):
        // Re = Ar'Br' - sa sb Ai'Bi',  Im = sb Ar'Bi' + sa Ai'Br'
        const double sa = ca ? -1.0 : 1.0, sb = cb ? -1.0 : 1.0;
        auto prod = [&](const T* X, const T* Y, T* Z, double al, double be) {
            Gemm g;
            g.m = M; g.n = N; g.k = k; g.ta = ta; g.tb = tb;
            g.A = X; g.lda = cA; g.B = Y; g.ldb = cB; g.C = Z; g.ldc = N;
            g.alpha = al; g.beta = be;
            return real_product<T>(g, ctl, s, &err);
        };
        if ((st = prod(Ar, Br, Pr, 1.0, 0.0)) != GB300_OK || (st = prod(Ai, Bi, Pr, -sa * sb, 1.0)) != GB300_OK ||
            (st = prod(Ar, Bi, Pi, sb, 0.0)) != GB300_OK || (st = prod(Ai, Br, Pi, sa, 1.0)) != GB300_OK)
            return fail(st, err);
    } else {
        cudaMemsetAsync(Pr, 0, size_t(2) * size_t(M) * size_t(N) * sizeof(T), s);
    }
    cudaError_t e = launch_complex_epilogue<T>(M, N, Pr, Pi, ar, ai, br, bi, dC, ldc, s);
    if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("complex epilogue: ") + cudaGetErrorString(e));
    if (!cdev && (e = unstage(C, dC, M, N, ldc, 2 * sizeof(T), s)) != cudaSuccess)
        return fail(GB300_ERR_CUDA, std::string("copy of C back: ") + cudaGetErrorString(e));
    st = finish(s, &err);
    return st == GB300_OK ? GB300_OK : fail(st, err);
}

// ---- trmm --------------------------------------------------------------------------------------
template <typename T>
int trmm_entry(int order, int side, int uplo, int transA, int diag, int64_t m, int64_t n, T alpha, const T* A,
               int64_t lda, T* B, int64_t ldb, const char* routine) {
    auto fail = [&](int st, const std::string& msg) {
        set_error(st, std::string(routine) + ": " + msg);
        return st;
    };
    if (order != CblasRowMajor && order != CblasColMajor) return fail(GB300_ERR_INVALID_ARG, "parameter 1 (order) is invalid");
    if (side != CblasLeft && side != CblasRight) return fail(GB300_ERR_INVALID_ARG, "parameter 2 (side) is invalid");
    if (uplo != CblasUpper && uplo != CblasLower) return fail(GB300_ERR_INVALID_ARG, "parameter 3 (uplo) is invalid");
    if (transA != CblasNoTrans && transA != CblasTrans && transA != CblasConjTrans)
        return fail(GB300_ERR_INVALID_ARG, "parameter 4 (transA) is invalid");
    if (diag != CblasUnit && diag != CblasNonUnit) return fail(GB300_ERR_INVALID_ARG, "parameter 5 (diag) is invalid");
    if (m < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 6 (m) is negative");
    if (n < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 7 (n) is negative");
    const bool rm = order == CblasRowMajor, left = side == CblasLeft, ta = transA != CblasNoTrans;
    const int64_t ka = left ? m : n;
    if (lda < std::max<int64_t>(1, ka)) return fail(GB300_ERR_INVALID_ARG, "parameter 10 (lda) is too small");
    if (ldb < std::max<int64_t>(1, rm ? n : m)) return fail(GB300_ERR_INVALID_ARG, "parameter 12 (ldb) is too small");
    clear_error();
    if (m == 0 || n == 0) return GB300_OK;
    if (B == nullptr || (alpha != T(0) && A == nullptr)) return fail(GB300_ERR_INVALID_ARG, "A or B is NULL");

    Runtime& r = runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = ensure_init(&err);
    if (st != GB300_OK) return fail(st, err);
    cudaStream_t s = r.stream;
    const LaunchCtl ctl = fresh_ctl(s);

    // row-major storage: SB = B (m x n) or B^T (n x m); SA = A or A^T, whose triangle flips for
    // column-major.  Left / right swap for column-major: B = op(A) B becomes SB = SB op(SA).
    const int64_t sbr = rm ? m : n, sbc = rm ? n : m;
    const bool lower = rm ? (uplo == CblasLower) : (uplo == CblasUpper);
    const bool sa_left = rm ? left : !left;
    const bool bdev = on_device(B);
    T* dB = static_cast<T*>(stage(B, sbr, sbc, ldb, sizeof(T), kAuxB, bdev, s, &err));
    T* tmp = static_cast<T*>(r.aux.get(kAuxP, size_t(sbr) * size_t(sbc) * sizeof(T), &err));
    if (!dB || !tmp) return fail(GB300_ERR_NO_MEMORY, err);
    Gemm g;
    g.m = sbr; g.n = sbc; g.C = tmp; g.ldc = sbc; g.alpha = double(alpha); g.beta = 0.0;
    if (alpha == T(0)) {
        g.k = 0;  // B = 0 without reading A
        g.A = dB; g.lda = sbc; g.B = dB; g.ldb = sbc;
    } else {
        const T* dA = static_cast<const T*>(stage(A, ka, ka, lda, sizeof(T), kAuxA, on_device(A), s, &err));
        T* tri = static_cast<T*>(r.aux.get(kAuxAr, size_t(ka) * size_t(ka) * sizeof(T), &err));
        if (!dA || !tri) return fail(GB300_ERR_NO_MEMORY, err);
        cudaError_t e = launch_triangle<T>(ka, dA, lda, lower, diag == CblasUnit, tri, s);
        if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("triangle: ") + cudaGetErrorString(e));
        g.k = ka;
        if (sa_left) {  // SB = op(T) SB
            g.ta = ta; g.tb = false;
            g.A = tri; g.lda = ka; g.B = dB; g.ldb = ldb;
        } else {  // SB = SB op(T)
            g.ta = false; g.tb = ta;
            g.A = dB; g.lda = ldb; g.B = tri; g.ldb = ka;
        }
    }
    if ((st = real_product<T>(g, ctl, s, &err)) != GB300_OK) return fail(st, err);
    // the product back into B (its pitch)
    cudaError_t e = cudaMemcpy2DAsync(bdev ? static_cast<void*>(B) : static_cast<void*>(dB), size_t(ldb) * sizeof(T), tmp,
                                      size_t(sbc) * sizeof(T), size_t(sbc) * sizeof(T), size_t(sbr),
                                      cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && !bdev) e = unstage(B, dB, sbr, sbc, ldb, sizeof(T), s);
    if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("copy of B back: ") + cudaGetErrorString(e));
    st = finish(s, &err);
    return st == GB300_OK ? GB300_OK : fail(st, err);
}

template int gemv_entry<double>(int, int, int64_t, int64_t, double, const double*, int64_t, const double*, int64_t,
                                double, double*, int64_t, const char*);
template int gemv_entry<float>(int, int, int64_t, int64_t, float, const float*, int64_t, const float*, int64_t, float,
                               float*, int64_t, const char*);
template int cgemm_entry<double>(int, int, int, int64_t, int64_t, int64_t, const double*, const double*, int64_t,
                                 const double*, int64_t, const double*, double*, int64_t, const char*);
template int cgemm_entry<float>(int, int, int, int64_t, int64_t, int64_t, const float*, const float*, int64_t,
                                const float*, int64_t, const float*, float*, int64_t, const char*);
template int trmm_entry<double>(int, int, int, int, int, int64_t, int64_t, double, const double*, int64_t, double*,
                                int64_t, const char*);
template int trmm_entry<float>(int, int, int, int, int, int64_t, int64_t, float, const float*, int64_t, float*, int64_t,
                               const char*);
}  // namespace gb
