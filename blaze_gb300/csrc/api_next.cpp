// api_next.cpp — the BLAS routines next to ?gemm on Blaze's seam, on the GPU:
//
//   cblas_?gemv   y = alpha op(A) x + beta y (real and complex)
//                                                     blaze/math/blas/cblas/gemv.h:116-235
//   cblas_?trmv   x = op(A) x, A triangular (real and complex)
//                                                     blaze/math/blas/cblas/trmv.h:111-218
//   cblas_zgemm / cblas_cgemm  complex C = alpha op(A) op(B) + beta C
//                                                     blaze/math/blas/cblas/gemm.h:196-256
//   cblas_?trmm   B = alpha op(A) B or alpha B op(A), A triangular (real and complex)
//                                                     blaze/math/blas/cblas/trmm.h:116-235
//   cblas_?trsm   B = alpha op(A)^-1 B or alpha B op(A)^-1 (real and complex)
//                                                     blaze/math/blas/cblas/trsm.h:111-236
//   cblas_?axpy   y = alpha x + y                     blaze/math/blas/cblas/axpy.h:100-200
//   cblas_?dot, cblas_?dotu_sub, cblas_?dotc_sub      blaze/math/blas/cblas/dotu.h:97-210,
//                                                     blaze/math/blas/cblas/dotc.h:97-210
//
// Semantics follow CBLAS (argument positions as in xerbla, quick returns, beta == 0 does not read
// the output, alpha == 0 does not read the inputs).  A complex product is one real product of the
// stacked real and imaginary planes, whose four quadrants combine into the result (a conjugate
// transpose flips the sign of an imaginary part), through the library's real product:
// FP64-accurate split precision for double by default, the native kernel for float.  A triangular product runs on a dense copy of the triangle (zeros
// elsewhere, ones on a unit diagonal); a triangular matrix x vector product masks the triangle in
// the matrix x vector kernel itself.  Host operands are staged through device buffers; device or
// managed operands are used in place (complex ones when 2 * sizeof(T)-aligned, else copied).
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
enum AuxSlot : int { kAuxA = 0, kAuxB, kAuxC, kAuxX, kAuxY, kAuxAr, kAuxBr, kAuxP, kAuxT };
static_assert(kAuxT < kSlotCount, "aux slots");

// A device or managed operand aligned for `elem`-byte element loads is used in place.
bool in_place(const void* p, size_t elem) {
    return on_device(p) && reinterpret_cast<uintptr_t>(p) % elem == 0;
}

// Device copy of `rows` x `cols` elements (pitch ld, elem bytes each) of a host or device buffer into
// aux slot `slot` with the same pitch; returns the device pointer (or the buffer itself when `dev`:
// it is used in place).
void* stage(const void* p, int64_t rows, int64_t cols, int64_t ld, size_t elem, int slot, bool dev, cudaStream_t st,
            std::string* err) {
    if (dev || rows == 0 || cols == 0) return const_cast<void*>(p);
    const size_t bytes = (size_t(std::max<int64_t>(rows - 1, 0)) * size_t(ld) + size_t(cols)) * elem;
    void* d = runtime().aux.get(slot, bytes, err);
    if (!d) return nullptr;
    const cudaError_t e = cudaMemcpy2DAsync(d, size_t(ld) * elem, p, size_t(ld) * elem, size_t(cols) * elem,
                                            size_t(rows), cudaMemcpyDefault, st);
    if (e != cudaSuccess) {
        if (err) *err = std::string("operand copy: ") + cudaGetErrorString(e);
        return nullptr;
    }
    return d;
}

// The staged copy back into the caller's buffer (host, or a device buffer that was not used in
// place): one linear copy when the rows are contiguous (see copy_to_host).
cudaError_t unstage(void* dst, const void* dev, int64_t rows, int64_t cols, int64_t ld, size_t elem, cudaStream_t st) {
    if (rows == 0 || cols == 0) return cudaSuccess;
    if (rows == 1 || ld == cols)
        return cudaMemcpyAsync(dst, dev, size_t(rows) * size_t(cols) * elem, cudaMemcpyDefault, st);
    return cudaMemcpy2DAsync(dst, size_t(ld) * elem, dev, size_t(ld) * elem, size_t(cols) * elem, size_t(rows),
                             cudaMemcpyDefault, st);
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

// ---- gemv / trmv ------------------------------------------------------------------------------
namespace {
// alpha / beta as (re, im) for complex, one value for real
template <typename T, bool CPLX>
bool scalar_is(const T* v, T re) {
    return v[0] == re && (!CPLX || v[1] == T(0));
}
}  // namespace

template <typename T, bool CPLX>
int gemv_any(int order, int transA, int64_t m, int64_t n, const T* alpha, const T* A, int64_t lda, const T* x,
             int64_t incx, const T* beta, T* y, int64_t incy, const char* routine) {
    const CallTrace trace(routine, m, n, 1);
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
    if (alpha == nullptr || beta == nullptr) return fail(GB300_ERR_INVALID_ARG, "alpha or beta is NULL");
    clear_error();
    const bool alpha0 = scalar_is<T, CPLX>(alpha, T(0));
    if (m == 0 || n == 0 || (alpha0 && scalar_is<T, CPLX>(beta, T(1)))) return GB300_OK;
    if (y == nullptr) return fail(GB300_ERR_INVALID_ARG, "parameter 11 (y) is NULL");
    if (!alpha0 && (A == nullptr || x == nullptr)) return fail(GB300_ERR_INVALID_ARG, "A or x is NULL");

    Runtime& r = runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = ensure_init(&err);
    if (st != GB300_OK) return fail(st, err);
    cudaStream_t s = r.stream;
    fresh_ctl(s);

    const size_t elem = (CPLX ? 2 : 1) * sizeof(T);
    const int64_t w = CPLX ? 2 : 1;  // T values per element
    // stored row-major S: A itself (row-major, m x n) or A^T (column-major, n x m)
    const int64_t srows = rm ? m : n, scols = rm ? n : m;
    const int64_t xl = ta ? m : n, yl = ta ? n : m;
    const bool use_a = !alpha0;
    const T* dS = A;
    if (use_a) {
        dS = static_cast<const T*>(stage(A, srows, scols, lda, elem, kAuxA, in_place(A, elem), s, &err));
        if (!dS) return fail(GB300_ERR_NO_MEMORY, err);
    }
    const int64_t ax = incx < 0 ? -incx : incx, ay = incy < 0 ? -incy : incy;
    const T* dx = x;
    if (use_a) {
        dx = static_cast<const T*>(stage(x, 1, 1 + (xl - 1) * ax, 1 + (xl - 1) * ax, elem, kAuxX, in_place(x, elem), s, &err));
        if (!dx) return fail(GB300_ERR_NO_MEMORY, err);
    }
    const bool ydev = in_place(y, elem);
    T* dy = static_cast<T*>(stage(y, 1, 1 + (yl - 1) * ay, 1 + (yl - 1) * ay, elem, kAuxY, ydev, s, &err));
    if (!dy) return fail(GB300_ERR_NO_MEMORY, err);
    // logical element j of a strided vector: base + j * inc, the base at the far end for inc < 0
    const T* xb = dx + (incx < 0 ? (xl - 1) * ax : 0) * w;
    T* yb = dy + (incy < 0 ? (yl - 1) * ay : 0) * w;
    MvForm f;
    f.cols_form = use_a && (rm ? ta : !ta);  // y = S x (rows form) or y = S^T x (cols form)
    f.conj = CPLX && transA == CblasConjTrans;
    const int64_t rows = f.cols_form ? srows : yl, cols = f.cols_form ? yl : (use_a ? scols : 0);
    int slices = 1;
    T* part = nullptr;
    if (f.cols_form) {
        slices = mv_cols_slices<T, CPLX>(srows, yl);
        part = static_cast<T*>(r.aux.get(kAuxP, size_t(slices) * size_t(yl) * elem, &err));
        if (!part) return fail(GB300_ERR_NO_MEMORY, err);
    }
    cudaError_t e = launch_mv<T, CPLX>(f, rows, cols, alpha, dS, lda, xb, incx, beta, yb, incy, part, slices, s);
    if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("gemv launch: ") + cudaGetErrorString(e));
    if (!ydev && (e = unstage(y, dy, 1, 1 + (yl - 1) * ay, 1 + (yl - 1) * ay, elem, s)) != cudaSuccess)
        return fail(GB300_ERR_CUDA, std::string("copy of y back: ") + cudaGetErrorString(e));
    st = finish(s, &err);
    return st == GB300_OK ? GB300_OK : fail(st, err);
}

template <typename T>
int gemv_entry(int order, int transA, int64_t m, int64_t n, T alpha, const T* A, int64_t lda, const T* x,
               int64_t incx, T beta, T* y, int64_t incy, const char* routine) {
    return gemv_any<T, false>(order, transA, m, n, &alpha, A, lda, x, incx, &beta, y, incy, routine);
}

template <typename T>
int cgemv_entry(int order, int transA, int64_t m, int64_t n, const T* alpha, const T* A, int64_t lda, const T* x,
                int64_t incx, const T* beta, T* y, int64_t incy, const char* routine) {
    return gemv_any<T, true>(order, transA, m, n, alpha, A, lda, x, incx, beta, y, incy, routine);
}

// x = op(A) x with A n x n triangular: the matrix x vector kernel over the triangle only (the
// other half is not read), into a copy of x's span that then replaces x.
template <typename T, bool CPLX>
int trmv_entry(int order, int uplo, int transA, int diag, int64_t n, const T* A, int64_t lda, T* x, int64_t incx,
               const char* routine) {
    const CallTrace trace(routine, n, n, 1);
    auto fail = [&](int st, const std::string& msg) {
        set_error(st, std::string(routine) + ": " + msg);
        return st;
    };
    if (order != CblasRowMajor && order != CblasColMajor) return fail(GB300_ERR_INVALID_ARG, "parameter 1 (order) is invalid");
    if (uplo != CblasUpper && uplo != CblasLower) return fail(GB300_ERR_INVALID_ARG, "parameter 2 (uplo) is invalid");
    if (transA != CblasNoTrans && transA != CblasTrans && transA != CblasConjTrans)
        return fail(GB300_ERR_INVALID_ARG, "parameter 3 (transA) is invalid");
    if (diag != CblasUnit && diag != CblasNonUnit) return fail(GB300_ERR_INVALID_ARG, "parameter 4 (diag) is invalid");
    if (n < 0) return fail(GB300_ERR_INVALID_ARG, "parameter 5 (n) is negative");
    if (lda < std::max<int64_t>(1, n)) return fail(GB300_ERR_INVALID_ARG, "parameter 7 (lda) is too small");
    if (incx == 0) return fail(GB300_ERR_INVALID_ARG, "parameter 9 (incx) is zero");
    clear_error();
    if (n == 0) return GB300_OK;
    if (A == nullptr || x == nullptr) return fail(GB300_ERR_INVALID_ARG, "A or x is NULL");

    Runtime& r = runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = ensure_init(&err);
    if (st != GB300_OK) return fail(st, err);
    cudaStream_t s = r.stream;
    fresh_ctl(s);

    const size_t elem = (CPLX ? 2 : 1) * sizeof(T);
    const int64_t w = CPLX ? 2 : 1;
    const bool rm = order == CblasRowMajor, ta = transA != CblasNoTrans;
    MvForm f;
    f.cols_form = rm ? ta : !ta;
    // S = A (row-major) or A^T (column-major), whose triangle is the other one
    f.tri = (rm ? uplo == CblasLower : uplo == CblasUpper) ? 1 : 2;
    f.unit = diag == CblasUnit;
    f.conj = CPLX && transA == CblasConjTrans;
    const T* dS = static_cast<const T*>(stage(A, n, n, lda, elem, kAuxA, in_place(A, elem), s, &err));
    if (!dS) return fail(GB300_ERR_NO_MEMORY, err);
    const int64_t ax = incx < 0 ? -incx : incx, span = 1 + (n - 1) * ax;
    const bool xdev = in_place(x, elem);
    const T* dx = static_cast<const T*>(stage(x, 1, span, span, elem, kAuxX, xdev, s, &err));
    T* tmp = static_cast<T*>(r.aux.get(kAuxY, size_t(span) * elem, &err));
    if (!dx || !tmp) return fail(GB300_ERR_NO_MEMORY, err);
    cudaError_t e = cudaMemcpyAsync(tmp, dx, size_t(span) * elem, cudaMemcpyDeviceToDevice, s);  // keeps the gaps
    const int64_t off = (incx < 0 ? (n - 1) * ax : 0) * w;
    int slices = 1;
    T* part = nullptr;
    if (f.cols_form) {
        slices = mv_cols_slices<T, CPLX>(n, n);
        part = static_cast<T*>(r.aux.get(kAuxP, size_t(slices) * size_t(n) * elem, &err));
        if (!part) return fail(GB300_ERR_NO_MEMORY, err);
    }
    const T one[2] = {T(1), T(0)}, zero[2] = {T(0), T(0)};
    if (e == cudaSuccess)
        e = launch_mv<T, CPLX>(f, n, n, one, dS, lda, dx + off, incx, zero, tmp + off, incx, part, slices, s);
    if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("trmv launch: ") + cudaGetErrorString(e));
    if ((e = unstage(x, tmp, 1, span, span, elem, s)) != cudaSuccess)
        return fail(GB300_ERR_CUDA, std::string("copy of x back: ") + cudaGetErrorString(e));
    st = finish(s, &err);
    return st == GB300_OK ? GB300_OK : fail(st, err);
}

// ---- complex gemm ------------------------------------------------------------------------------
namespace {
// C (M x N interleaved complex, device, pitch ldc) = alpha op(A) op(B) + beta C in the logical
// row-major form.  A and B are device interleaved complex operands in their stored shapes (pitches
// la, lb); ca / cb conjugate an operand.  product == false (alpha == 0 or k == 0): C = beta C with
// A and B not read.
//
// The four real products are one: the planes are laid out as [op(Ar); op(Ai)] (2M x k) and
// [op(Br), op(Bi)] (k x 2N), so the library's real product of the two gives all four quadrants
// (2M x 2N) at once.  Each operand is analysed and sliced once instead of twice, the fixed costs of
// a product are paid once, and the larger product fills more tiles.  In stored terms, an untransposed
// A keeps its planes one below the other and a transposed one side by side; for B it is the other
// way round.  Its error bound is relative to the complex Frobenius norms ||A|| ||B||.
template <typename T>
int complex_product(int64_t M, int64_t N, int64_t k, bool ta, bool tb, bool ca, bool cb, const T* dA, int64_t la,
                    const T* dB, int64_t lb, const T* alpha, const T* beta, T* dC, int64_t ldc, bool product,
                    const LaunchCtl& ctl, cudaStream_t s, std::string* err) {
    Runtime& r = runtime();
    T* P = static_cast<T*>(r.aux.get(kAuxP, size_t(4) * size_t(M) * size_t(N) * sizeof(T), err));
    if (!P) return GB300_ERR_NO_MEMORY;
    if (product) {
        const int64_t ra = ta ? k : M, cA = ta ? M : k;  // stored shapes
        const int64_t rb = tb ? N : k, cB = tb ? k : N;
        T* A2 = static_cast<T*>(r.aux.get(kAuxAr, size_t(2) * size_t(ra) * size_t(cA) * sizeof(T), err));
        T* B2 = static_cast<T*>(r.aux.get(kAuxBr, size_t(2) * size_t(rb) * size_t(cB) * sizeof(T), err));
        if (!A2 || !B2) return GB300_ERR_NO_MEMORY;
        const int64_t la2 = ta ? 2 * cA : cA, lb2 = tb ? cB : 2 * cB;
        cudaError_t e = launch_split_complex<T>(ra, cA, dA, la, A2, ta ? A2 + cA : A2 + ra * cA, la2, s);
        if (e == cudaSuccess) e = launch_split_complex<T>(rb, cB, dB, lb, B2, tb ? B2 + rb * cB : B2 + cB, lb2, s);
        if (e != cudaSuccess) {
            if (err) *err = std::string("complex split: ") + cudaGetErrorString(e);
            return GB300_ERR_CUDA;
        }
        Gemm g;
        g.m = 2 * M; g.n = 2 * N; g.k = k; g.ta = ta; g.tb = tb;
        g.A = A2; g.lda = la2; g.B = B2; g.ldb = lb2; g.C = P; g.ldc = 2 * N;
        g.alpha = 1.0; g.beta = 0.0;
        const int st = real_product<T>(g, ctl, s, err);
        if (st != GB300_OK) return st;
    } else {
        cudaMemsetAsync(P, 0, size_t(4) * size_t(M) * size_t(N) * sizeof(T), s);
    }
    const cudaError_t e = launch_complex_quadrants<T>(M, N, P, product && ca, product && cb, alpha[0], alpha[1],
                                                      beta[0], beta[1], dC, ldc, s);
    if (e != cudaSuccess) {
        if (err) *err = std::string("complex epilogue: ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    return GB300_OK;
}
}  // namespace

template <typename T>
int cgemm_entry(int order, int transA, int transB, int64_t m, int64_t n, int64_t k, const T* alpha, const T* A,
                int64_t lda, const T* B, int64_t ldb, const T* beta, T* C, int64_t ldc, const char* routine) {
    const CallTrace trace(routine, m, n, k);
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
    clear_error();
    const bool alpha0 = scalar_is<T, true>(alpha, T(0)), beta1 = scalar_is<T, true>(beta, T(1));
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
    const size_t elem = 2 * sizeof(T);

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
    // C: row-major M x N (pitch ldc) in either case
    const bool cdev = in_place(C, elem);
    T* dC = static_cast<T*>(stage(C, M, N, ldc, elem, kAuxC, cdev, s, &err));
    if (!dC) return fail(GB300_ERR_NO_MEMORY, err);
    const T* dA = nullptr;
    const T* dB = nullptr;
    if (product) {
        dA = static_cast<const T*>(stage(pA, ta ? k : M, ta ? M : k, la, elem, kAuxA, in_place(pA, elem), s, &err));
        dB = static_cast<const T*>(stage(pB, tb ? N : k, tb ? k : N, lb, elem, kAuxB, in_place(pB, elem), s, &err));
        if (!dA || !dB) return fail(GB300_ERR_NO_MEMORY, err);
    }
    st = complex_product<T>(M, N, k, ta, tb, ca, cb, dA, la, dB, lb, alpha, beta, dC, ldc, product, ctl, s, &err);
    if (st != GB300_OK) return fail(st, err);
    cudaError_t e;
    if (!cdev && (e = unstage(C, dC, M, N, ldc, elem, s)) != cudaSuccess)
        return fail(GB300_ERR_CUDA, std::string("copy of C back: ") + cudaGetErrorString(e));
    st = finish(s, &err);
    return st == GB300_OK ? GB300_OK : fail(st, err);
}

// ---- trmm --------------------------------------------------------------------------------------
template <typename T>
int trmm_entry(int order, int side, int uplo, int transA, int diag, int64_t m, int64_t n, T alpha, const T* A,
               int64_t lda, T* B, int64_t ldb, const char* routine) {
    const CallTrace trace(routine, m, n, side == CblasLeft ? m : n);
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
    const bool bdev = in_place(B, sizeof(T));
    T* dB = static_cast<T*>(stage(B, sbr, sbc, ldb, sizeof(T), kAuxB, bdev, s, &err));
    T* tmp = static_cast<T*>(r.aux.get(kAuxP, size_t(sbr) * size_t(sbc) * sizeof(T), &err));
    if (!dB || !tmp) return fail(GB300_ERR_NO_MEMORY, err);
    Gemm g;
    g.m = sbr; g.n = sbc; g.C = tmp; g.ldc = sbc; g.alpha = double(alpha); g.beta = 0.0;
    if (alpha == T(0)) {
        g.k = 0;  // B = 0 without reading A
        g.A = dB; g.lda = sbc; g.B = dB; g.ldb = sbc;
    } else {
        const T* dA = static_cast<const T*>(stage(A, ka, ka, lda, sizeof(T), kAuxA, in_place(A, sizeof(T)), s, &err));
        T* tri = static_cast<T*>(r.aux.get(kAuxAr, size_t(ka) * size_t(ka) * sizeof(T), &err));
        if (!dA || !tri) return fail(GB300_ERR_NO_MEMORY, err);
        cudaError_t e = launch_triangle<T, false>(ka, dA, lda, lower, diag == CblasUnit, tri, s);
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

// Complex B = alpha op(A) B or alpha B op(A), A triangular: the masked complex triangle and one
// complex product.
template <typename T>
int ctrmm_entry(int order, int side, int uplo, int transA, int diag, int64_t m, int64_t n, const T* alpha, const T* A,
                int64_t lda, T* B, int64_t ldb, const char* routine) {
    const CallTrace trace(routine, m, n, side == CblasLeft ? m : n);
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
    if (alpha == nullptr) return fail(GB300_ERR_INVALID_ARG, "parameter 8 (alpha) is NULL");
    clear_error();
    if (m == 0 || n == 0) return GB300_OK;
    const bool alpha0 = scalar_is<T, true>(alpha, T(0));
    if (B == nullptr || (!alpha0 && A == nullptr)) return fail(GB300_ERR_INVALID_ARG, "A or B is NULL");

    Runtime& r = runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = ensure_init(&err);
    if (st != GB300_OK) return fail(st, err);
    cudaStream_t s = r.stream;
    const LaunchCtl ctl = fresh_ctl(s);
    const size_t elem = 2 * sizeof(T);

    // as for the real case: SB = B or B^T in row-major storage, the triangle flips for column-major
    // and so does the side; a conjugate transpose conjugates the triangle's elements
    const int64_t sbr = rm ? m : n, sbc = rm ? n : m;
    const bool lower = rm ? (uplo == CblasLower) : (uplo == CblasUpper);
    const bool sa_left = rm ? left : !left;
    const bool conj = transA == CblasConjTrans;
    const bool bdev = in_place(B, elem);
    T* dB = static_cast<T*>(stage(B, sbr, sbc, ldb, elem, kAuxB, bdev, s, &err));
    T* tmp = static_cast<T*>(r.aux.get(kAuxC, size_t(sbr) * size_t(sbc) * elem, &err));
    if (!dB || !tmp) return fail(GB300_ERR_NO_MEMORY, err);
    const T zero[2] = {T(0), T(0)};
    if (alpha0) {
        st = complex_product<T>(sbr, sbc, 0, false, false, false, false, nullptr, 1, nullptr, 1, alpha, zero, tmp, sbc,
                                false, ctl, s, &err);
    } else {
        const T* dA = static_cast<const T*>(stage(A, ka, ka, lda, elem, kAuxA, in_place(A, elem), s, &err));
        T* tri = static_cast<T*>(r.aux.get(kAuxT, size_t(ka) * size_t(ka) * elem, &err));
        if (!dA || !tri) return fail(GB300_ERR_NO_MEMORY, err);
        cudaError_t e = launch_triangle<T, true>(ka, dA, lda, lower, diag == CblasUnit, tri, s);
        if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("triangle: ") + cudaGetErrorString(e));
        if (sa_left)  // SB = op(T) SB
            st = complex_product<T>(sbr, sbc, ka, ta, false, conj, false, tri, ka, dB, ldb, alpha, zero, tmp, sbc, true,
                                    ctl, s, &err);
        else  // SB = SB op(T)
            st = complex_product<T>(sbr, sbc, ka, false, ta, false, conj, dB, ldb, tri, ka, alpha, zero, tmp, sbc, true,
                                    ctl, s, &err);
    }
    if (st != GB300_OK) return fail(st, err);
    cudaError_t e = cudaMemcpy2DAsync(bdev ? static_cast<void*>(B) : static_cast<void*>(dB), size_t(ldb) * elem, tmp,
                                      size_t(sbc) * elem, size_t(sbc) * elem, size_t(sbr), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && !bdev) e = unstage(B, dB, sbr, sbc, ldb, elem, s);
    if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("copy of B back: ") + cudaGetErrorString(e));
    st = finish(s, &err);
    return st == GB300_OK ? GB300_OK : fail(st, err);
}

// ---- axpy and the dot products -----------------------------------------------------------------
// y = alpha x + y over n elements of strided vectors (CBLAS: n <= 0 or alpha == 0 leave y as it is).
template <typename T, bool CPLX>
int axpy_entry(int64_t n, const T* alpha, const T* x, int64_t incx, T* y, int64_t incy, const char* routine) {
    const CallTrace trace(routine, n, 1, 1);
    auto fail = [&](int st, const std::string& msg) {
        set_error(st, std::string(routine) + ": " + msg);
        return st;
    };
    if (alpha == nullptr) return fail(GB300_ERR_INVALID_ARG, "parameter 2 (alpha) is NULL");
    clear_error();
    if (n <= 0 || scalar_is<T, CPLX>(alpha, T(0))) return GB300_OK;
    if (x == nullptr || y == nullptr) return fail(GB300_ERR_INVALID_ARG, "x or y is NULL");

    Runtime& r = runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = ensure_init(&err);
    if (st != GB300_OK) return fail(st, err);
    cudaStream_t s = r.stream;
    fresh_ctl(s);
    const size_t elem = (CPLX ? 2 : 1) * sizeof(T);
    const int64_t w = CPLX ? 2 : 1;
    const int64_t ax = incx < 0 ? -incx : incx, ay = incy < 0 ? -incy : incy;
    const int64_t xspan = 1 + (n - 1) * ax, yspan = 1 + (n - 1) * ay;
    const T* dx = static_cast<const T*>(stage(x, 1, xspan, xspan, elem, kAuxX, in_place(x, elem), s, &err));
    const bool ydev = in_place(y, elem);
    T* dy = dx ? static_cast<T*>(stage(y, 1, yspan, yspan, elem, kAuxY, ydev, s, &err)) : nullptr;
    if (!dx || !dy) return fail(GB300_ERR_NO_MEMORY, err);
    // logical element 0 sits at the far end of a vector with a negative stride
    cudaError_t e = launch_axpy<T, CPLX>(n, alpha, dx + (incx < 0 ? (n - 1) * ax : 0) * w, incx,
                                         dy + (incy < 0 ? (n - 1) * ay : 0) * w, incy, s);
    if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("axpy launch: ") + cudaGetErrorString(e));
    if (!ydev && (e = unstage(y, dy, 1, yspan, yspan, elem, s)) != cudaSuccess)
        return fail(GB300_ERR_CUDA, std::string("copy of y back: ") + cudaGetErrorString(e));
    st = finish(s, &err);
    return st == GB300_OK ? GB300_OK : fail(st, err);
}

// *result = sum_i op(x_i) y_i (op = conjugation when CONJ), summed in double precision in a fixed
// order and rounded once to T; n <= 0 gives zero.
template <typename T, bool CPLX, bool CONJ>
int dot_entry(int64_t n, const T* x, int64_t incx, const T* y, int64_t incy, T* result, const char* routine) {
    const CallTrace trace(routine, n, 1, 1);
    auto fail = [&](int st, const std::string& msg) {
        set_error(st, std::string(routine) + ": " + msg);
        return st;
    };
    if (result == nullptr) return fail(GB300_ERR_INVALID_ARG, "the result pointer is NULL");
    result[0] = T(0);
    if (CPLX) result[1] = T(0);
    clear_error();
    if (n <= 0) return GB300_OK;
    if (x == nullptr || y == nullptr) return fail(GB300_ERR_INVALID_ARG, "x or y is NULL");

    Runtime& r = runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = ensure_init(&err);
    if (st != GB300_OK) return fail(st, err);
    cudaStream_t s = r.stream;
    fresh_ctl(s);
    const size_t elem = (CPLX ? 2 : 1) * sizeof(T);
    const int64_t w = CPLX ? 2 : 1;
    const int64_t ax = incx < 0 ? -incx : incx, ay = incy < 0 ? -incy : incy;
    const int64_t xspan = 1 + (n - 1) * ax, yspan = 1 + (n - 1) * ay;
    const T* dx = static_cast<const T*>(stage(x, 1, xspan, xspan, elem, kAuxX, in_place(x, elem), s, &err));
    const T* dy = dx ? static_cast<const T*>(stage(y, 1, yspan, yspan, elem, kAuxY, in_place(y, elem), s, &err))
                     : nullptr;
    const int parts = dot_parts(n);
    double* part = static_cast<double*>(r.aux.get(kAuxP, size_t(parts + 1) * size_t(w) * sizeof(double), &err));
    if (!dx || !dy || !part) return fail(GB300_ERR_NO_MEMORY, err);
    double* out = part + size_t(parts) * size_t(w);
    cudaError_t e = launch_dot<T, CPLX, CONJ>(n, dx + (incx < 0 ? (n - 1) * ax : 0) * w, incx,
                                              dy + (incy < 0 ? (n - 1) * ay : 0) * w, incy, part, out, s);
    if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("dot launch: ") + cudaGetErrorString(e));
    st = finish(s, &err);
    if (st != GB300_OK) return fail(st, err);
    double v[2] = {0.0, 0.0};
    if ((e = cudaMemcpy(v, out, size_t(w) * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return fail(GB300_ERR_CUDA, std::string("copy of the result: ") + cudaGetErrorString(e));
    result[0] = T(v[0]);
    if (CPLX) result[1] = T(v[1]);
    return GB300_OK;
}

// ---- trsm --------------------------------------------------------------------------------------
namespace {
// A triangular system in row-major storage: op(SA) X = SB (left) or X op(SA) = SB (right), X
// overwriting SB (sbr x sbc, pitch ldb); SA ka x ka (pitch lda), `lower` its stored triangle.
struct SolveForm {
    bool left = true, lower = true, trans = false, conj = false, unit = false;
};

// Recursive blocked solve.  [lo, hi) is a range of op(SA)'s rows and columns whose right-hand sides
// (rows of SB when left, columns when right) are to be solved.  It is halved at a multiple of the
// leaf size solve_block().  The half whose unknowns do not depend on the other is solved first, then one
// product subtracts its contribution from the other half's right-hand sides (alpha = -1,
// beta = 1), then the other half is solved.  A range of at most one leaf is multiplied by its
// block's inverse, into `tmp` and copied back.
template <typename T, bool CPLX>
int solve_range(const SolveForm& f, int64_t lo, int64_t hi, int64_t sbr, int64_t sbc, const T* SA, int64_t lda,
                T* SB, int64_t ldb, const T* inv, T* tmp, const LaunchCtl& ctl, cudaStream_t s, std::string* err) {
    const int64_t w = CPLX ? 2 : 1;
    const size_t elem = size_t(w) * sizeof(T);
    const int nb = solve_block(elem);
    // C (M x N, pitch ldc) = -X Y + C (update) or X Y (leaf); X and Y stored at pitches lx / ly
    auto product = [&](int64_t M, int64_t N, int64_t K, bool tx, bool ty, bool cx, bool cy, const T* X, int64_t lx,
                       const T* Y, int64_t ly, bool update, T* C, int64_t ldc) -> int {
        if (CPLX) {
            const T one[2] = {T(1), T(0)}, zero[2] = {T(0), T(0)}, minus[2] = {T(-1), T(0)};
            return complex_product<T>(M, N, K, tx, ty, cx, cy, X, lx, Y, ly, update ? minus : one,
                                      update ? one : zero, C, ldc, true, ctl, s, err);
        }
        Gemm g;
        g.m = M; g.n = N; g.k = K; g.ta = tx; g.tb = ty;
        g.A = X; g.lda = lx; g.B = Y; g.ldb = ly; g.C = C; g.ldc = ldc;
        g.alpha = update ? -1.0 : 1.0;
        g.beta = update ? 1.0 : 0.0;
        return real_product<T>(g, ctl, s, err);
    };
    // the block of op(SA) at rows i0.., columns j0.. as a product operand (stored transposed when
    // op transposes)
    auto block = [&](int64_t i0, int64_t j0) { return SA + (f.trans ? j0 * lda + i0 : i0 * lda + j0) * w; };
    auto rows_of = [&](int64_t i) { return SB + i * ldb * w; };  // left: right-hand sides are rows
    auto cols_of = [&](int64_t j) { return SB + j * w; };        // right: they are columns
    if (hi - lo <= nb) {
        const int64_t nk = hi - lo;
        const T* Ib = inv + (lo / nb) * int64_t(nb) * nb * w;
        int st;
        cudaError_t e;
        if (f.left) {
            if ((st = product(nk, sbc, nk, false, false, false, false, Ib, nb, rows_of(lo), ldb, false, tmp, sbc)) != GB300_OK)
                return st;
            e = cudaMemcpy2DAsync(rows_of(lo), size_t(ldb) * elem, tmp, size_t(sbc) * elem, size_t(sbc) * elem,
                                  size_t(nk), cudaMemcpyDeviceToDevice, s);
        } else {
            if ((st = product(sbr, nk, nk, false, false, false, false, cols_of(lo), ldb, Ib, nb, false, tmp, nk)) != GB300_OK)
                return st;
            e = cudaMemcpy2DAsync(cols_of(lo), size_t(ldb) * elem, tmp, size_t(nk) * elem, size_t(nk) * elem,
                                  size_t(sbr), cudaMemcpyDeviceToDevice, s);
        }
        if (e != cudaSuccess) {
            if (err) *err = std::string("solve copy: ") + cudaGetErrorString(e);
            return GB300_ERR_CUDA;
        }
        return GB300_OK;
    }
    const int64_t blocks = (hi - lo + nb - 1) / nb, h = lo + int64_t(nb) * ((blocks + 1) / 2);
    const bool eff_lower = f.lower != f.trans;  // op(SA) lower triangular
    // the half solved first: the top one when op(SA) is lower and the system is a left one
    const bool top_first = eff_lower == f.left;
    auto solve = [&](int64_t a, int64_t b) {
        return solve_range<T, CPLX>(f, a, b, sbr, sbc, SA, lda, SB, ldb, inv, tmp, ctl, s, err);
    };
    int st = top_first ? solve(lo, h) : solve(h, hi);
    if (st != GB300_OK) return st;
    if (f.left) {
        // the other half's rows -= op(SA)[other, first] X[first]
        st = top_first ? product(hi - h, sbc, h - lo, f.trans, false, f.conj, false, block(h, lo), lda, rows_of(lo), ldb,
                                 true, rows_of(h), ldb)
                       : product(h - lo, sbc, hi - h, f.trans, false, f.conj, false, block(lo, h), lda, rows_of(h), ldb,
                                 true, rows_of(lo), ldb);
    } else {
        // the other half's columns -= X[first] op(SA)[first, other]
        st = top_first ? product(sbr, hi - h, h - lo, false, f.trans, false, f.conj, cols_of(lo), ldb, block(lo, h), lda,
                                 true, cols_of(h), ldb)
                       : product(sbr, h - lo, hi - h, false, f.trans, false, f.conj, cols_of(h), ldb, block(h, lo), lda,
                                 true, cols_of(lo), ldb);
    }
    if (st != GB300_OK) return st;
    return top_first ? solve(h, hi) : solve(lo, h);
}
}  // namespace

// B = alpha op(A)^-1 B (left) or alpha B op(A)^-1 (right), A triangular (m x m or n x n): B scaled
// by alpha, the diagonal blocks of op(A) inverted, then the recursive blocked solve above.
// alpha == 0 sets B to zero without reading A.
template <typename T, bool CPLX>
int trsm_entry(int order, int side, int uplo, int transA, int diag, int64_t m, int64_t n, const T* alpha, const T* A,
               int64_t lda, T* B, int64_t ldb, const char* routine) {
    const CallTrace trace(routine, m, n, side == CblasLeft ? m : n);
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
    const bool rm = order == CblasRowMajor, left = side == CblasLeft;
    const int64_t ka = left ? m : n;
    if (lda < std::max<int64_t>(1, ka)) return fail(GB300_ERR_INVALID_ARG, "parameter 10 (lda) is too small");
    if (ldb < std::max<int64_t>(1, rm ? n : m)) return fail(GB300_ERR_INVALID_ARG, "parameter 12 (ldb) is too small");
    if (alpha == nullptr) return fail(GB300_ERR_INVALID_ARG, "parameter 8 (alpha) is NULL");
    clear_error();
    if (m == 0 || n == 0) return GB300_OK;
    const bool alpha0 = scalar_is<T, CPLX>(alpha, T(0));
    if (B == nullptr || (!alpha0 && A == nullptr)) return fail(GB300_ERR_INVALID_ARG, "A or B is NULL");

    Runtime& r = runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    int st = ensure_init(&err);
    if (st != GB300_OK) return fail(st, err);
    cudaStream_t s = r.stream;
    const LaunchCtl ctl = fresh_ctl(s);
    const size_t elem = (CPLX ? 2 : 1) * sizeof(T);

    // row-major storage as for trmm: SB = B or B^T, SA = A or A^T (its triangle flips for
    // column-major, and so does the side); the transposition and conjugation stay
    const int64_t sbr = rm ? m : n, sbc = rm ? n : m;
    SolveForm f;
    f.left = rm ? left : !left;
    f.lower = rm ? (uplo == CblasLower) : (uplo == CblasUpper);
    f.trans = transA != CblasNoTrans;
    f.conj = CPLX && transA == CblasConjTrans;
    f.unit = diag == CblasUnit;
    const bool bdev = in_place(B, elem);
    T* dB = static_cast<T*>(stage(B, sbr, sbc, ldb, elem, kAuxB, bdev, s, &err));
    if (!dB) return fail(GB300_ERR_NO_MEMORY, err);
    cudaError_t e = cudaSuccess;
    if (alpha0) {
        e = cudaMemset2DAsync(dB, size_t(ldb) * elem, 0, size_t(sbc) * elem, size_t(sbr), s);
    } else {
        const T* dA = static_cast<const T*>(stage(A, ka, ka, lda, elem, kAuxA, in_place(A, elem), s, &err));
        const int64_t nb = solve_block(elem), nblk = (ka + nb - 1) / nb;
        T* inv = static_cast<T*>(r.aux.get(kAuxT, size_t(nblk) * size_t(nb) * size_t(nb) * elem, &err));
        T* tmp = static_cast<T*>(r.aux.get(kAuxC, size_t(f.left ? sbc : sbr) * size_t(std::min<int64_t>(nb, ka)) * elem, &err));
        if (!dA || !inv || !tmp) return fail(GB300_ERR_NO_MEMORY, err);
        if (!scalar_is<T, CPLX>(alpha, T(1))) e = launch_scale<T, CPLX>(sbr, sbc, alpha, dB, ldb, s);
        if (e == cudaSuccess)
            e = launch_tri_inverse<T, CPLX>(ka, int(nb), dA, lda, f.trans, f.conj, f.lower == f.trans, f.unit, inv, s);
        if (e != cudaSuccess) return fail(GB300_ERR_CUDA, std::string("trsm launch: ") + cudaGetErrorString(e));
        if ((st = solve_range<T, CPLX>(f, 0, ka, sbr, sbc, dA, lda, dB, ldb, inv, tmp, ctl, s, &err)) != GB300_OK)
            return fail(st, err);
    }
    if (e == cudaSuccess && !bdev) e = unstage(B, dB, sbr, sbc, ldb, elem, s);
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
template int cgemv_entry<double>(int, int, int64_t, int64_t, const double*, const double*, int64_t, const double*,
                                 int64_t, const double*, double*, int64_t, const char*);
template int cgemv_entry<float>(int, int, int64_t, int64_t, const float*, const float*, int64_t, const float*, int64_t,
                                const float*, float*, int64_t, const char*);
template int trmv_entry<double, false>(int, int, int, int, int64_t, const double*, int64_t, double*, int64_t,
                                       const char*);
template int trmv_entry<float, false>(int, int, int, int, int64_t, const float*, int64_t, float*, int64_t, const char*);
template int trmv_entry<double, true>(int, int, int, int, int64_t, const double*, int64_t, double*, int64_t,
                                      const char*);
template int trmv_entry<float, true>(int, int, int, int, int64_t, const float*, int64_t, float*, int64_t, const char*);
template int ctrmm_entry<double>(int, int, int, int, int, int64_t, int64_t, const double*, const double*, int64_t,
                                 double*, int64_t, const char*);
template int ctrmm_entry<float>(int, int, int, int, int, int64_t, int64_t, const float*, const float*, int64_t, float*,
                                int64_t, const char*);
template int axpy_entry<double, false>(int64_t, const double*, const double*, int64_t, double*, int64_t, const char*);
template int axpy_entry<float, false>(int64_t, const float*, const float*, int64_t, float*, int64_t, const char*);
template int axpy_entry<double, true>(int64_t, const double*, const double*, int64_t, double*, int64_t, const char*);
template int axpy_entry<float, true>(int64_t, const float*, const float*, int64_t, float*, int64_t, const char*);
#define GB_DOT(T, C, J) \
    template int dot_entry<T, C, J>(int64_t, const T*, int64_t, const T*, int64_t, T*, const char*);
GB_DOT(double, false, false)
GB_DOT(float, false, false)
GB_DOT(double, true, false)
GB_DOT(double, true, true)
GB_DOT(float, true, false)
GB_DOT(float, true, true)
#undef GB_DOT
#define GB_TRSM(T, C)                                                                                          \
    template int trsm_entry<T, C>(int, int, int, int, int, int64_t, int64_t, const T*, const T*, int64_t, T*, \
                                  int64_t, const char*);
GB_TRSM(double, false)
GB_TRSM(float, false)
GB_TRSM(double, true)
GB_TRSM(float, true)
#undef GB_TRSM
}  // namespace gb
