// gb300_internal.h — internal host-side interfaces shared by the translation units of
// libgb300blas (not installed; the public C-ABI is include/gb300_cblas.h and include/gb300_blas.h).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/gb300_blas.h"

namespace gb {

// A product in logical row-major form:  C (m x n) = alpha * op(A) (m x k) * op(B) (k x n) + beta*C.
//   ta == false: A(i,p) = A[i*lda + p]  (k contiguous);   ta == true: A(i,p) = A[p*lda + i]
//   tb == false: B(p,j) = B[p*ldb + j]  (n contiguous);   tb == true: B(p,j) = B[j*ldb + p]
//   C(i,j) = C[i*ldc + j].
// A column-major CBLAS call is brought to this form by C^T = op(B)^T op(A)^T (swap the operands,
// m <-> n, and the transposition flags).  All pointers are device (or managed) addresses.
struct Gemm {
    int64_t m = 0, n = 0, k = 0;
    bool ta = false, tb = false;
    const void* A = nullptr;
    int64_t lda = 0;
    const void* B = nullptr;
    int64_t ldb = 0;
    void* C = nullptr;
    int64_t ldc = 0;
    double alpha = 1.0, beta = 0.0;
};

// Per-launch controls shared by the kernels.
struct LaunchCtl {
    int* status = nullptr;          // device status word (DeviceStatus), zeroed before the launch
    uint64_t wait_limit_ns = 4000000000ull;
    int inject_stall = 0;           // test hook: the TMA producer issues nothing (waits run out)
};

// Device -> host copy of `rows` rows of `width` bytes: one linear copy when both pitches equal the
// width, else a pitched copy.  On a Grace host a pitched copy into pageable pages that were never
// touched runs over ten times slower than a linear one (430 ms against 40 ms for 512 MiB, measured
// on a GB300); into resident pages the two take the same time.
inline cudaError_t copy_to_host(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t rows,
                                cudaStream_t st) {
    if (rows <= 1 || (dpitch == width && spitch == width))
        return cudaMemcpyAsync(dst, src, width * rows, cudaMemcpyDeviceToHost, st);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, cudaMemcpyDeviceToHost, st);
}

// ---- tensor maps ----------------------------------------------------------------------------
// Encode a 2-D tiled tensor map over a row-major matrix of `rows` x `cols` elements of
// `dtype` with a row pitch of `ld` elements; the box is box_cols (innermost) x box_rows.
// Returns false (and fills err) when the driver rejects the layout.
bool encode_tmap_2d(CUtensorMap* map, CUtensorMapDataType dtype, size_t elem_bytes, const void* base,
                    uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows, uint32_t box_cols,
                    CUtensorMapSwizzle swizzle, std::string* err);

// 3-D variant: a stack of `planes` row-major matrices, plane pitch `plane_stride` elements.
bool encode_tmap_3d(CUtensorMap* map, CUtensorMapDataType dtype, size_t elem_bytes, const void* base,
                    uint64_t planes, uint64_t rows, uint64_t cols, uint64_t ld, uint64_t plane_stride,
                    uint32_t box_rows, uint32_t box_cols, CUtensorMapSwizzle swizzle, std::string* err);

// ---- native (DFMA / FFMA) GEMM --------------------------------------------------------------
// Launches the TMA-staged SIMT kernel.  `splits` > 1 partitions k; the partial products then go
// through `workspace` (splits * m * n elements of T) and a fixed-order reduction.
template <typename T>
cudaError_t native_gemm(const Gemm& g, int splits, T* workspace, const LaunchCtl& ctl, cudaStream_t s,
                        std::string* err);

// Split count the native kernel uses for a shape on `num_sms` SMs (1 = no split).
int native_choose_splits(int64_t m, int64_t n, int64_t k, int elem_bytes, int num_sms);
// The shared implementation behind cblas_?gemm and gb300_?gemm_ex (CBLAS argument conventions).
// The method cblas_?gemm uses (GB300_DGEMM_METHOD / gb300_set_default_method).
int library_default_method();

template <typename T>
int gemv_entry(int order, int transA, int64_t m, int64_t n, T alpha, const T* A, int64_t lda, const T* x,
               int64_t incx, T beta, T* y, int64_t incy, const char* routine);
// complex interleaved (re, im) operands, T = double or float; alpha, beta point to two T each
template <typename T>
int cgemm_entry(int order, int transA, int transB, int64_t m, int64_t n, int64_t k, const T* alpha, const T* A,
                int64_t lda, const T* B, int64_t ldb, const T* beta, T* C, int64_t ldc, const char* routine);
template <typename T>
int trmm_entry(int order, int side, int uplo, int transA, int diag, int64_t m, int64_t n, T alpha, const T* A,
               int64_t lda, T* B, int64_t ldb, const char* routine);
// complex interleaved y = alpha op(A) x + beta y; alpha, beta point to (re, im)
template <typename T>
int cgemv_entry(int order, int transA, int64_t m, int64_t n, const T* alpha, const T* A, int64_t lda, const T* x,
                int64_t incx, const T* beta, T* y, int64_t incy, const char* routine);
// x = op(A) x, A triangular; CPLX: interleaved complex elements
template <typename T, bool CPLX>
int trmv_entry(int order, int uplo, int transA, int diag, int64_t n, const T* A, int64_t lda, T* x, int64_t incx,
               const char* routine);
// complex interleaved B = alpha op(A) B or alpha B op(A), A triangular; alpha points to (re, im)
template <typename T>
int ctrmm_entry(int order, int side, int uplo, int transA, int diag, int64_t m, int64_t n, const T* alpha, const T* A,
                int64_t lda, T* B, int64_t ldb, const char* routine);
// B = alpha op(A)^-1 B or alpha B op(A)^-1, A triangular; alpha points to one T, or (re, im) for CPLX
template <typename T, bool CPLX>
int trsm_entry(int order, int side, int uplo, int transA, int diag, int64_t m, int64_t n, const T* alpha, const T* A,
               int64_t lda, T* B, int64_t ldb, const char* routine);
// y = alpha x + y; alpha points to one T, or (re, im) for CPLX
template <typename T, bool CPLX>
int axpy_entry(int64_t n, const T* alpha, const T* x, int64_t incx, T* y, int64_t incy, const char* routine);
// *result = sum_i op(x_i) y_i, op = conjugation when CONJ; result holds one T, or (re, im) for CPLX
template <typename T, bool CPLX, bool CONJ>
int dot_entry(int64_t n, const T* x, int64_t incx, const T* y, int64_t incy, T* result, const char* routine);

template <typename T>
int gemm_entry(int order, int transA, int transB, int64_t m, int64_t n, int64_t k, T alpha, const T* A, int64_t lda,
               const T* B, int64_t ldb, T beta, T* C, int64_t ldc, gb300_gemm_opts* opts, const char* routine);

// Grouped launches of the serving loop (grouped.cu): a lane stages the problem table of a batch of
// small FP64 products and runs them as one persistent grouped launch on its stream.  A lane's next
// launch must wait until its previous one has finished.
struct GroupedLane;
GroupedLane* grouped_lane_create(cudaStream_t stream, std::string* err);
void grouped_lane_destroy(GroupedLane* lane);
int grouped_lane_launch(GroupedLane* lane, const gb300_gemm_problem* probs, int64_t count, double* useful_flops,
                        std::string* err);

}  // namespace gb
