/*
 * gb300_blas.h — extended C-ABI of libgb300blas (GB300 / sm_103a dense matrix multiplication).
 *
 * The drop-in CBLAS surface is include/gb300_cblas.h.  This header adds what CBLAS cannot say:
 * the choice between the native FP64 kernel and the split-precision tensor-core forms, device-
 * resident operands and streams, and status reporting.  All signatures use plain pointers,
 * sizes and enums; no CUDA or C++ types appear.
 */
#ifndef GB300_BLAS_H
#define GB300_BLAS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* Status codes (returned by the *_ex functions and recorded for the CBLAS entry points). */
enum gb300_status {
    GB300_OK = 0,
    GB300_ERR_INVALID_ARG = 1,     /* an argument violates the CBLAS contract (see message) */
    GB300_ERR_CUDA = 2,            /* a CUDA runtime call failed */
    GB300_ERR_NO_MEMORY = 3,       /* device or pinned-host allocation failed */
    GB300_ERR_DEVICE_TIMEOUT = 4,  /* a kernel's bounded wait ran out; the launch was abandoned */
    GB300_ERR_NOT_SUPPORTED = 5,   /* routine declared for Blaze but not provided on the GPU */
    GB300_ERR_NO_DEVICE = 6,       /* no CUDA device is visible */
    GB300_ERR_ADMISSION = 7        /* a request exceeds the server's memory budget */
};

/* Arithmetic forms of the product. */
enum gb300_method {
    GB300_METHOD_AUTO = 0,    /* FP64-accurate: split-precision where it is faster, else native */
    GB300_METHOD_NATIVE = 1,  /* native FP64 DFMA (FP32 FFMA for sgemm) */
    GB300_METHOD_SPLIT = 2,   /* Ozaki-style BF16 slices on tcgen05, FP64 recombination (double only) */
    GB300_METHOD_BF16X3 = 3,  /* three BF16 products (hi*hi + hi*lo + lo*hi), FP32 accumulation */
    GB300_METHOD_BF16 = 4,    /* one BF16 product, FP32 accumulation */
    GB300_METHOD_SPLIT_CRT = 5 /* FP64-accurate, residue (CRT) scheme: operands rounded to beta-bit
                                  integers per row / column, one BF16 product per modulus, exact
                                  reconstruction; GB300_METHOD_SPLIT uses it whenever its worst-case
                                  plan fits 15 moduli and no slice count is requested */
};

/* Where the operand pointers live. */
enum gb300_residency {
    GB300_PTR_DETECT = 0,     /* ask the CUDA driver (cudaPointerGetAttributes) */
    GB300_PTR_DEVICE = 1,     /* device or managed memory: used in place, no copies */
    GB300_PTR_HOST = 2        /* host memory: staged to the device and back inside the call */
};

typedef struct gb300_gemm_opts {
    int method;            /* gb300_method */
    int slices;            /* GB300_METHOD_SPLIT: digit slices per operand (0 = choose from target;
                              a positive count selects the digit scheme); SPLIT_CRT: moduli cap */
    double target_error;   /* GB300_METHOD_SPLIT: normwise bound to reach; <= 0 means k * 2^-53 */
    int residency;         /* gb300_residency */
    void* stream;          /* cudaStream_t to run on; NULL = the library's stream.  All of a call's
                              device work is ordered on it: what the library runs on a second
                              stream inside the call is joined back to it. */
    int synchronous;       /* non-zero: return after the result is in C */
    /* outputs */
    int method_used;       /* the form that ran */
    int slices_used;       /* split forms: digit slices per operand, or moduli (CRT scheme) */
    double error_bound;    /* a-priori normwise bound ||C-AB||_F/(||A||_F||B||_F) of the form
                              that ran (split: computed from the operands' exponents; other forms:
                              the textbook bound of their arithmetic) */
} gb300_gemm_opts;

/* Fill `opts` with defaults: method from the library default, target k*2^-53, detect residency,
 * library stream, synchronous. */
void gb300_gemm_opts_init(gb300_gemm_opts* opts);

/* C = alpha*op(A)*op(B) + beta*C with CBLAS argument conventions and 64-bit sizes.
 * Returns a gb300_status (also recorded as the thread's last error). */
int gb300_dgemm_ex(int order, int transA, int transB, int64_t m, int64_t n, int64_t k, double alpha,
                   const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
                   int64_t ldc, gb300_gemm_opts* opts);
int gb300_sgemm_ex(int order, int transA, int transB, int64_t m, int64_t n, int64_t k, float alpha,
                   const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C,
                   int64_t ldc, gb300_gemm_opts* opts);

/* Default method used by cblas_dgemm (initially GB300_METHOD_AUTO, or the GB300_DGEMM_METHOD
 * environment variable: auto|native|split|bf16x3|bf16).  Returns the previous value. */
int gb300_set_default_method(int method);

/* Last status of the calling thread (also declared in gb300_cblas.h). */
int gb300_last_error(void);
const char* gb300_last_error_message(void);
void gb300_clear_error(void);

/* Device facts the library uses: SM count, free and total device memory in bytes.
 * Returns GB300_ERR_NO_DEVICE when no GPU is visible. */
int gb300_device_info(int* num_sms, int64_t* free_bytes, int64_t* total_bytes);

/* Measure the device's sustained FP64 FMA rate (TFLOP/s) with independent DFMA chains on every
 * SM.  The automatic method choice uses it; benchmarks report it as the FP64 roofline. */
int gb300_measure_fp64_peak(double* tflops);
/* The same with FFMA chains: the sustained FP32 rate (TFLOP/s), the roofline of the FP32 kernels. */
int gb300_measure_fp32_peak(double* tflops);

/* Make `ordinal` the library's device.  Call before the first product of the process (each
 * process of a multi-GPU job owns one device). */
int gb300_select_device(int ordinal);

/* Kernel timing for benchmarks: while enabled, the library records CUDA events on the launching
 * stream around the dominant kernel of every product ("tc_gemm" for the tensor-core forms,
 * "native_gemm" for the native kernel).  gb300_profile_read waits for the recorded events, returns
 * the summed milliseconds and the launch count of kernels whose name starts with `prefix` (NULL:
 * all), and clears the record. */
void gb300_profile_enable(int on);
int gb300_profile_read(const char* prefix, double* total_ms, int64_t* launches);

/* Count of kernel launches the library has issued in this process (all entry points). */
int64_t gb300_launch_count(void);

/* Device bytes held by the library's own grow-only buffers in this process (the default context,
 * the buffers of the routines next to ?gemm and every server slot).  Memory accounting for hosts
 * that budget device memory; plans of the grouped API are not included. */
int64_t gb300_pool_bytes(void);

/* Wait until all work the library queued on its own stream has finished. */
int gb300_synchronize(void);

/* ---- grouped (batched) products -----------------------------------------------------------
 * Many independent, uneven products (Blaze's StaticMatrix / HybridMatrix sizes) in one persistent
 * launch.  Each problem uses the CBLAS conventions of gb300_dgemm_ex; A, B and C must be device (or
 * managed) memory.  alpha/beta are taken as double (converted for the float form).  Blaze has no
 * batched product: this replaces a loop of per-product calls (blaze/math/expressions/
 * DMatDMatMultExpr.h:864-1878, the small kernel each such product runs on the CPU). */
typedef struct gb300_gemm_problem {
    int order, transA, transB;
    int64_t m, n, k;
    double alpha, beta;
    const void* A;
    int64_t lda;
    const void* B;
    int64_t ldb;
    void* C;
    int64_t ldc;
} gb300_gemm_problem;

typedef struct gb300_grouped_plan gb300_grouped_plan;

/* Tile every problem with the warp-tile shape of its size class (autotuned, see below), upload the
 * problem and tile tables and capture the launch in a CUDA graph.  elem_bytes: 8 (double) or 4. */
int gb300_grouped_plan_create(int elem_bytes, const gb300_gemm_problem* problems, int64_t count,
                              gb300_grouped_plan** plan);
/* One graph launch on `stream` (NULL: the library stream); asynchronous. */
int gb300_grouped_plan_run(gb300_grouped_plan* plan, void* stream);
/* Tiles of the plan and the useful / padded multiply-add work (2*m*n*k summed, in flops). */
int gb300_grouped_plan_info(const gb300_grouped_plan* plan, int64_t* tiles, double* useful_flops,
                            double* padded_flops);
void gb300_grouped_plan_destroy(gb300_grouped_plan* plan);
/* Plan, run and destroy in one call; returns after the products finished. */
int gb300_dgemm_grouped(const gb300_gemm_problem* problems, int64_t count, void* stream);
int gb300_sgemm_grouped(const gb300_gemm_problem* problems, int64_t count, void* stream);
/* Autotuner: time every warp-tile shape on synthetic batches of each size class (m, n bucketed by
 * powers of two up to 256, k in three ranges) and keep the fastest per class.  effort >= 1 scales
 * the batch size.  Tables persist through save/load ("gb300-grouped-tune v1" text files). */
int gb300_grouped_autotune(int elem_bytes, int effort);
int gb300_grouped_tuning_save(const char* path);
int gb300_grouped_tuning_load(const char* path);
/* Shape index the planner uses for a product, with its warp-tile rows and columns. */
int gb300_grouped_shape_for(int elem_bytes, int64_t m, int64_t n, int64_t k, int* rows, int* cols);

/* ---- serving: continuous batching of product requests ---------------------------------------
 * A server admits requests as stream slots and device memory free up (FIFO with backfill under a
 * device-memory budget), runs admitted requests concurrently on their own streams and workspaces,
 * and records per-request latency.  Small requests (every dimension at most batch_threshold) are
 * coalesced: at each scheduling step the queued ones go out together as one persistent grouped
 * launch in FP64 (which meets the bound of every accuracy class), on one of two batch lanes;
 * large requests (max(m, n) >= large_threshold) run only on large_slots slots of their own, whose
 * streams have the lowest priority (the other slots' streams a higher one, the batch lanes' the
 * highest), so that neither slots nor SMs stay held by them while smaller requests wait.  The server's streams do not wait for work on other
 * streams: A, B and C must hold their values when a request is submitted (synchronize any copy or
 * fill still queued for them first).  Operands are resident: A, B and C are device (or managed)
 * memory owned by the caller (operands that TMA cannot address in place — odd leading dimension or
 * a base not 16-byte aligned — are realigned into the request's workspace).  Blaze has no server;
 * each request is the same product as gb300_dgemm_ex with the accuracy class as its method. */
typedef struct gb300_server_config {
    int64_t memory_budget_bytes;  /* scratch the server may hold (default 150 GiB, capped by free memory) */
    int slots;                    /* requests running at once (default 8) */
    int reserve_sms;              /* SMs kept out of large tensor-core products for small requests (16) */
    double aging_ms;              /* a queue head older than this stops backfilling (50 ms) */
    int64_t large_threshold;      /* max(m, n) from which a request counts as large (2048) */
    int64_t batch_threshold;      /* requests with max(m, n, k) <= this run in grouped launches (256; 0: never) */
    int batch_max;                /* requests per grouped launch at most (2048) */
    int large_slots;              /* slots kept for large requests, at the lowest stream priority (2) */
} gb300_server_config;

typedef struct gb300_serve_request {
    int order, transA, transB;
    int64_t m, n, k;
    double alpha, beta;
    const double* A;
    int64_t lda;
    const double* B;
    int64_t ldb;
    double* C;
    int64_t ldc;
    int accuracy;          /* gb300_method: NATIVE, SPLIT (<= target_error), BF16X3, BF16, AUTO */
    double target_error;   /* SPLIT: normwise target; <= 0 means k * 2^-53 */
} gb300_serve_request;

typedef struct gb300_serve_result {
    int status;            /* gb300_status of the request */
    int method_used;
    int slices;
    double error_bound;    /* a-priori normwise bound of the form that ran */
    double queue_ms;       /* submission -> start */
    double run_ms;         /* start -> completion seen */
    double latency_ms;     /* submission -> completion seen */
} gb300_serve_result;

typedef struct gb300_server_stats {
    int64_t submitted, completed, rejected, failed, queued;
    double p50_ms, p99_ms, mean_ms, max_ms;   /* latency of completed requests */
    double wall_s;                            /* since the first submission (or the last reset) */
    double tflops;                            /* 2*m*n*k of completed requests / wall_s */
    int64_t bytes_in_use, peak_bytes, budget_bytes;
    /* per size class: 0 small (grouped launches), 1 medium, 2 large (max(m, n) >= large_threshold) */
    int64_t class_completed[3];
    double class_p50_ms[3], class_p99_ms[3];
    int64_t grouped_launches;                 /* grouped launches issued */
    double grouped_mean_batch;                /* requests per grouped launch */
} gb300_server_stats;

typedef struct gb300_server gb300_server;

void gb300_server_config_init(gb300_server_config* config);
int gb300_server_create(const gb300_server_config* config, gb300_server** server);
/* Queue a request; the ticket identifies it.  GB300_ERR_ADMISSION when it can never fit the budget. */
int gb300_server_submit(gb300_server* server, const gb300_serve_request* request, uint64_t* ticket);
/* Wait for a request (timeout_ms < 0: no limit), fill `result` and forget the ticket; returns the
 * request's status (GB300_ERR_DEVICE_TIMEOUT if the timeout passed first; the ticket stays valid). */
int gb300_server_wait(gb300_server* server, uint64_t ticket, double timeout_ms, gb300_serve_result* result);
int gb300_server_poll(gb300_server* server, uint64_t ticket, int* done);
int gb300_server_get_stats(gb300_server* server, gb300_server_stats* stats);
void gb300_server_reset_stats(gb300_server* server);
/* Stop the scheduler after the running requests finished and free the server's memory. */
void gb300_server_destroy(gb300_server* server);

/* Allocation-free variant of the native FP64 product, for callers that cannot allocate device
 * memory themselves (a host framework that owns all device memory through its own pool or
 * budget, or a latency-critical loop where cudaMalloc/cudaFree and their implicit device
 * synchronization are not allowed).  It has no counterpart in the reference.
 * Operands and C must be device memory of the current device (or managed memory) with 16-byte
 * aligned bases and even leading dimensions; a non-NULL `stream` must belong to the current
 * device.  The split-k scratch comes from a fixed 16 MiB array compiled into the library (held on
 * every GPU that loads the library until exit); products that need more are rejected with
 * GB300_ERR_INVALID_ARG before anything is queued, C unchanged.  The array's device address is
 * looked up on every call; the first call on a device also loads the library's device code there,
 * so make that first call before any stream capture.  Calls share the array: the function
 * serializes its callers and returns after its kernels finished on `stream` (NULL: the legacy
 * default stream), on error paths too.  gb300_debug_inject_stall applies to it like to the other
 * native launches. */
int gb300_dgemm_native_noalloc(int order, int transA, int transB, int64_t m, int64_t n, int64_t k,
                               double alpha, const double* A, int64_t lda, const double* B,
                               int64_t ldb, double beta, double* C, int64_t ldc, void* stream);

/* Test hooks for failure detection (no fault is involved): the next `count` native-kernel
 * launches run with their TMA producer disabled and their waits limited to `limit_ns`, so they
 * end with GB300_ERR_DEVICE_TIMEOUT.  count = 0 clears the hook. */
void gb300_debug_inject_stall(int count, uint64_t limit_ns);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* GB300_BLAS_H */
