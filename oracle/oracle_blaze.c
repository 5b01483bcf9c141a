/*
 * oracle_blaze.c — C restatement of Blaze's CPU dense matrix-multiplication kernels.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); see oracle.h.
 *
 * Two kernels, both with CBLAS argument semantics:
 *
 *  orc_gemm_default_*   blaze/math/expressions/DMatDMatMultExpr.h:590-681
 *      For each row i:  C(i,j) = A(i,0)*B(0,j)  then  C(i,j) += A(i,k)*B(k,j)  for k = 1..K-1,
 *      i.e. every element is accumulated sequentially in k order.  (The row x column default
 *      kernel, DMatTDMatMultExpr.h:566-665, forms the same sequential dot product per element.)
 *      The alpha/beta update follows Blaze's scaled/add-assign expressions: the product is
 *      formed first, then C = alpha*P (beta == 0: C is not read) or C = alpha*P + beta*C.
 *
 *  orc_gemm_small_*     blaze/math/expressions/DMatDMatMultExpr.h:864-1878 (selectSmallAssignKernel,
 *      row-major C; column-major C through the transposed identity below)
 *      Column panels of 5, 4, 3, 2 and 1 SIMD widths (then single columns; the width of the
 *      build target's vectors, 128 bits here), two rows of C at a time, k innermost with one accumulator per output: C(i,j) = A(i,0)*B(0,j), then
 *      += A(i,k)*B(k,j) for k = 1..K-1 — the same sequential per-element order as the default
 *      kernel, in the register-blocked loop nest that makes it Blaze's fast path for small and
 *      skinny products.  orc_gemm_batch_small_* runs it over a list of products (the batched
 *      configuration's CPU baseline), products spread over OpenMP threads.
 *
 *  orc_gemm_blocked_*   blaze/math/dense/MMM.h:105-600 (`mmm`, row-major C)
 *      beta == 0 resets C without reading it, beta != 1 scales C (MMM.h:146-151);
 *      k-panels of KBLOCK = MMM_OUTER_BLOCK_SIZE*16/sizeof(T) = 112*16/sizeof(T) columns
 *      (blaze/system/Blocking.h:60-61, MMM.h:131) with A's panel packed row-major (A2) and
 *      JBLOCK = MMM_INNER_BLOCK_SIZE = 96 column panels of B packed column-major (B2);
 *      each C element of a panel pair is a SIMDSIZE-lane split dot product over the panel,
 *      reduced by a horizontal sum and added as C(i,j) += sum*alpha (MMM.h:190-330); when K is
 *      not a multiple of SIMDSIZE the trailing columns are added term by term as
 *      C(i,j) += A2(i,k)*B2(k,j)*alpha (MMM.h:470-575).  SIMDSIZE is 8 doubles / 16 floats
 *      (the AVX-512 width Blaze selects on an AVX-512 host).
 *      Column-major C (MMM.h:605-1080) is evaluated through the identity
 *      C^T = op(B)^T op(A)^T, which maps a column-major call onto the row-major kernel.
 *      Rows of C are split across OpenMP threads (Blaze's SMP layer splits C into thread
 *      tiles, blaze/math/smp/openmp/DenseMatrix.h:97-160; every tile runs the same kernel).
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KBLOCK_D (112 * 16 / 8)   /* 224 */
#define KBLOCK_S (112 * 16 / 4)   /* 448 */
#define JBLOCK 96
#define LANES_D 8
#define LANES_S 16

/* Logical element (r,c) of op(X) for a row-major call: X stored row-major with leading
 * dimension ld; trans selects X^T. */
#define OPX(X, ld, trans, r, c) ((trans) ? (X)[(int64_t)(c) * (ld) + (r)] : (X)[(int64_t)(r) * (ld) + (c)])

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------------------------------------------------------------------------------------
 * default (scalar i-k-j) kernel
 * ------------------------------------------------------------------------------------------- */
#define DEFINE_DEFAULT(SUFFIX, T)                                                                  \
static void default_rm_##SUFFIX(int tA, int tB, int64_t m, int64_t n, int64_t k, T alpha,        \
                                const T* A, int64_t lda, const T* B, int64_t ldb, T beta, T* C,  \
                                int64_t ldc) {                                                   \
    T* row = (T*)malloc(sizeof(T) * (size_t)(n > 0 ? n : 1));                                   \
    for (int64_t i = 0; i < m; ++i) {                                                            \
        if (k == 0) {                                                                            \
            for (int64_t j = 0; j < n; ++j) row[j] = (T)0;                                       \
        } else {                                                                                 \
            const T a0 = OPX(A, lda, tA, i, 0);                                                  \
            for (int64_t j = 0; j < n; ++j) row[j] = a0 * OPX(B, ldb, tB, 0, j);                 \
            for (int64_t p = 1; p < k; ++p) {                                                    \
                const T a = OPX(A, lda, tA, i, p);                                               \
                for (int64_t j = 0; j < n; ++j) row[j] += a * OPX(B, ldb, tB, p, j);             \
            }                                                                                    \
        }                                                                                        \
        T* c = C + i * ldc;                                                                      \
        if (beta == (T)0) {                                                                      \
            for (int64_t j = 0; j < n; ++j) c[j] = alpha * row[j];                               \
        } else {                                                                                 \
            for (int64_t j = 0; j < n; ++j) c[j] = alpha * row[j] + beta * c[j];                 \
        }                                                                                        \
    }                                                                                            \
    free(row);                                                                                   \
}                                                                                                \
void orc_gemm_default_##SUFFIX(int order, int transA, int transB, int64_t m, int64_t n,         \
                               int64_t k, T alpha, const T* A, int64_t lda, const T* B,          \
                               int64_t ldb, T beta, T* C, int64_t ldc) {                         \
    const int tA = (transA != ORC_NO_TRANS), tB = (transB != ORC_NO_TRANS);                      \
    if (m <= 0 || n <= 0) return;                                                                \
    if (order == ORC_ROW_MAJOR)                                                                  \
        default_rm_##SUFFIX(tA, tB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);               \
    else                                                                                         \
        default_rm_##SUFFIX(tB, tA, n, m, k, alpha, B, ldb, A, lda, beta, C, ldc);               \
}

DEFINE_DEFAULT(d, double)
DEFINE_DEFAULT(s, float)

/* ---------------------------------------------------------------------------------------------
 * small (register-blocked) kernel
 * ------------------------------------------------------------------------------------------- */
/* One panel of W columns (W a multiple of the lane count, or 1) for rows i0..i0+R-1 (R = 1 or 2);
 * called with W a literal, so that the loops over the panel have fixed trip counts. */
#define DEFINE_SMALL(SUFFIX, T, LANES)                                                             \
static inline __attribute__((always_inline)) void small_panel_##SUFFIX(                          \
        int tA, int tB, int64_t i0, int R, int64_t j0, const int W, int64_t k, T alpha,          \
        const T* A, int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc) {           \
    T acc0[5 * LANES], acc1[5 * LANES], bp[5 * LANES];                                           \
    const int64_t sa = tA ? 1 : lda, pa = tA ? lda : 1; /* A(i,p) = A[i*sa + p*pa] */            \
    const T* a0 = A + i0 * sa;                                                                   \
    const T* a1 = A + (i0 + (R > 1 ? 1 : 0)) * sa;                                               \
    for (int64_t p = 0; p < k; ++p) {                                                            \
        const T* b;                                                                              \
        if (!tB) {                                                                               \
            b = B + p * ldb + j0;                                                                \
        } else {                                                                                 \
            for (int w = 0; w < W; ++w) bp[w] = B[(j0 + w) * ldb + p];                           \
            b = bp;                                                                              \
        }                                                                                        \
        const T x0 = a0[p * pa], x1 = a1[p * pa];                                                \
        if (p == 0) {                                                                            \
            for (int w = 0; w < W; ++w) { acc0[w] = x0 * b[w]; acc1[w] = x1 * b[w]; }            \
        } else {                                                                                 \
            for (int w = 0; w < W; ++w) { acc0[w] += x0 * b[w]; acc1[w] += x1 * b[w]; }          \
        }                                                                                        \
    }                                                                                            \
    for (int r = 0; r < R; ++r) {                                                                \
        const T* acc = r ? acc1 : acc0;                                                          \
        T* c = C + (i0 + r) * ldc + j0;                                                          \
        if (beta == (T)0)                                                                        \
            for (int w = 0; w < W; ++w) c[w] = alpha * acc[w];                                   \
        else                                                                                     \
            for (int w = 0; w < W; ++w) c[w] = alpha * acc[w] + beta * c[w];                     \
    }                                                                                            \
}                                                                                                \
static void small_cols_##SUFFIX(int tA, int tB, int64_t m, int64_t j, const int W, int64_t k,    \
                                T alpha, const T* A, int64_t lda, const T* B, int64_t ldb,       \
                                T beta, T* C, int64_t ldc) {                                     \
    for (int64_t i = 0; i < m; i += 2)                                                           \
        small_panel_##SUFFIX(tA, tB, i, (i + 2 <= m) ? 2 : 1, j, W, k, alpha, A, lda, B, ldb,    \
                             beta, C, ldc);                                                      \
}                                                                                                \
static void small_rm_##SUFFIX(int tA, int tB, int64_t m, int64_t n, int64_t k, T alpha,          \
                              const T* A, int64_t lda, const T* B, int64_t ldb, T beta, T* C,    \
                              int64_t ldc) {                                                     \
    if (k == 0) {                                                                                \
        for (int64_t i = 0; i < m; ++i)                                                          \
            for (int64_t j = 0; j < n; ++j)                                                      \
                C[i * ldc + j] = beta == (T)0 ? (T)0 : beta * C[i * ldc + j];                     \
        return;                                                                                  \
    }                                                                                            \
    int64_t j = 0;                                                                               \
    for (; j + 5 * LANES <= n; j += 5 * LANES)                                                   \
        small_cols_##SUFFIX(tA, tB, m, j, 5 * LANES, k, alpha, A, lda, B, ldb, beta, C, ldc);    \
    for (; j + 4 * LANES <= n; j += 4 * LANES)                                                   \
        small_cols_##SUFFIX(tA, tB, m, j, 4 * LANES, k, alpha, A, lda, B, ldb, beta, C, ldc);    \
    for (; j + 3 * LANES <= n; j += 3 * LANES)                                                   \
        small_cols_##SUFFIX(tA, tB, m, j, 3 * LANES, k, alpha, A, lda, B, ldb, beta, C, ldc);    \
    for (; j + 2 * LANES <= n; j += 2 * LANES)                                                   \
        small_cols_##SUFFIX(tA, tB, m, j, 2 * LANES, k, alpha, A, lda, B, ldb, beta, C, ldc);    \
    for (; j + LANES <= n; j += LANES)                                                           \
        small_cols_##SUFFIX(tA, tB, m, j, LANES, k, alpha, A, lda, B, ldb, beta, C, ldc);        \
    for (; j < n; ++j)                                                                           \
        small_cols_##SUFFIX(tA, tB, m, j, 1, k, alpha, A, lda, B, ldb, beta, C, ldc);            \
}                                                                                                \
void orc_gemm_small_##SUFFIX(int order, int transA, int transB, int64_t m, int64_t n, int64_t k, \
                             T alpha, const T* A, int64_t lda, const T* B, int64_t ldb, T beta,  \
                             T* C, int64_t ldc) {                                                \
    const int tA = (transA != ORC_NO_TRANS), tB = (transB != ORC_NO_TRANS);                      \
    if (m <= 0 || n <= 0) return;                                                                \
    if (order == ORC_ROW_MAJOR)                                                                  \
        small_rm_##SUFFIX(tA, tB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);                 \
    else                                                                                         \
        small_rm_##SUFFIX(tB, tA, n, m, k, alpha, B, ldb, A, lda, beta, C, ldc);                 \
}                                                                                                \
void orc_gemm_batch_small_##SUFFIX(int64_t count, const int64_t* desc, const T* ab, const T* A,  \
                                   const T* B, T* C, int nthreads) {                             \
    int nt = nthreads > 0 ? nthreads : orc_max_threads();                                        \
    if (nt < 1) nt = 1;                                                                          \
    _Pragma("omp parallel for num_threads(nt) schedule(dynamic, 16)")                            \
    for (int64_t q = 0; q < count; ++q) {                                                        \
        const int64_t* d = desc + 12 * q;                                                        \
        orc_gemm_small_##SUFFIX((int)d[0], (int)d[1], (int)d[2], d[3], d[4], d[5], ab[2 * q],    \
                                A + d[9], d[6], B + d[10], d[7], ab[2 * q + 1], C + d[11], d[8]); \
    }                                                                                            \
}

/* Blaze sizes these panels by the SIMD width of the build target; the oracle is built for the
 * baseline 128-bit vectors of both hosts (SSE2 on x86-64, NEON on Arm): 2 doubles, 4 floats. */
#define SMALL_LANES_D 2
#define SMALL_LANES_S 4
DEFINE_SMALL(d, double, SMALL_LANES_D)
DEFINE_SMALL(s, float, SMALL_LANES_S)

/* ---------------------------------------------------------------------------------------------
 * blocked (mmm) kernel
 * ------------------------------------------------------------------------------------------- */
#define DEFINE_BLOCKED(SUFFIX, T, KBLOCK, LANES)                                                   \
static void blocked_rows_##SUFFIX(int tA, int tB, int64_t i0, int64_t i1, int64_t n, int64_t k,  \
                                  T alpha, const T* A, int64_t lda, const T* B, int64_t ldb,     \
                                  T* C, int64_t ldc, T* A2, T* B2) {                             \
    const int64_t isize = i1 - i0;                                                               \
    for (int64_t kk = 0; kk < k; kk += KBLOCK) {                                                 \
        const int64_t kb = (kk + KBLOCK <= k) ? KBLOCK : (k - kk);                               \
        const int64_t kv = kb - kb % LANES; /* lane-split part of the panel */                  \
        for (int64_t i = 0; i < isize; ++i)                                                      \
            for (int64_t p = 0; p < kb; ++p) A2[i * KBLOCK + p] = OPX(A, lda, tA, i0 + i, kk + p);\
        for (int64_t jj = 0; jj < n; jj += JBLOCK) {                                             \
            const int64_t jb = (jj + JBLOCK <= n) ? JBLOCK : (n - jj);                           \
            for (int64_t j = 0; j < jb; ++j)                                                     \
                for (int64_t p = 0; p < kb; ++p) B2[j * KBLOCK + p] = OPX(B, ldb, tB, kk + p, jj + j);\
            int64_t i = 0;                                                                       \
            for (; i + 4 <= isize; i += 4) {                                                     \
                int64_t j = 0;                                                                   \
                for (; j + 2 <= jb; j += 2) {                                                    \
                    T x[4][2][LANES];                                                            \
                    memset(x, 0, sizeof(x));                                                     \
                    const T* a0 = A2 + (i + 0) * KBLOCK; const T* a1 = A2 + (i + 1) * KBLOCK;    \
                    const T* a2 = A2 + (i + 2) * KBLOCK; const T* a3 = A2 + (i + 3) * KBLOCK;    \
                    const T* b0 = B2 + (j + 0) * KBLOCK; const T* b1 = B2 + (j + 1) * KBLOCK;    \
                    for (int64_t p = 0; p < kv; p += LANES) {                                    \
                        for (int l = 0; l < LANES; ++l) {                                        \
                            x[0][0][l] += a0[p + l] * b0[p + l]; x[0][1][l] += a0[p + l] * b1[p + l];\
                            x[1][0][l] += a1[p + l] * b0[p + l]; x[1][1][l] += a1[p + l] * b1[p + l];\
                            x[2][0][l] += a2[p + l] * b0[p + l]; x[2][1][l] += a2[p + l] * b1[p + l];\
                            x[3][0][l] += a3[p + l] * b0[p + l]; x[3][1][l] += a3[p + l] * b1[p + l];\
                        }                                                                        \
                    }                                                                            \
                    for (int r = 0; r < 4; ++r)                                                  \
                        for (int c = 0; c < 2; ++c) {                                            \
                            T s = (T)0;                                                          \
                            for (int l = 0; l < LANES; ++l) s += x[r][c][l];                     \
                            T* cij = C + (i0 + i + r) * ldc + jj + j + c;                        \
                            *cij += s * alpha;                                                   \
                            const T* ar = A2 + (i + r) * KBLOCK; const T* bc = B2 + (j + c) * KBLOCK;\
                            for (int64_t p = kv; p < kb; ++p) *cij += ar[p] * bc[p] * alpha;     \
                        }                                                                        \
                }                                                                                \
                for (; j < jb; ++j)                                                              \
                    for (int r = 0; r < 4; ++r) {                                                \
                        T x1[LANES];                                                             \
                        memset(x1, 0, sizeof(x1));                                               \
                        const T* ar = A2 + (i + r) * KBLOCK; const T* bc = B2 + j * KBLOCK;      \
                        for (int64_t p = 0; p < kv; p += LANES)                                  \
                            for (int l = 0; l < LANES; ++l) x1[l] += ar[p + l] * bc[p + l];      \
                        T s = (T)0;                                                              \
                        for (int l = 0; l < LANES; ++l) s += x1[l];                              \
                        T* cij = C + (i0 + i + r) * ldc + jj + j;                                \
                        *cij += s * alpha;                                                       \
                        for (int64_t p = kv; p < kb; ++p) *cij += ar[p] * bc[p] * alpha;         \
                    }                                                                            \
            }                                                                                    \
            for (; i < isize; ++i)                                                               \
                for (int64_t j = 0; j < jb; ++j) {                                               \
                    T x1[LANES];                                                                 \
                    memset(x1, 0, sizeof(x1));                                                   \
                    const T* ar = A2 + i * KBLOCK; const T* bc = B2 + j * KBLOCK;                \
                    for (int64_t p = 0; p < kv; p += LANES)                                      \
                        for (int l = 0; l < LANES; ++l) x1[l] += ar[p + l] * bc[p + l];          \
                    T s = (T)0;                                                                  \
                    for (int l = 0; l < LANES; ++l) s += x1[l];                                  \
                    T* cij = C + (i0 + i) * ldc + jj + j;                                        \
                    *cij += s * alpha;                                                           \
                    for (int64_t p = kv; p < kb; ++p) *cij += ar[p] * bc[p] * alpha;             \
                }                                                                                \
        }                                                                                        \
    }                                                                                            \
}                                                                                                \
static void blocked_rm_##SUFFIX(int tA, int tB, int64_t m, int64_t n, int64_t k, T alpha,        \
                                const T* A, int64_t lda, const T* B, int64_t ldb, T beta, T* C,  \
                                int64_t ldc, int nthreads) {                                     \
    /* beta pre-scale, MMM.h:146-151: reset (no read) for beta == 0, scale for beta != 1 */      \
    for (int64_t i = 0; i < m; ++i) {                                                            \
        T* c = C + i * ldc;                                                                      \
        if (beta == (T)0) { for (int64_t j = 0; j < n; ++j) c[j] = (T)0; }                       \
        else if (beta != (T)1) { for (int64_t j = 0; j < n; ++j) c[j] *= beta; }                 \
    }                                                                                            \
    if (k == 0) return;                                                                          \
    int nt = nthreads > 0 ? nthreads : orc_max_threads();                                        \
    if (nt < 1) nt = 1;                                                                          \
    /* row tiles of at least 20 rows per thread, multiples of the 4-row micro-tile */            \
    int64_t chunk = (m + nt - 1) / nt;                                                           \
    chunk = ((chunk + 3) / 4) * 4;                                                               \
    if (chunk < 20) chunk = 20;                                                                  \
    const int64_t ntiles = (m + chunk - 1) / chunk;                                              \
    _Pragma("omp parallel for num_threads(nt) schedule(static)")                                 \
    for (int64_t t = 0; t < ntiles; ++t) {                                                       \
        const int64_t i0 = t * chunk;                                                            \
        const int64_t i1 = (i0 + chunk < m) ? i0 + chunk : m;                                    \
        T* A2 = (T*)malloc(sizeof(T) * (size_t)(i1 - i0) * KBLOCK);                              \
        T* B2 = (T*)malloc(sizeof(T) * (size_t)JBLOCK * KBLOCK);                                 \
        blocked_rows_##SUFFIX(tA, tB, i0, i1, n, k, alpha, A, lda, B, ldb, C, ldc, A2, B2);      \
        free(A2);                                                                                \
        free(B2);                                                                                \
    }                                                                                            \
}                                                                                                \
void orc_gemm_blocked_##SUFFIX(int order, int transA, int transB, int64_t m, int64_t n,         \
                               int64_t k, T alpha, const T* A, int64_t lda, const T* B,          \
                               int64_t ldb, T beta, T* C, int64_t ldc, int nthreads) {           \
    const int tA = (transA != ORC_NO_TRANS), tB = (transB != ORC_NO_TRANS);                      \
    if (m <= 0 || n <= 0) return;                                                                \
    if (order == ORC_ROW_MAJOR)                                                                  \
        blocked_rm_##SUFFIX(tA, tB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, nthreads);     \
    else                                                                                         \
        blocked_rm_##SUFFIX(tB, tA, n, m, k, alpha, B, ldb, A, lda, beta, C, ldc, nthreads);     \
}

DEFINE_BLOCKED(d, double, KBLOCK_D, LANES_D)
DEFINE_BLOCKED(s, float, KBLOCK_S, LANES_S)

/* ---- triangular solve (the CBLAS ?trsm definition) ---------------------------------------------
 * T X = X in place by substitution: T is ka x ka dense row-major, lower (forward substitution) or
 * upper (back substitution), with its diagonal as given (a unit diagonal is already ones); X is
 * ka x nrhs row-major.  cplx != 0: both hold interleaved complex doubles.  Row i of X is finished
 * as X_i = (X_i - sum_{k before i} T_ik X_k) / T_ii, the order of reference BLAS's row-oriented
 * left-side loops; the complex division is the textbook formula. */
void orc_trsm_left(int cplx, int lower, int64_t ka, int64_t nrhs, const double* T, double* X) {
    const int64_t w = cplx ? 2 : 1;
    for (int64_t s = 0; s < ka; ++s) {
        const int64_t i = lower ? s : ka - 1 - s;
        double* xi = X + i * nrhs * w;
        const int64_t k0 = lower ? 0 : i + 1, k1 = lower ? i : ka;
        for (int64_t k = k0; k < k1; ++k) {
            const double* t = T + (i * ka + k) * w;
            const double* xk = X + k * nrhs * w;
            if (!cplx) {
                for (int64_t j = 0; j < nrhs; ++j) xi[j] -= t[0] * xk[j];
            } else {
                for (int64_t j = 0; j < nrhs; ++j) {
                    const double ar = xk[2 * j], ai = xk[2 * j + 1];
                    xi[2 * j] -= t[0] * ar - t[1] * ai;
                    xi[2 * j + 1] -= t[0] * ai + t[1] * ar;
                }
            }
        }
        const double* d = T + (i * ka + i) * w;
        if (!cplx) {
            for (int64_t j = 0; j < nrhs; ++j) xi[j] /= d[0];
        } else {
            const double den = d[0] * d[0] + d[1] * d[1];
            for (int64_t j = 0; j < nrhs; ++j) {
                const double ar = xi[2 * j], ai = xi[2 * j + 1];
                xi[2 * j] = (ar * d[0] + ai * d[1]) / den;
                xi[2 * j + 1] = (ai * d[0] - ar * d[1]) / den;
            }
        }
    }
}
