/*
 * oracle.h — CPU oracle for the dense matrix-multiplication path (C = alpha*op(A)*op(B) + beta*C).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU kernels: the parity tests,
 * smoke() and bench.py's CPU-baseline leg call it.  Nothing in the shipped library (libgb300blas)
 * links or calls it, and the GPU path never falls back to it.
 *
 * Contents
 *   - seeded input generators (MT19937, the 1998 Matsumoto–Nishimura generator, with 53-bit
 *     uniform doubles) for the two input distributions of the workload: uniform [lo,hi] and the
 *     exponent-spread form u*2^e (u in [1,2), random sign, integer e in [emin,emax]);
 *   - a plain C restatement of Blaze's CPU GEMM kernels with CBLAS argument semantics
 *     (order, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc):
 *       * orc_gemm_default_*  — the scalar i-k-j default kernel
 *         (blaze/math/expressions/DMatDMatMultExpr.h:590-681; the dot-product default kernel of
 *         DMatTDMatMultExpr.h:566-665 accumulates each element in the same k order);
 *       * orc_gemm_blocked_*  — the packed/blocked large kernel `mmm`
 *         (blaze/math/dense/MMM.h:105-600): beta pre-scale (reset when beta==0, so C is not read),
 *         KBLOCK = 112*16/sizeof(T) k-panels of A packed row-major, JBLOCK = 96 column panels of
 *         B packed column-major, lane-split partial sums of width SIMDSIZE reduced with a
 *         horizontal sum and added as C(i,j) += sum*alpha per k-panel.  Rows of C are split
 *         across OpenMP threads the way Blaze's SMP layer splits C into thread tiles
 *         (blaze/math/smp/openmp/DenseMatrix.h:97-160).
 *   - a compensated (Ogita–Rump–Oishi Dot2) FP64 product for normwise error measurement, on all
 *     rows or on a sampled row subset;
 *   - Frobenius norms and the normwise error ||C - Cref||_F / (||A||_F ||B||_F).
 *
 * Parity pin: the restatement is checked against Blaze itself (oracle/_ref/libblazeref.so, built
 * from the reference headers by oracle/Makefile) through golden fixtures committed under
 * tests/golden/ (generated by tests/golden/make_golden.py).
 */
#ifndef GB300_ORACLE_H
#define GB300_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* CBLAS enum values (standard CBLAS ABI: blaze/math/blas/cblas/gemm.h passes these through). */
enum { ORC_ROW_MAJOR = 101, ORC_COL_MAJOR = 102, ORC_NO_TRANS = 111, ORC_TRANS = 112 };

/* ---- generators ---------------------------------------------------------------------------- */
void orc_fill_uniform_d(double* x, int64_t n, uint32_t seed, double lo, double hi);
void orc_fill_uniform_s(float* x, int64_t n, uint32_t seed, float lo, float hi);
void orc_fill_spread_d(double* x, int64_t n, uint32_t seed, int emin, int emax);
void orc_fill_spread_s(float* x, int64_t n, uint32_t seed, int emin, int emax);
/* Integer-valued uniform in [lo,hi] (blazetest's integer operand type), stored as double. */
void orc_fill_int_d(double* x, int64_t n, uint32_t seed, int lo, int hi);
/* Raw MT19937 outputs, for pinning the generator against its published first outputs. */
void orc_mt19937_raw(uint32_t seed, uint32_t* out, int64_t n);

/* ---- Blaze kernels (CBLAS argument semantics) ---------------------------------------------- */
void orc_gemm_default_d(int order, int transA, int transB, int64_t m, int64_t n, int64_t k,
                        double alpha, const double* A, int64_t lda, const double* B, int64_t ldb,
                        double beta, double* C, int64_t ldc);
void orc_gemm_default_s(int order, int transA, int transB, int64_t m, int64_t n, int64_t k,
                        float alpha, const float* A, int64_t lda, const float* B, int64_t ldb,
                        float beta, float* C, int64_t ldc);
/* nthreads <= 0 selects the OpenMP default. */
/* Blaze's register-blocked small kernel (see oracle_blaze.c); same arguments as above. */
void orc_gemm_small_d(int order, int transA, int transB, int64_t m, int64_t n, int64_t k,
                      double alpha, const double* A, int64_t lda, const double* B, int64_t ldb,
                      double beta, double* C, int64_t ldc);
void orc_gemm_small_s(int order, int transA, int transB, int64_t m, int64_t n, int64_t k,
                      float alpha, const float* A, int64_t lda, const float* B, int64_t ldb,
                      float beta, float* C, int64_t ldc);
/* The small kernel over `count` products: desc holds 12 integers per product (order, transA,
 * transB, m, n, k, lda, ldb, ldc, and the element offsets of A, B and C in the three buffers),
 * ab holds alpha and beta per product; products are spread over nthreads (<= 0: all) threads. */
void orc_gemm_batch_small_d(int64_t count, const int64_t* desc, const double* ab, const double* A,
                            const double* B, double* C, int nthreads);
void orc_gemm_batch_small_s(int64_t count, const int64_t* desc, const float* ab, const float* A,
                            const float* B, float* C, int nthreads);
void orc_gemm_blocked_d(int order, int transA, int transB, int64_t m, int64_t n, int64_t k,
                        double alpha, const double* A, int64_t lda, const double* B, int64_t ldb,
                        double beta, double* C, int64_t ldc, int nthreads);
void orc_gemm_blocked_s(int order, int transA, int transB, int64_t m, int64_t n, int64_t k,
                        float alpha, const float* A, int64_t lda, const float* B, int64_t ldb,
                        float beta, float* C, int64_t ldc, int nthreads);

/* ---- compensated reference ------------------------------------------------------------------ */
/* Rows `rows[0..nrows)` of the logical m x n product P = op(A)*op(B), computed with Dot2 and
 * written row-major to P (nrows x n, leading dimension n).  rows == NULL means all m rows. */
void orc_product_rows_dot2(int order, int transA, int transB, int64_t m, int64_t n, int64_t k,
                           const double* A, int64_t lda, const double* B, int64_t ldb,
                           const int64_t* rows, int64_t nrows, double* P, int nthreads);
/* Frobenius norm of a stored matrix (rows x cols, leading dimension ld, row-major storage
 * when rowmajor != 0), accumulated in compensated arithmetic. */
double orc_fro_norm_d(const double* X, int64_t rows, int64_t cols, int64_t ld, int rowmajor);
double orc_fro_norm_s(const float* X, int64_t rows, int64_t cols, int64_t ld, int rowmajor);

/* ---- triangular solve ---------------------------------------------------------------------- */
/* T X = X in place, T ka x ka dense row-major lower (lower != 0) or upper triangular with the
 * diagonal as given, X ka x nrhs row-major; cplx != 0: interleaved complex doubles.  The CBLAS
 * ?trsm cases reduce to this one (oracle/__init__.py: trsm): a right-side solve X op(A) = B is
 * op(A)^T X^T = B^T.  ?trsm has no kernel in Blaze itself (blaze/math/blas/cblas/trsm.h hands it
 * to CBLAS), so this restates the BLAS definition; blazetest's BLAS operation test checks its
 * result the same way (blazetest/mathtest/blas/OperationTest.h:255-715: A * x == b). */
void orc_trsm_left(int cplx, int lower, int64_t ka, int64_t nrhs, const double* T, double* X);

/* Number of OpenMP threads available to the oracle. */
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
