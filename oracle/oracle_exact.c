/*
 * oracle_exact.c — seeded generators, compensated products and norms for the GEMM oracle.
 *
 * TEST INFRASTRUCTURE ONLY; see oracle.h.  Compiled with -ffp-contract=off: the error-free
 * transformations below (TwoSum, TwoProduct) are exact only when the compiler does not fuse
 * or reassociate them.
 *
 * MT19937 follows Matsumoto & Nishimura (1998); uniform doubles use the 53-bit construction
 * (a>>5, b>>6) -> (a*2^26 + b) / 2^53 of the same authors' reference code, which is also what
 * numpy's legacy RandomState.random_sample produces for the same integer seed.  The tests pin
 * both facts (the C++ standard's 10000th-output value and numpy's stream).
 *
 * The compensated product is Dot2 of Ogita, Rump and Oishi, "Accurate sum and dot product",
 * SIAM J. Sci. Comput. 26(6), 2005 (Algorithm 5.3): the result is as accurate as if computed in
 * twice the working precision and then rounded.  It serves as the FP64 reference against which
 * normwise errors ||C - Cref||_F / (||A||_F ||B||_F) are reported.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---- MT19937 -------------------------------------------------------------------------------- */
typedef struct { uint32_t mt[624]; int idx; } mt_state;

static void mt_seed(mt_state* s, uint32_t seed) {
    s->mt[0] = seed;
    for (int i = 1; i < 624; ++i)
        s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->idx = 624;
}

static uint32_t mt_next(mt_state* s) {
    if (s->idx >= 624) {
        /* the recurrence in three index ranges, so that no index needs a modulo */
        uint32_t* mt = s->mt;
        int i = 0;
        for (; i < 624 - 397; ++i) {
            const uint32_t y = (mt[i] & 0x80000000u) | (mt[i + 1] & 0x7fffffffu);
            mt[i] = mt[i + 397] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        for (; i < 623; ++i) {
            const uint32_t y = (mt[i] & 0x80000000u) | (mt[i + 1] & 0x7fffffffu);
            mt[i] = mt[i + 397 - 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        {
            const uint32_t y = (mt[623] & 0x80000000u) | (mt[0] & 0x7fffffffu);
            mt[623] = mt[396] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        s->idx = 0;
    }
    uint32_t y = s->mt[s->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

static double mt_res53(mt_state* s) {
    const uint32_t a = mt_next(s) >> 5, b = mt_next(s) >> 6;
    return ((double)a * 67108864.0 + (double)b) * (1.0 / 9007199254740992.0);
}

void orc_mt19937_raw(uint32_t seed, uint32_t* out, int64_t n) {
    mt_state s;
    mt_seed(&s, seed);
    for (int64_t i = 0; i < n; ++i) out[i] = mt_next(&s);
}

void orc_fill_uniform_d(double* x, int64_t n, uint32_t seed, double lo, double hi) {
    mt_state s;
    mt_seed(&s, seed);
    for (int64_t i = 0; i < n; ++i) x[i] = lo + (hi - lo) * mt_res53(&s);
}

void orc_fill_uniform_s(float* x, int64_t n, uint32_t seed, float lo, float hi) {
    mt_state s;
    mt_seed(&s, seed);
    for (int64_t i = 0; i < n; ++i) x[i] = (float)((double)lo + ((double)hi - (double)lo) * mt_res53(&s));
}

/* u*2^e with u uniform in [1,2), sign uniform, e uniform integer in [emin, emax]. */
static double spread_one(mt_state* s, int emin, int emax) {
    const double u = 1.0 + mt_res53(s);
    const uint32_t w = mt_next(s);
    const int e = emin + (int)((w & 0xffffu) % (uint32_t)(emax - emin + 1));
    const double v = ldexp(u, e);
    return (w >> 31) ? -v : v;
}

void orc_fill_spread_d(double* x, int64_t n, uint32_t seed, int emin, int emax) {
    mt_state s;
    mt_seed(&s, seed);
    for (int64_t i = 0; i < n; ++i) x[i] = spread_one(&s, emin, emax);
}

void orc_fill_spread_s(float* x, int64_t n, uint32_t seed, int emin, int emax) {
    mt_state s;
    mt_seed(&s, seed);
    for (int64_t i = 0; i < n; ++i) x[i] = (float)spread_one(&s, emin, emax);
}

void orc_fill_int_d(double* x, int64_t n, uint32_t seed, int lo, int hi) {
    mt_state s;
    mt_seed(&s, seed);
    const uint32_t span = (uint32_t)(hi - lo + 1);
    for (int64_t i = 0; i < n; ++i) x[i] = (double)(lo + (int)(mt_next(&s) % span));
}

/* ---- error-free transformations (Ogita–Rump–Oishi) ----------------------------------------- */
static inline void two_sum(double a, double b, double* x, double* y) {
    const double s = a + b;
    const double z = s - a;
    *y = (a - (s - z)) + (b - z);
    *x = s;
}

static inline void two_prod(double a, double b, double* x, double* y) {
    const double p = a * b;
    *y = fma(a, b, -p);
    *x = p;
}

/* Strides of op(X)(r,c) = X[r*sr + c*sc] for CBLAS (order, trans). `first` says whether the
 * matrix is the left operand (rows = i, cols = p) or the right one (rows = p, cols = j). */
static void op_strides(int order, int trans, int64_t ld, int64_t* sr, int64_t* sc) {
    const int t = (trans != ORC_NO_TRANS);
    if (order == ORC_ROW_MAJOR) { *sr = t ? 1 : ld; *sc = t ? ld : 1; }
    else                        { *sr = t ? ld : 1; *sc = t ? 1 : ld; }
}

#define DOT2_JBLOCK 64

void orc_product_rows_dot2(int order, int transA, int transB, int64_t m, int64_t n, int64_t k,
                           const double* A, int64_t lda, const double* B, int64_t ldb,
                           const int64_t* rows, int64_t nrows, double* P, int nthreads) {
    int64_t sAi, sAp, sBp, sBj;
    op_strides(order, transA, lda, &sAi, &sAp);
    op_strides(order, transB, ldb, &sBp, &sBj);
    if (rows == NULL) nrows = m;
    if (nrows <= 0 || n <= 0) return;
    if (k == 0) { memset(P, 0, sizeof(double) * (size_t)nrows * (size_t)n); return; }
    /* pack the requested rows of op(A) contiguously */
    double* Ar = (double*)malloc(sizeof(double) * (size_t)nrows * (size_t)k);
    for (int64_t r = 0; r < nrows; ++r) {
        const int64_t i = rows ? rows[r] : r;
        for (int64_t p = 0; p < k; ++p) Ar[r * k + p] = A[i * sAi + p * sAp];
    }
    int nt = nthreads > 0 ? nthreads : orc_max_threads();
    if (nt < 1) nt = 1;
    const int64_t nblk = (n + DOT2_JBLOCK - 1) / DOT2_JBLOCK;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1)
    for (int64_t jb = 0; jb < nblk; ++jb) {
        const int64_t j0 = jb * DOT2_JBLOCK;
        const int64_t j1 = (j0 + DOT2_JBLOCK < n) ? j0 + DOT2_JBLOCK : n;
        double* Bc = (double*)malloc(sizeof(double) * (size_t)(j1 - j0) * (size_t)k);
        for (int64_t j = j0; j < j1; ++j)
            for (int64_t p = 0; p < k; ++p) Bc[(j - j0) * k + p] = B[p * sBp + j * sBj];
        for (int64_t r = 0; r < nrows; ++r) {
            const double* a = Ar + r * k;
            for (int64_t j = j0; j < j1; ++j) {
                const double* b = Bc + (j - j0) * k;
                double p, s, h, q, e;
                two_prod(a[0], b[0], &p, &s);
                for (int64_t t = 1; t < k; ++t) {
                    two_prod(a[t], b[t], &h, &e);
                    two_sum(p, h, &p, &q);
                    s += q + e;
                }
                P[r * n + j] = p + s;
            }
        }
        free(Bc);
    }
    free(Ar);
}

/* Compensated sum of squares (Dot2 of the matrix with itself), then sqrt. */
#define DEFINE_NORM(SUFFIX, T)                                                                    \
double orc_fro_norm_##SUFFIX(const T* X, int64_t rows, int64_t cols, int64_t ld, int rowmajor) { \
    double p = 0.0, s = 0.0;                                                                      \
    for (int64_t r = 0; r < rows; ++r)                                                            \
        for (int64_t c = 0; c < cols; ++c) {                                                      \
            const double v = (double)(rowmajor ? X[r * ld + c] : X[c * ld + r]);                  \
            double h, e, q;                                                                       \
            two_prod(v, v, &h, &e);                                                               \
            two_sum(p, h, &p, &q);                                                                \
            s += q + e;                                                                           \
        }                                                                                         \
    return sqrt(p + s);                                                                           \
}

DEFINE_NORM(d, double)
DEFINE_NORM(s, float)
