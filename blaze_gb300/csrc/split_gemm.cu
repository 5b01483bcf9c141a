// split_gemm.cu — K2/K3: the tensor-core forms of the double-precision product on sm_103a.
//
//   GB300_METHOD_SPLIT   Ozaki-style split-precision product that reaches FP64-level normwise
//                        accuracy: A and B are scaled per row / per column by powers of two and
//                        cut into BF16 "digit" slices; the slice products run on tcgen05 tensor
//                        cores (FP32 accumulators in TMEM) in groups whose sums stay exactly
//                        representable, so every partial product is an exact integer; the
//                        integers are accumulated exactly (int32) and only the final
//                        recombination, the exponent rescale and alpha/beta run in FP64.
//   GB300_METHOD_BF16X3  hi*hi + hi*lo + lo*hi with BF16 hi/lo parts, FP32 accumulation.
//   GB300_METHOD_BF16    one BF16 product, FP32 accumulation.
//   GB300_METHOD_AUTO    the split form when it is predicted faster than the native kernel.
//
// They replace the same CBLAS dgemm call as the native kernel (blaze/math/blas/cblas/gemm.h:
// 156-162, reached from DMatDMatMultExpr.h:2021-2037 and siblings).
//
// ---- split arithmetic --------------------------------------------------------------------------
// Row i of op(A) is scaled by 2^-e_i with e_i = frexp exponent of max_p |A(i,p)|, so the scaled
// entries x satisfy |x| < 1.  Digits: d_1 = rint(x*2^7), r_1 = x*2^7 - d_1, then
// d_s = rint(r_{s-1}*2^8), r_s = r_{s-1}*2^8 - d_s (all exact in FP64; |d_s| <= 128, |r_s| <= 1/2),
// so x = sum_s d_s 2^(1-8s) + r_S 2^(1-8S).  Columns of op(B) likewise with exponents f_j.
// With planes numbered a = s-1, the pair (a, b) has weight 2^(-14-8(a+b)); all pairs with
// a + b = L form "level" L, L = 0..S-1 (the triangle s + t <= S + 1 of Ozaki's scheme).
//   Exactness: one TMEM drain group accumulates at most 16 x 64 = 1024 products of digits,
//   |product| <= 128^2 = 2^14, so every partial sum is an integer of magnitude at most 2^24, which
//   FP32 holds exactly (2^24 itself only as the group's final value, when all 1024 products are
//   largest with one sign).  The epilogue converts the FP32 integer v with cvt.rni (exact) and
//   adds it in int32.  A level's int32 sum over a k-segment is bounded by
//   n_L * Kseg * 2^14 < 2^31.
//   Error bound (elementwise, scaled units): |dC_ij| <= (S+1) K 2^(-8S); normwise
//   ||dC||_F / (||A||_F ||B||_F) <= (S+1) K 2^(-8S) ||2^e||_2 ||2^f||_2 / (||A||_F ||B||_F)
//   plus (S+3) 2^-53 for the FP64 recombination.  The slice count is the smallest S whose bound
//   meets the target (default K * 2^-53, the classical worst-case FP64 dot-product bound); it is
//   chosen on the device, so the whole product is stream-ordered without a host round trip.
//
// ---- kernel structure (tc_gemm_kernel) ---------------------------------------------------------
// Persistent CTAs, one per SM, each owning whole 128 x 256 output tiles (and a k-segment).
//   warp 0      TMA producer: 128x64 A-plane box + 256x64 B-plane box per item, 128B swizzle,
//               4-stage ring of 48 KB stages.
//   warp 1      TMEM allocator and MMA issuer: 4 x tcgen05.mma (M=128, N=256, K=16, BF16->FP32)
//               per item; tcgen05.commit releases the smem stage and, at the end of a drain
//               group, hands the accumulator buffer to the epilogue.  Two 256-column TMEM
//               accumulators let the MMAs of one group overlap the drain of the previous one.
//   warps 2-9   epilogue: tcgen05.ld of its 32 lanes x 128 columns, exact integer accumulation
//               in registers, and at each level end a store of the int32 level sums (float
//               modes: the FP32 tile) to the level planes in global memory.
// A separate combine kernel forms C = alpha * 2^(e_i+f_j) * sum_L 2^(-14-8L) T_L + beta*C in FP64
// (float modes: alpha * sum of segment partials + beta*C).  Every wait is bounded.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <cmath>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/gb300_blas.h"
#include "gb300_internal.h"
#include "ptx.cuh"
#include "runtime.h"
#include "profile.h"
#include "split_api.h"
#include "crt_tables.h"

namespace gb {
namespace {

constexpr int TM = 128;                 // A rows held by each CTA of a pair
constexpr int TN = 256;                 // tile cols (pair MMA N)
constexpr int TMP = 2 * TM;             // rows of a CTA pair's tile (pair MMA M = 256)
constexpr int TNH = TN / 2;             // B rows (tile columns) held by each CTA of the pair
constexpr int TK = 64;                  // k per item (one 128-byte swizzle row of bf16)
constexpr int STAGES = 6;
constexpr int A_BYTES = TM * TK * 2;    // 16 KB
constexpr int B_BYTES = TNH * TK * 2;   // 16 KB (this CTA's half of the B tile)
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int GROUP_ITEMS = 16;         // exact mode: 16 items (1024 products) per TMEM drain
constexpr int EPI_WARPS = 8;
constexpr int THREADS = 64 + EPI_WARPS * 32;
constexpr int MAX_SLICES = 10;
constexpr int KSEG_UNIT = 256;          // k-segments are multiples of this
constexpr int kPipeMaxQ = 2;            // column blocks of B in the host-operand pipeline
constexpr uint32_t MAGIC_BITS = 0x4B400000u;  // bits of 1.5 * 2^23
constexpr float MAGIC = 12582912.0f;

enum Mode : int { kExact = 0, kBf16 = 1, kBf16x3 = 2, kCrt = 3 };

// ---- moduli of the CRT (Ozaki scheme II) form ----------------------------------------------------
// Pairwise coprime moduli <= 257, largest first: a residue in the symmetric range has |r| <= 128,
// so it is exactly a BF16 and a 1024-product group of residue products stays within 2^24, where
// every partial sum is an integer exact in the FP32 accumulator (the same exactness argument as
// for the digits).  Prime factors: 257; 2; 3,5,17; 11,23; 251; 13,19; 241;
// 239; 233; 229; 227; 223; 7,31; 211; 199.  Product of all 15: about 2^118.2.
constexpr int MAX_MODULI = 15;
__constant__ uint32_t c_mod[MAX_MODULI] = {257, 256, 255, 253, 251, 247, 241, 239, 233, 229, 227, 223, 217, 211, 199};
// floor(2^32 / p) for the reduction of 32-bit values.
__constant__ uint32_t c_mod_inv32[MAX_MODULI] = {
    16711935u, 16777216u, 16843009u, 16976155u, 17111423u, 17388531u, 17821441u, 17970574u,
    18433336u, 18755315u, 18920560u, 19259943u, 19792476u, 20355295u, 21582750u};
// log2 of each modulus (device copy: the plan kernels sum these instead of calling log2).
__constant__ double c_mod_log2[MAX_MODULI] = {
    8.005624549193879, 8.0, 7.994353436858858, 7.98299357469431, 7.971543553950772, 7.948367231584678,
    7.912889336229962, 7.900866807980749, 7.864186144654281, 7.839203788096944, 7.826548487290915,
    7.800899899920305, 7.7615512324444795, 7.721099188707185, 7.636624620543649};
// log2 of the running products of the moduli (host-side copy for the worst-case plan).
constexpr double kModLog2[MAX_MODULI] = {8.00562, 8.0, 7.99435, 7.98299, 7.97154, 7.94837, 7.91289, 7.90087,
                                         7.86419, 7.83920, 7.82655, 7.80090, 7.76155, 7.72110, 7.63662};

// Residues on the FP32 pipe: a 56-bit integer U = sum_i w_i 2^(14 i) (14-bit chunks, i = 0..3) is
// congruent to x = w_0 + sum_{i>0} w_i K_i with K_i = 2^(14 i) mod p in the symmetric range
// (|K_i| <= 128), so |x| <= 16383 * 385 < 2^23 and every partial sum is an exact FP32 integer.
// q = rint(x fl(1/p)) is the nearest integer to x / p: the relative error 2^-24 of fl(1/p) moves
// x / p by less than 2^23 / p * 2^-24 = 0.5 / p, the smallest distance of x / p from a half
// integer for odd p (p = 256 is exact), so r = x - p q lies in [-p/2, p/2] and |r| <= 128.
__constant__ float c_modf[MAX_MODULI] = {257.f, 256.f, 255.f, 253.f, 251.f, 247.f, 241.f, 239.f,
                                         233.f, 229.f, 227.f, 223.f, 217.f, 211.f, 199.f};
__constant__ float c_modf_inv[MAX_MODULI] = {
    0x1.fe01fe0000000p-9f, 0x1.0000000000000p-8f, 0x1.0101020000000p-8f, 0x1.03091c0000000p-8f,
    0x1.0519800000000p-8f, 0x1.0953f40000000p-8f, 0x1.0fef020000000p-8f, 0x1.12358e0000000p-8f,
    0x1.1945380000000p-8f, 0x1.1e2ef40000000p-8f, 0x1.20b4700000000p-8f, 0x1.25e2280000000p-8f,
    0x1.2e025c0000000p-8f, 0x1.3698e00000000p-8f, 0x1.49539e0000000p-8f};
__constant__ float c_mod_k14[3][MAX_MODULI] = {
    {-64.f, 0.f, 64.f, -61.f, 69.f, 82.f, -4.f, -107.f, 74.f, -104.f, 40.f, 105.f, -108.f, -74.f, 66.f},
    {-16.f, 0.f, 16.f, -74.f, -8.f, 55.f, 16.f, -23.f, -116.f, 53.f, 11.f, 98.f, -54.f, -10.f, -22.f},
    {-4.f, 0.f, 4.f, -40.f, -50.f, 64.f, -64.f, 71.f, 37.f, -16.f, -14.f, 32.f, -27.f, -104.f, -59.f}};

// Device-side result of the pre-pass: the slice count and the bound it guarantees.
struct SplitInfo {
    int slices;           // S (digit mode); residue products N (CRT mode); planes per operand otherwise
    int nonfinite;        // inputs contained Inf/NaN
    double bound;         // a-priori normwise bound of the result
    double normA, normB;  // Frobenius norms
    double scaleA, scaleB;// ||2^e||_2, ||2^f||_2
    // CRT mode
    int beta;             // rows of A are rounded to beta-bit integers
    int beta_b;           // columns of B are rounded to beta_b-bit integers (= beta unless B is sliced
                          // ahead of A, in the panel pipeline for host operands)
    double qmaxB;         // largest column sum of squares of B relative to 2^(2f)
    double qmaxA;         // largest row sum of squares of A relative to 2^(2e) (block pipeline)
};

// ---- pre-pass ------------------------------------------------------------------------------
// Row statistics of a logical R x K operand X(r,p) = X[r*sr + p*sp]: e_r = frexp exponent of
// max |X(r,:)| (kNonFinite if the row holds Inf/NaN) and q_r = sum_p (X(r,p) * 2^-e_r)^2, the
// row's sum of squares relative to 2^(2 e_r) (so that norms of huge or tiny inputs stay finite).
//
// stats_tile_kernel reads 32-row x 64-k tiles (coalesced along whichever dimension is
// contiguous, like slice_kernel) and folds each row's tile maximum and sum of squares into
// per-row accumulators with atomics; stats_finalize_kernel turns them into (e_r, q_r).  A row
// whose values leave [2^-500, 2^500] would over- or underflow the unscaled sum of squares; the
// finalize kernel recomputes such (rare) rows on scaled values.
constexpr int kNonFinite = 0x7fff;

struct RowAcc {
    // max |x| to its high 32 bits (sign, exponent, 20 mantissa bits; non-negative doubles order
    // like integers), bit 0 set when some value has non-zero low bits: the frexp exponent of the
    // maximum follows whenever the high word is a normal number, and a row whose high words are
    // all zero or subnormal is rescanned exactly
    unsigned long long maxbits;
    double sumsq;
    int flags;                   // 1: non-finite value seen
    int pad;
};

// Operands stream through shared memory in tiles of 32 rows x 64 k, TILE_KT tiles per block, with
// two buffers filled by cp.async: the copies of the next tile are in flight while the current one
// is processed.
constexpr int TILE_KT = 8;

// The eight copies of one thread per tile: element (rr0 + i drr, pp0 + i dpp) of the tile,
// i = 0..7, coalesced along whichever index of X(r, p) = X[r*sr + p*sp] is contiguous (a warp
// reads 256 consecutive bytes); src points at the first one in tile 0, di and dk step to copy i
// and to the next tile of 64 k.
struct TileSrc {
    const unsigned long long* src;
    int64_t di, dk;
    int rr0, pp0, drr, dpp;
};

__device__ __forceinline__ TileSrc tile_src(const double* X, int64_t sr, int64_t sp, int64_t r0) {
    const int t = threadIdx.x;  // 256 threads
    TileSrc s;
    if (sp == 1) {
        s.rr0 = t >> 6; s.drr = 4; s.pp0 = t & 63; s.dpp = 0;
        s.di = 4 * sr;
        s.dk = 64;
    } else {
        s.rr0 = t & 31; s.drr = 0; s.pp0 = t >> 5; s.dpp = 8;
        s.di = 8 * sp;
        s.dk = 64 * sp;
    }
    s.src = reinterpret_cast<const unsigned long long*>(X) + (r0 + s.rr0) * sr + int64_t(s.pp0) * sp;
    return s;
}

// Issue the copies of tile `it` (k from 64 it) into the buffer at shared address sbuf, where
// off(rr, pp) places element (rr, pp); zeros outside R x K; one commit group per tile.
template <typename Off>
__device__ __forceinline__ void tile_issue(uint32_t sbuf, const TileSrc& s, const double* X, int64_t R, int64_t K,
                                           int64_t r0, int64_t it, Off off) {
    const unsigned long long* src = s.src + it * s.dk;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int rr = s.rr0 + i * s.drr, pp = s.pp0 + i * s.dpp;
        const bool ok = r0 + rr < R && it * 64 + pp < K;
        cp_async8(sbuf + off(rr, pp), ok ? src + i * s.di : reinterpret_cast<const unsigned long long*>(X), ok);
    }
    cp_async_commit();
}

// 2^x in FP32 for x <= 127, 0 below the normal range.
__device__ __forceinline__ float pow2f_or0(int x) { return x < -126 ? 0.f : __uint_as_float(uint32_t(x + 127) << 23); }

// Row statistics over TILE_KT tiles: thread (rr = t % 32, g = t / 32) keeps, for row rr and the
// eight k of group g in every tile, the largest high word of |x|, the OR of the low words and the
// sum of squares in FP32 relative to its running largest exponent `base`: f = |x| 2^(1023 - base)
// is the high word times 8 (exponent and 20 mantissa bits moved into FP32 position) minus
// (base - 127) 2^23, one integer multiply-add, valid for exponents above base - 127 (smaller
// values add less than 2^-252 relative and are dropped; zeros and subnormals always are).  The
// running sum is rescaled exactly by a power of two when a larger exponent arrives.  The block
// folds the eight groups of a row and issues one set of atomics per row; an Inf/NaN shows as a
// largest exponent of 0x7ff.
__device__ __forceinline__ void stats_rows(const double* __restrict__ X, int64_t R, int64_t K, int64_t sr, int64_t sp,
                                           RowAcc* __restrict__ acc, int by) {
    __shared__ __align__(16) unsigned long long tile[2][32][65];
    __shared__ uint32_t red_mx[8][32], red_lo[8][32];
    __shared__ int red_base[8][32];
    __shared__ float red_sq[8][32];
    const int t = threadIdx.x, rr = t & 31, g = t >> 5;
    const int64_t r0 = int64_t(by) * 32;
    const int64_t ntiles = (K + 63) / 64;
    const int64_t tb = int64_t(blockIdx.x) * TILE_KT, te = min(ntiles, tb + TILE_KT);
    const uint32_t s0 = smem_u32(&tile[0][0][0]);
    constexpr uint32_t BUF = 32 * 65 * 8;
    auto off = [](int r_, int p_) { return uint32_t(r_ * 65 + p_) * 8u; };
    uint32_t mx = 0, lo = 0, cbias = 0;
    int base = 127;  // f = |x| 2^(1023 - base); values with exponent field 0 never count
    float sq = 0.f;
    const TileSrc ts = tile_src(X, sr, sp, r0);
    if (tb < te) tile_issue(s0, ts, X, R, K, r0, tb, off);
    for (int64_t it = tb; it < te; ++it) {
        const int b = int(it - tb) & 1;
        if (it + 1 < te) tile_issue(s0 + uint32_t(b ^ 1) * BUF, ts, X, R, K, r0, it + 1, off);
        else cp_async_commit();  // an empty group keeps the wait count uniform
        cp_async_wait1();
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const unsigned long long a = tile[b][rr][8 * g + q];
            const uint32_t hi = uint32_t(a >> 32) & 0x7fffffffu;
            lo |= uint32_t(a);
            mx = max(mx, hi);
            const int ea = int(hi >> 20);
            if (ea > base) {
                sq *= pow2f_or0(2 * (base - ea));
                base = ea;
                cbias = uint32_t(base - 127) << 23;
            }
            const float f = ea > base - 127 ? __uint_as_float(hi * 8u - cbias) : 0.f;
            sq = fmaf(f, f, sq);
        }
        __syncthreads();
    }
    red_mx[g][rr] = mx;
    red_lo[g][rr] = lo;
    red_base[g][rr] = base;
    red_sq[g][rr] = sq;
    __syncthreads();
    if (g == 0) {
        int E = 0;
        uint32_t m = 0, l = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            E = max(E, red_base[i][rr]);
            m = max(m, red_mx[i][rr]);
            l |= red_lo[i][rr];
        }
        float s = 0.f;
#pragma unroll
        for (int i = 0; i < 8; ++i) s = fmaf(red_sq[i][rr], pow2f_or0(2 * (red_base[i][rr] - E)), s);
        const int64_t r = r0 + rr;
        if (r < R) {
            if (m >= 0x7ff00000u) atomicOr(&acc[r].flags, 1);
            if (m != 0 || l != 0) {
                atomicMax(&acc[r].maxbits, ((unsigned long long)m << 32) | (l != 0 ? 1ull : 0ull));
                // sum of squares of the unscaled values: s * 2^(2 (E - 1023))
                if (s > 0.f) atomicAdd(&acc[r].sumsq, ldexp(double(s), 2 * (E - 1023)));
            }
        }
    }
}

__device__ __forceinline__ void stats_finalize_row(const double* __restrict__ X, int64_t R, int64_t K, int64_t sr,
                                                   int64_t sp, const RowAcc* __restrict__ acc, int* __restrict__ rexp,
                                                   double* __restrict__ rsq, int64_t r) {
    if (r >= R) return;
    const RowAcc a = acc[r];
    if (a.flags & 1) {
        rexp[r] = kNonFinite;
        rsq[r] = 0.0;
        return;
    }
    unsigned long long mb = a.maxbits;
    if (mb != 0 && (mb >> 52) == 0) {
        // every high word zero or subnormal: the exact maximum decides the exponent
        mb = 0;
        for (int64_t p = 0; p < K; ++p) {
            const unsigned long long v =
                static_cast<unsigned long long>(__double_as_longlong(X[r * sr + p * sp])) & 0x7fffffffffffffffull;
            mb = v > mb ? v : mb;
        }
    }
    const double mx = __longlong_as_double(static_cast<long long>(mb));
    int e = 0;
    if (mx > 0.0) frexp(mx, &e);
    double q = ldexp(a.sumsq, -2 * e);
    if (mx > 0.0 && (e > 500 || e < -500)) {
        q = 0.0;
        for (int64_t p = 0; p < K; ++p) {
            const double v = ldexp(X[r * sr + p * sp], -e);
            q = fma(v, v, q);
        }
    }
    rexp[r] = e;
    rsq[r] = q;
}

// Both operands of a product go through one launch: blocks with blockIdx.y < yb0 work on A (its
// rows), the others on B (its columns), so the two passes overlap on the device.
struct OperandPair {
    const double* X[2];
    int64_t R[2], sr[2], sp[2];
    RowAcc* acc[2];
    int* rexp[2];
    double* rsq[2];
    __nv_bfloat16* planes[2];
    int64_t rpad[2];
    unsigned yb0;  // row blocks of A
};

__global__ void __launch_bounds__(256, 4) stats_tile_kernel(const OperandPair op, int64_t K) {
    const int w = blockIdx.y < op.yb0 ? 0 : 1;
    const int by = w ? int(blockIdx.y - op.yb0) : int(blockIdx.y);
    stats_rows(op.X[w], op.R[w], K, op.sr[w], op.sp[w], op.acc[w], by);
}

// Per-block summary of the row statistics of one operand side, for split_info_kernel: Inf/NaN
// flag, largest exponent E of the rows with q > 0 (kNoRows when none), largest q (its bit pattern:
// non-negative doubles order like integers), s = sum 2^(2(e - E)) and nrm = sum 2^(2(e - E)) q.
constexpr int kNoRows = -100000;
struct RowPartial {
    int bad, E;
    long long Qbits;
    double s, nrm;
};

__device__ double block_sum(double v, double* red);
__device__ long long block_max_ll(long long v, long long* red);
__device__ int block_max_int(int v, int* red);
__device__ __forceinline__ double pow2i(int x);

// blockIdx.x < xb0: rows of A, else columns of B (256 a block); with `part`, each block also
// writes its RowPartial (part[blockIdx.x]).
__global__ void __launch_bounds__(256) stats_finalize_pair_kernel(const OperandPair op, int64_t K, unsigned xb0,
                                                                  RowPartial* __restrict__ part) {
    const int w = blockIdx.x < xb0 ? 0 : 1;
    const int64_t r = int64_t(w ? blockIdx.x - xb0 : blockIdx.x) * blockDim.x + threadIdx.x;
    stats_finalize_row(op.X[w], op.R[w], K, op.sr[w], op.sp[w], op.acc[w], op.rexp[w], op.rsq[w], r);
    if (part == nullptr) return;  // uniform over the launch
    __shared__ double redd[32];
    __shared__ int redi[32];
    int e = kNoRows, bad = 0;
    double q = 0.0;
    if (r < op.R[w]) {
        e = op.rexp[w][r];
        q = op.rsq[w][r];
        if (e == kNonFinite) {
            bad = 1;
            e = kNoRows;
            q = 0.0;
        }
    }
    const long long qb = __double_as_longlong(q);
    RowPartial pr;
    pr.bad = block_max_int(bad, redi);
    pr.E = block_max_int(qb > 0 ? e : kNoRows, redi);
    pr.Qbits = block_max_ll(qb, reinterpret_cast<long long*>(redd));
    const double wgt = (qb > 0 && pr.E != kNoRows) ? pow2i(2 * (e - pr.E)) : 0.0;
    pr.s = block_sum(wgt, redd);
    pr.nrm = block_sum(wgt * q, redd);
    if (threadIdx.x == 0) part[blockIdx.x] = pr;
}

// One block: norms, scale norms, slice count and bound.  Sums are formed relative to the largest
// row exponent, so the ratio rho = ||2^e|| ||2^f|| / (||A|| ||B||) is finite for any finite input.
//
// On GB300 every FP64 warp instruction occupies the narrow FP64 pipe for many cycles whatever the
// number of active lanes, so these planning kernels keep FP64 work off long serial chains: block
// sums finish in one warp's shuffles, and the searches below test 32 candidates per instruction.
__device__ double block_sum(double v, double* red) {
    __shared__ double total;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) total = t;
    }
    __syncthreads();
    return total;
}

// Smallest b in [lo, hi] with ok(b), hi + 1 when there is none (ok false, then true as b grows):
// the 32 lanes of the calling warp test 32 candidates at a time.
template <typename F>
__device__ int warp_first_true(int lo, int hi, F ok) {
    const int lane = threadIdx.x & 31;
    for (int base = lo; base <= hi; base += 32) {
        const int b = base + lane;
        const unsigned m = __ballot_sync(0xffffffffu, b <= hi && ok(b));
        if (m) return base + __ffs(int(m)) - 1;
    }
    return hi + 1;
}

// Largest b in [lo, hi] with ok(b), lo - 1 when there is none (ok true, then false as b grows).
template <typename F>
__device__ int warp_last_true(int lo, int hi, F ok) {
    const int lane = threadIdx.x & 31;
    for (int base = hi; base >= lo; base -= 32) {
        const int b = base - lane;
        const unsigned m = __ballot_sync(0xffffffffu, b >= lo && ok(b));
        if (m) return base - (__ffs(int(m)) - 1);
    }
    return lo - 1;
}

__device__ long long block_max_ll(long long v, long long* red) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    long long t = red[0];
    for (int i = 1; i < int(blockDim.x >> 5); ++i) t = max(t, red[i]);
    return t;
}

__device__ int block_max_int(int v, int* red) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = red[0];
    for (int i = 1; i < int(blockDim.x >> 5); ++i) t = max(t, red[i]);
    return t;
}

// 2^x for an integer x <= 0 from the bit pattern (0 below the normal range, where the weight of a
// row in a norm sum no longer matters)
__device__ __forceinline__ double pow2i(int x) {
    return x < -1022 ? 0.0 : __longlong_as_double((long long)(x + 1023) << 52);
}

// One warp: the partials are few (one per 256 rows or columns), and the shuffle reductions need no
// barriers.  A block of 1024 threads spent most of the kernel's 25 us in the barriers and the
// serial combining steps of nine block-wide reductions.
__device__ __forceinline__ int warp_max(int v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ long long warp_max(long long v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(32) split_info_kernel(const RowPartial* __restrict__ part, int nA, int nB, int64_t k,
                                                         int mode, int fixed_slices, int cap_planes, double target,
                                                         SplitInfo* info) {
    // the per-block partials of A (the first nA) and B: Inf/NaN flag, largest exponents, largest
    // row / column sums of squares relative to 2^(2e)
    int bad = 0, EA = kNoRows, EB = kNoRows;
    long long QAb = 0, QBb = 0;
    for (int i = threadIdx.x; i < nA + nB; i += 32) {
        const RowPartial p = part[i];
        bad |= p.bad;
        if (i < nA) {
            EA = max(EA, p.E);
            QAb = max(QAb, p.Qbits);
        } else {
            EB = max(EB, p.E);
            QBb = max(QBb, p.Qbits);
        }
    }
    bad = warp_max(bad);
    EA = warp_max(EA);
    EB = warp_max(EB);
    const double QA = __longlong_as_double(warp_max(QAb));
    const double QB = __longlong_as_double(warp_max(QBb));
    // the sums relative to the largest exponent: each block's relative to its own, rescaled by an
    // exact power of two
    double sa = 0, na = 0, sb = 0, nb = 0;
    for (int i = threadIdx.x; i < nA + nB; i += 32) {
        const RowPartial p = part[i];
        if (p.E == kNoRows) continue;
        if (i < nA) {
            const double w = pow2i(2 * (p.E - EA));
            sa += w * p.s;
            na += w * p.nrm;
        } else {
            const double w = pow2i(2 * (p.E - EB));
            sb += w * p.s;
            nb += w * p.nrm;
        }
    }
    sa = warp_sum(sa);
    na = warp_sum(na);
    sb = warp_sum(sb);
    nb = warp_sum(nb);
    if (threadIdx.x < 32) {  // warp 0 plans; lane 0 writes
        const int lane = threadIdx.x;
        // Each FP64 function below runs once for the warp with a different argument in each lane
        // (the cost of one evaluation, same operations as one at a time): lanes 0-3 the norms, 4-5
        // sqrt(k s / n), 6-7 sqrt(Q (1 + 2^-10)), 8 sqrt(k), 9-10 sqrt(s / n).
        double num = 0.0, den = 1.0;
        switch (lane) {
            case 0: num = na; break;
            case 1: num = nb; break;
            case 2: num = sa; break;
            case 3: num = sb; break;
            case 4: num = double(k) * sa; den = na > 0 ? na : 1.0; break;
            case 5: num = double(k) * sb; den = nb > 0 ? nb : 1.0; break;
            case 6: num = QA * (1.0 + 0x1p-10); break;
            case 7: num = QB * (1.0 + 0x1p-10); break;
            case 8: num = double(k); break;
            case 9: num = sa; den = na > 0 ? na : 1.0; break;
            case 10: num = sb; den = nb > 0 ? nb : 1.0; break;
            default: break;
        }
        const double root = sqrt(num / den);
        const double scaled = ldexp(root, (lane == 0 || lane == 2) ? EA : EB);  // lanes 0-3
        auto from = [&](double v, int l) { return __shfl_sync(0xffffffffu, v, l); };
        const double nA_ = from(scaled, 0), nB_ = from(scaled, 1), sA_ = from(scaled, 2), sB_ = from(scaled, 3);
        const double rAk = from(root, 4), rBk = from(root, 5), sqa = from(root, 6), sqb = from(root, 7);
        const double sqk = from(root, 8), ra = from(root, 9), rb = from(root, 10);
        SplitInfo r;
        r.nonfinite = bad;
        r.normA = (na > 0) ? nA_ : 0.0;
        r.normB = (nb > 0) ? nB_ : 0.0;
        r.scaleA = (sa > 0) ? sA_ : 0.0;
        r.scaleB = (sb > 0) ? sB_ : 0.0;
        const double rho = (na > 0 && nb > 0) ? ra * rb : 0.0;
        if (mode == kCrt) {
            // operands rounded to beta-bit integers: |dA_ip| <= 2^(e_i-beta-1), so
            // ||dC||_F/(||A|| ||B||) <= 2^(-beta-1)(rA + rB) + 2^(-2beta-2) rA rB + 2^-52 with
            // rA = sqrt(k) ||2^e|| / ||A|| (and 2^-52 for the final conversion and the alpha scaling)
            const double rA = (na > 0) ? rAk : 0.0;
            const double rB = (nb > 0) ? rBk : 0.0;
            auto bnd = [&](int b) {
                return pow2i(-b - 1) * (rA + rB) + pow2i(-2 * b - 2) * rA * rB + pow2i(-52);
            };
            // the smallest beta in [1, 55] that meets the target (beta <= 55 keeps |A'| < 2^56, the
            // range of the residue extraction)
            int beta = min(55, warp_first_true(1, 54, [&](int b) { return bnd(b) <= target; }));
            // The scaled rows satisfy ||A'_i|| <= 2^beta sqrt(Q_A) + sqrt(k)/2 (the rounding adds
            // at most 1/2 per entry), so by Cauchy-Schwarz every exact product entry T has
            // |T| <= (2^beta sqrt(Q_A) + sqrt(k)/2)(2^beta sqrt(Q_B) + sqrt(k)/2).  The moduli's
            // product P must exceed 2.125 |T| (symmetric residues, with room for the FP32 quotient
            // estimate of the reconstruction); Q carries a 2^-10 allowance for its own rounding.
            const double hk = 0.5 * sqk;
            auto need = [&](int b) {
                const double x = ldexp(sqa, b) + hk, y = ldexp(sqb, b) + hk;
                return 1.0875 + log2(x) + log2(y);
            };
            // lanes 0-1: the two factors of need(beta); lanes 2-3: log2 sqa and log2 sqb
            const double lg = log2(ldexp((lane & 1) ? sqb : sqa, lane < 2 ? beta : 0) + (lane < 2 ? hk : 0.0));
            const double lg0 = from(lg, 0), lg1 = from(lg, 1), lsqa = from(lg, 2), lsqb = from(lg, 3);
            double have = 0.0;
            // a fixed count is used as given (at least two); otherwise the fewest that carry the
            // target, within the planes the host sized for
            int N = 0;
            const int nfix = fixed_slices > 0 ? (fixed_slices < 2 ? 2 : fixed_slices) : 0;
            const double need0 = 1.0875 + lg0 + lg1;  // need(beta)
            while (nfix ? N < nfix : (N < 2 || (N < cap_planes && have < need0))) {
                have += c_mod_log2[N];
                ++N;
            }
            // the moduli chosen may carry more bits than needed: round to as many bits as they allow.
            // need(b) exceeds 1.0875 + 2b + log2(sqa sqb), so no b above b0 qualifies: the largest b
            // in (-60, b0] with need(b) <= have, -60 when none
            int bhi = 55;
            if (sqa > 0 && sqb > 0) {
                const int b0 = int(floor((have - 1.0875 - lsqa - lsqb) / 2.0));
                bhi = b0 < 55 ? (b0 > -60 ? b0 : -60) : 55;
            }
            beta = warp_last_true(-59, bhi, [&](int b) { return need(b) <= have; });
            r.slices = N;
            r.beta = beta;
            r.beta_b = beta;
            r.qmaxB = QB;
            // a beta the search found has need(beta) <= have; -60 (none found) was not tested.  Too
            // few moduli for even the coarsest rounding: no bound
            const bool fits = beta >= -59 || need(beta) <= have;
            r.bound = fits ? bnd(beta) : __longlong_as_double(0x7ff0000000000000ll);
        } else if (mode == kExact) {
            int S = fixed_slices;
            if (S <= 0) {
                S = MAX_SLICES;
                for (int s = 2; s <= MAX_SLICES; ++s) {
                    const double b = (s + 1) * double(k) * ldexp(1.0, -8 * s) * rho + (s + 3) * ldexp(1.0, -53);
                    if (b <= target) { S = s; break; }
                }
            }
            r.slices = S;
            r.bound = (S + 1) * double(k) * ldexp(1.0, -8 * S) * rho + (S + 3) * ldexp(1.0, -53);
        } else if (mode == kBf16) {
            // each operand rounded to 8 significant bits, FP32 accumulation
            r.slices = 1;
            r.bound = 2.0 * ldexp(1.0, -8) + double(k) * ldexp(1.0, -24);
        } else {
            // hi/lo split keeps 16 bits; the dropped lo*lo term and the FP32 accumulation remain
            r.slices = 2;
            r.bound = 3.0 * ldexp(1.0, -16) + double(k) * ldexp(1.0, -24);
        }
        if (threadIdx.x == 0) *info = r;
    }
}

// ---- panel pipeline (host operands): B is sliced ahead of A -----------------------------------
// Block-wide statistics of one operand side from its row exponents e and relative sums of squares
// q: Inf/NaN flag, largest exponent E, largest q, s = sum 2^(2(e-E)) and nrm = sum 2^(2(e-E)) q.
struct SideStats {
    int bad, E;
    double Q, s, nrm;
};

__device__ SideStats side_stats(const int* __restrict__ e, const double* __restrict__ q, int64_t count, double* redd,
                                int* redi) {
    SideStats r;
    int bad = 0, E = -100000;
    long long Qb = 0;  // non-negative doubles: their bit patterns order like integers
    for (int64_t i = threadIdx.x; i < count; i += blockDim.x) {
        if (e[i] == kNonFinite) bad = 1;
        else {
            const long long qb = __double_as_longlong(q[i]);
            if (qb > 0) E = max(E, e[i]);
            Qb = max(Qb, qb);
        }
    }
    r.bad = block_max_int(bad, redi);
    r.E = block_max_int(E, redi);
    r.Q = __longlong_as_double(block_max_ll(Qb, reinterpret_cast<long long*>(redd)));
    double sv = 0, nv = 0;
    for (int64_t i = threadIdx.x; i < count; i += blockDim.x) {
        if (e[i] == kNonFinite || q[i] <= 0.0) continue;
        const double w = pow2i(2 * (e[i] - r.E));
        sv += w;
        nv += w * q[i];
    }
    r.s = block_sum(sv, redd);
    r.nrm = block_sum(nv, redd);
    return r;
}

// One operand side of a block of the host pipeline (a row panel of A or a column block of B): its
// norms and largest relative sum of squares (stored in both the A and the B fields), and the
// smallest beta with 2^(-beta-1) r <= target / 2: each side takes half of the bound for its own
// rounding, so the two sides are sliced independently.  `slices` = the planes the side is sliced
// into (the host's largest modulus count).
__global__ void __launch_bounds__(1024) split_side_kernel(const int* __restrict__ e, const double* __restrict__ q,
                                                          int64_t count, int64_t k, int planes, double target,
                                                          SplitInfo* out) {
    __shared__ double redd[32];
    __shared__ int redi[32];
    const SideStats t = side_stats(e, q, count, redd, redi);
    if (threadIdx.x < 32) {  // warp 0 plans; lane 0 writes
        SplitInfo r;
        r.nonfinite = t.bad;
        r.normA = r.normB = (t.nrm > 0) ? ldexp(sqrt(t.nrm), t.E) : 0.0;
        r.scaleA = r.scaleB = (t.s > 0) ? ldexp(sqrt(t.s), t.E) : 0.0;
        r.qmaxA = r.qmaxB = t.Q;
        const double rr = (t.nrm > 0) ? sqrt(double(k) * t.s / t.nrm) : 0.0;
        const int beta = min(55, warp_first_true(1, 54, [&](int b) { return pow2i(-b - 1) * rr <= 0.5 * target; }));
        r.beta = r.beta_b = beta;
        r.slices = planes;
        r.bound = 0.0;
        if (threadIdx.x == 0) *out = r;
    }
}

// A block (row panel i of A, column block j of B) from the two sides: the moduli that carry
// (2^beta_a sqrt(Q_A) + sqrt(k)/2)(2^beta_b sqrt(Q_B) + sqrt(k)/2) with the margin of
// split_info_kernel, and the block's bound 2^(-beta_a-1) r_A + 2^(-beta_b-1) r_B +
// 2^(-beta_a-beta_b-2) r_A r_B + 2^-52 relative to ||A_i|| ||B_j|| (infinite when even cap_planes
// moduli are too few).
__global__ void split_block_kernel(const SplitInfo* __restrict__ ia, const SplitInfo* __restrict__ ib, int64_t k,
                                   int cap_planes, SplitInfo* out) {
    if (threadIdx.x != 0) return;
    const SplitInfo A = *ia, B = *ib;
    SplitInfo r;
    r.nonfinite = A.nonfinite | B.nonfinite;
    r.normA = A.normA;
    r.scaleA = A.scaleA;
    r.qmaxA = A.qmaxA;
    r.normB = B.normB;
    r.scaleB = B.scaleB;
    r.qmaxB = B.qmaxB;
    const double rA = (A.normA > 0) ? sqrt(double(k)) * A.scaleA / A.normA : 0.0;
    const double rB = (B.normB > 0) ? sqrt(double(k)) * B.scaleB / B.normB : 0.0;
    const int ba = A.beta, bb = B.beta_b;
    const double hk = 0.5 * sqrt(double(k));
    const double need = 1.0875 + log2(ldexp(sqrt(A.qmaxA * (1.0 + 0x1p-10)), ba) + hk) +
                        log2(ldexp(sqrt(B.qmaxB * (1.0 + 0x1p-10)), bb) + hk);
    double have = 0.0;
    int N = 0;
    while (N < 2 || (N < cap_planes && have < need)) {
        have += c_mod_log2[N];
        ++N;
    }
    r.slices = N;
    r.beta = ba;
    r.beta_b = bb;
    r.bound = need > have ? __longlong_as_double(0x7ff0000000000000ll)
                          : pow2i(-ba - 1) * rA + pow2i(-bb - 1) * rB + pow2i(-ba - bb - 2) * rA * rB + pow2i(-52);
    *out = r;
}

// Summary of the blocks for the caller: the largest modulus count and bound (infos `stride` bytes
// apart).
// The level count of a launch that covers several blocks of one panel: the largest of its blocks'
// (each block's reconstruction reads its own count of levels; the launch reads only the count).
__global__ void split_max_slices_kernel(const uint8_t* __restrict__ infos, size_t stride, int count,
                                        SplitInfo* __restrict__ out) {
    if (threadIdx.x != 0) return;
    SplitInfo r = *reinterpret_cast<const SplitInfo*>(infos);
    for (int i = 1; i < count; ++i)
        r.slices = max(r.slices, reinterpret_cast<const SplitInfo*>(infos + size_t(i) * stride)->slices);
    *out = r;
}

__global__ void split_panels_summary_kernel(const uint8_t* __restrict__ infos, size_t stride, int count,
                                            SplitInfo* out) {
    if (threadIdx.x != 0) return;
    SplitInfo r = *reinterpret_cast<const SplitInfo*>(infos);
    for (int i = 1; i < count; ++i) {
        const SplitInfo& x = *reinterpret_cast<const SplitInfo*>(infos + size_t(i) * stride);
        r.slices = max(r.slices, x.slices);
        r.bound = fmax(r.bound, x.bound);
        r.nonfinite |= x.nonfinite;
    }
    *out = r;
}

// Digit planes: planes[a][r][p] (bf16, pitch kpad, plane stride rpad*kpad) for r < rpad, p < kpad;
// zeros outside the R x K operand.  Each block covers 32 rows x 64 k.
//
// Exact mode: for |a| < 2^e (e the row exponent) the fixed-point integer
// X = round(|a| * 2^(8S-1-e)) (round half up below the last digit) satisfies X <= 2^(8S-1); its
// balanced base-256 digits d_S..d_2 in [-128, 127] and the top digit d_1 in [0, 128] give
// |a| * 2^-e = sum_s d_s 2^(1-8s) + rho, |rho| <= 2^-8S.  Everything is integer arithmetic on the
// FP64 bit pattern (64-bit for S <= 8, 128-bit beyond); digits become BF16 bit patterns through an
// exact FP32 add.  Float modes: BF16 hi part and BF16 rounding of the remainder.
__device__ __forceinline__ uint16_t digit_bf16(int d) {
    // float(d) exactly via the 1.5*2^23 bias; |d| <= 128 has at most 8 significant bits, so the
    // upper half of the FP32 pattern is the BF16 pattern
    const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
    return uint16_t(__float_as_uint(f) >> 16);
}

// Fixed-point magnitude V = X + sum_{s<S-1} 128*256^s of one element: with it, the balanced digit of
// plane a >= 1 is byte (S-1-a) of V minus 128 and the top digit (plane 0) is V >> 8(S-1); adding the
// 128s once replaces the digit-by-digit carry chain.
template <typename U_t>
__device__ __forceinline__ U_t fixed_point_biased(unsigned long long bits, int e, int S) {
    const int eb = int((bits >> 52) & 0x7ff);
    const unsigned long long mant = bits & 0xfffffffffffffull;
    const unsigned long long M = eb ? (mant | (1ull << 52)) : mant;
    const int E = (eb ? eb : 1) - 1075;  // |a| = M * 2^E
    const int sh = E + 8 * S - 1 - e;
    U_t U;
    if (M == 0) U = 0;
    else if (sh >= 0) U = U_t(M) << sh;
    else if (sh > -64) U = U_t((M + (1ull << (-sh - 1))) >> (-sh));
    else U = 0;
    U_t B = 0;
    for (int s = 0; s < S - 1; ++s) B = (B << 8) | 0x80;
    return U + B;
}

template <typename U_t>
__device__ __forceinline__ void write_planes(const U_t (&V)[8], const bool (&neg)[8], int S, uint16_t* dst,
                                             int64_t pstride) {
    for (int a = 0; a < S; ++a) {
        const int sft = 8 * (S - 1 - a);
        __align__(16) uint16_t d[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            int v = int(uint32_t(V[q] >> sft) & (a == 0 ? 0x1ffu : 0xffu));
            if (a != 0) v -= 128;
            d[q] = digit_bf16(neg[q] ? -v : v);
        }
        *reinterpret_cast<uint4*>(dst + a * pstride) = *reinterpret_cast<const uint4*>(d);
    }
}

// |round(a * 2^sh)| for a finite double given by its bits (round half up); the result must fit in
// 56 bits, which the CRT plan guarantees (beta <= 55 and |a| < 2^e).
__device__ __forceinline__ unsigned long long int_magnitude(unsigned long long bits, int sh_total) {
    const int eb = int((bits >> 52) & 0x7ff);
    const unsigned long long mant = bits & 0xfffffffffffffull;
    const unsigned long long M = eb ? (mant | (1ull << 52)) : mant;
    const int sh = (eb ? eb : 1) - 1075 + sh_total;
    if (M == 0) return 0;
    if (sh >= 0) return M << sh;
    if (sh > -64) return (M + (1ull << (-sh - 1))) >> (-sh);
    return 0;
}

// x mod p for x < 2^32 and p <= 257 with inv = floor(2^32 / p): the quotient estimate is at most
// one short, so one conditional subtraction finishes the reduction.
__device__ __forceinline__ uint32_t mod_small(uint32_t x, uint32_t p, uint32_t inv) {
    const uint32_t q = uint32_t((uint64_t(x) * inv) >> 32);
    uint32_t r = x - q * p;
    return r >= p ? r - p : r;
}

// Planes of eight consecutive elements xv of one row (row exponent e, bad: the row holds Inf/NaN)
// at dst, plane stride pstride; sl = slices (digits) or moduli (CRT), bt = beta (CRT).
template <int mode>
__device__ __forceinline__ void slice_emit(const unsigned long long (&xv)[8], int sl, int bt, int e, bool bad,
                                           uint16_t* __restrict__ dst, int64_t pstride) {
    if (mode == kCrt) {
        const int N = sl, beta = bt;
        // U = |round(a 2^(beta-e))| < 2^56 in signed FP32 chunks (the sign of a applied to each)
        float w0[8], w1[8], w2[8], w3[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const unsigned long long bits = bad ? 0ull : xv[q];
            const unsigned long long U = int_magnitude(bits, beta - e);
            const float sg = (bits >> 63) ? -1.f : 1.f, off = (bits >> 63) ? 8388608.f : -8388608.f;
            w0[q] = fmaf(__uint_as_float(0x4B000000u | (uint32_t(U) & 0x3fffu)), sg, off);
            w1[q] = fmaf(__uint_as_float(0x4B000000u | (uint32_t(U >> 14) & 0x3fffu)), sg, off);
            w2[q] = fmaf(__uint_as_float(0x4B000000u | (uint32_t(U >> 28) & 0x3fffu)), sg, off);
            w3[q] = fmaf(__uint_as_float(0x4B000000u | uint32_t(U >> 42)), sg, off);
        }
        for (int t = 0; t < N; ++t) {
            const float pf = c_modf[t], inv = c_modf_inv[t];
            const float k1 = c_mod_k14[0][t], k2 = c_mod_k14[1][t], k3 = c_mod_k14[2][t];
            uint32_t fb[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float x = fmaf(w3[q], k3, fmaf(w2[q], k2, fmaf(w1[q], k1, w0[q])));
                const float qf = fmaf(x, inv, MAGIC) - MAGIC;
                // exact symmetric residue, an integer of at most 8 significant bits: its FP32
                // pattern's upper half is the BF16 pattern
                fb[q] = __float_as_uint(fmaf(-pf, qf, x));
            }
            uint4 w;
            w.x = __byte_perm(fb[0], fb[1], 0x7632);
            w.y = __byte_perm(fb[2], fb[3], 0x7632);
            w.z = __byte_perm(fb[4], fb[5], 0x7632);
            w.w = __byte_perm(fb[6], fb[7], 0x7632);
            *reinterpret_cast<uint4*>(dst + t * pstride) = w;
        }
    } else if (mode == kExact) {
        const int S = sl;
        bool neg[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) neg[q] = !bad && (xv[q] >> 63) != 0;
        if (S <= 8) {
            unsigned long long V[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) V[q] = fixed_point_biased<unsigned long long>(bad ? 0ull : xv[q], e, S);
            write_planes(V, neg, S, dst, pstride);
        } else {
            unsigned __int128 V[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) V[q] = fixed_point_biased<unsigned __int128>(bad ? 0ull : xv[q], e, S);
            write_planes(V, neg, S, dst, pstride);
        }
    } else {
        __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const double x = __longlong_as_double(static_cast<long long>(xv[q]));
            hi[q] = __float2bfloat16_rn(float(x));
            lo[q] = __float2bfloat16_rn(float(x - double(__bfloat162float(hi[q]))));
        }
        *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(hi);
        if (mode == kBf16x3) *reinterpret_cast<uint4*>(dst + pstride) = *reinterpret_cast<const uint4*>(lo);
    }
}

// Planes of 32 rows over TILE_KT k-tiles.  Thread (rr = t / 8, L = t % 8) handles elements
// 8L..8L+7 of row rr and writes 16 bytes per plane (a warp: four 128-byte row segments).  The tile
// buffer keeps rows of 528 bytes with 16-byte chunk c of a row stored at c ^ (c >> 3), so that the
// eight threads of a row read their chunks 4L + j from eight different bank groups.
template <int mode>
__device__ __forceinline__ void slice_rows(int which, const double* __restrict__ X, int64_t R, int64_t K, int64_t sr,
                                           int64_t sp, const int* __restrict__ rexp, const SplitInfo* __restrict__ info,
                                           __nv_bfloat16* __restrict__ planes, int64_t rpad, int64_t kpad, int by) {
    constexpr uint32_t ROWB = 528, BUF = 32 * ROWB;
    __shared__ __align__(16) unsigned char tbuf[2 * BUF];
    const int t = threadIdx.x, rr = t >> 3, L = t & 7;
    const int64_t r0 = int64_t(by) * 32, r = r0 + rr;
    const int64_t ntiles = kpad / 64;
    const int64_t tb = int64_t(blockIdx.x) * TILE_KT, te = min(ntiles, tb + TILE_KT);
    const uint32_t s0 = smem_u32(tbuf);
    auto off = [](int r_, int p_) {
        const uint32_t c = uint32_t(p_) >> 1;
        return uint32_t(r_) * ROWB + ((c ^ (c >> 3)) << 4) + ((uint32_t(p_) & 1u) << 3);
    };
    const int sl = (mode == kExact || mode == kCrt) ? info->slices : 0;
    const int bt = (mode == kCrt) ? (which ? info->beta_b : info->beta) : 0;
    const int e = (r < R) ? rexp[r] : 0;
    const bool bad = (mode == kExact || mode == kCrt) && e == kNonFinite;
    const int64_t pstride = rpad * kpad;
    const TileSrc ts = tile_src(X, sr, sp, r0);
    if (tb < te) tile_issue(s0, ts, X, R, K, r0, tb, off);
    for (int64_t it = tb; it < te; ++it) {
        const int b = int(it - tb) & 1;
        if (it + 1 < te) tile_issue(s0 + uint32_t(b ^ 1) * BUF, ts, X, R, K, r0, it + 1, off);
        else cp_async_commit();  // an empty group keeps the wait count uniform
        cp_async_wait1();
        __syncthreads();
        unsigned long long xv[8];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t c = uint32_t(4 * L + j);
            const uint4 v = *reinterpret_cast<const uint4*>(tbuf + b * BUF + rr * ROWB + ((c ^ (c >> 3)) << 4));
            xv[2 * j] = (unsigned long long)v.x | ((unsigned long long)v.y << 32);
            xv[2 * j + 1] = (unsigned long long)v.z | ((unsigned long long)v.w << 32);
        }
        if (r < rpad)
            slice_emit<mode>(xv, sl, bt, e, bad, reinterpret_cast<uint16_t*>(planes) + r * kpad + it * 64 + 8 * L,
                             pstride);
        __syncthreads();
    }
}

template <int MODE>
__global__ void __launch_bounds__(256, 3) slice_kernel(const OperandPair op, int64_t K, const SplitInfo* __restrict__ info,
                                                       int64_t kpad) {
    const int w = blockIdx.y < op.yb0 ? 0 : 1;
    const int by = w ? int(blockIdx.y - op.yb0) : int(blockIdx.y);
    slice_rows<MODE>(w, op.X[w], op.R[w], K, op.sr[w], op.sp[w], op.rexp[w], info, op.planes[w], op.rpad[w], kpad, by);
}

// ---- level / pair schedule ---------------------------------------------------------------------
__device__ __forceinline__ int num_levels(int mode, int S) { return (mode == kExact || mode == kCrt) ? S : 1; }
__device__ __forceinline__ int pairs_in_level(int mode, int L) {
    return mode == kExact ? L + 1 : (mode == kBf16x3 ? 3 : 1);
}
// (A plane, B plane) of pair `i` of level `L`.
__device__ __forceinline__ void pair_planes(int mode, int L, int i, int& a, int& b) {
    if (mode == kExact) { a = i; b = L - i; }
    else if (mode == kCrt) { a = L; b = L; }
    else if (mode == kBf16) { a = 0; b = 0; }
    else { a = (i == 2) ? 1 : 0; b = (i == 1) ? 1 : 0; }
}

struct TcParams {
    int mode;
    int m_tiles, n_tiles, nseg;
    int kb_per_seg;          // 64-wide k-blocks per segment
    int kb_total;            // 64-wide k-blocks in the padded K
    int64_t mpad, npad;      // padded rows of the A / B planes
    int32_t* levels;         // [nseg][nlevels][mpad][npad] int32 (float modes: fp32 bits)
    int max_levels;          // level dimension of `levels`
    int band = 8;            // m-tiles per band of the unit order (2..32 measured alike at 8192^3)
    int tn0 = 0;             // first n-tile of this launch (a product launched in column parts)
    const SplitInfo* info;
    int* status;
    uint64_t limit_ns;
    int inject_stall;
};

struct __align__(8) TcBarriers {
    uint64_t full[STAGES];
    uint64_t empty[STAGES];
    uint64_t acc_full[2];
    uint64_t acc_empty[2];
    uint64_t drain;
    uint32_t tmem_base;
};

// Residue (CRT) level tiles leave through a per-warp staging tile (32 rows x 128 bytes, 128-byte
// swizzle) and a TMA store: full-line writes instead of 32 rows per store instruction.
constexpr int OUT_WARP_BYTES = 32 * 128;
constexpr int OUT_BYTES = EPI_WARPS * OUT_WARP_BYTES;
constexpr size_t kTcSmem = size_t(STAGES) * STAGE_BYTES + OUT_BYTES + sizeof(TcBarriers) + 1024;

__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFFu) >> 4);     // start address
    d |= uint64_t(1) << 16;                      // leading byte offset (unused for 128B swizzle)
    d |= uint64_t(1024 >> 4) << 32;              // stride byte offset: 8 rows x 128 B
    d |= uint64_t(1) << 46;                      // descriptor version (tcgen05)
    d |= uint64_t(2) << 61;                      // 128-byte swizzle
    return d;
}

// kind::f16 instruction descriptor: BF16 A and B (K-major), FP32 D, M = 256 (a CTA pair), N = 256.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(TN >> 3) << 17) | (uint32_t(TMP >> 4) << 24);

// Work unit u -> (level, tile m, tile n, segment): one level (a modulus, or the slice pairs of a
// digit level) of one pair tile, the level varying slowest so that concurrent pairs share the
// operand planes of one level in L2, with 8 m-tiles per band.  Units of one level have equal
// lengths, and many small units keep the last wave short.
__device__ __forceinline__ void unit_coords(const TcParams& p, int u, int& tm, int& tn, int& seg, int& L) {
    const int per_level = p.m_tiles * p.n_tiles * p.nseg;
    L = u / per_level;
    u -= L * per_level;
    seg = u % p.nseg;
    const int t = u / p.nseg;
    const int band = p.band;
    const int per_band = band * p.n_tiles;
    const int b = t / per_band, r = t % per_band;
    const int rows_in_band = min(band, p.m_tiles - b * band);
    tm = b * band + r % rows_in_band;
    tn = p.tn0 + r / rows_in_band;
}

template <int MODE>
__global__ void __cluster_dims__(2, 1, 1) __maxnreg__(168)
tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               const __grid_constant__ CUtensorMap tmC, const TcParams p) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* out_stage = smem + STAGES * STAGE_BYTES;
    TcBarriers* bars = reinterpret_cast<TcBarriers*>(out_stage + OUT_BYTES);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // CTA pair: both CTAs walk the same units; the even CTA issues the pair MMAs, each CTA loads its
    // 128 rows of A and its half of B and drains its own 128 TMEM lanes
    const uint32_t rank = cluster_ctarank();
    const bool leader = rank == 0;
    const int pair = int(blockIdx.x >> 1), npairs = int(gridDim.x >> 1);

    // the epilogue's arithmetic is fixed at compile time (exact integer sums or FP32 tiles); the
    // digit and residue schedules share the exact instantiation and differ only in the plane pairs
    constexpr int emode = MODE;
    const int mode = (MODE == kExact) ? p.mode : MODE;
    const int S = (mode == kExact || mode == kCrt) ? p.info->slices : 1;
    const int nlev = num_levels(mode, S);
    const int units = p.m_tiles * p.n_tiles * p.nseg * nlev;

    if (threadIdx.x == 0) {
        tma_prefetch_desc(&tmA);
        tma_prefetch_desc(&tmB);
        if (p.mode == kCrt) tma_prefetch_desc(&tmC);
        // full: the even CTA's arm plus both CTAs' bytes; empty / acc_full: one pair-MMA commit
        // (multicast to both CTAs); acc_empty (even CTA): every epilogue warp of both CTAs
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(smem_u32(&bars->full[s]), 1);
            mbar_init(smem_u32(&bars->empty[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&bars->acc_full[b]), 1);
            mbar_init(smem_u32(&bars->acc_empty[b]), 2 * EPI_WARPS);
        }
        mbar_init(smem_u32(&bars->drain), 1);
        fence_mbar_init();
    }
    if (warp == 1) {
        __syncwarp();
        tmem_alloc_pair(smem_u32(&bars->tmem_base), 512);
        tmem_relinquish_pair();
    }
    tc_fence_before();
    // barriers of both CTAs initialised before any cross-CTA arrival or copy
    cluster_sync();
    tc_fence_after();
    const uint32_t tmem = bars->tmem_base;

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0 && !p.inject_stall) {
            uint32_t it = 0;
            bool ok = true;
            for (int u = pair; u < units && ok; u += npairs) {
                int tm, tn, seg, Lu;
                unit_coords(p, u, tm, tn, seg, Lu);
                const int kb0 = seg * p.kb_per_seg;
                const int kbn = min(p.kb_per_seg, p.kb_total - kb0);
                {
                    const int L = Lu;
                    const int np = pairs_in_level(mode, L);
                    for (int kb = 0; kb < kbn && ok; ++kb) {
                        for (int i = 0; i < np; ++i, ++it) {
                            const int s = it % STAGES;
                            if (it >= STAGES &&
                                !mbar_wait(smem_u32(&bars->empty[s]), ((it / STAGES) - 1) & 1, p.status,
                                           kDevTimeoutEmpty, p.limit_ns)) {
                                ok = false;
                                break;
                            }
                            int a, b;
                            pair_planes(mode, L, i, a, b);
                            // both CTAs' bytes complete on the even CTA's full barrier, armed there
                            // for the two halves
                            const uint32_t full_local = smem_u32(&bars->full[s]);
                            if (leader) mbar_arrive_expect_tx(full_local, 2 * STAGE_BYTES);
                            const uint32_t full = mapa_shared(full_local, 0);
                            const uint32_t dst = smem_u32(smem + s * STAGE_BYTES);
                            const int32_t kx = (kb0 + kb) * TK;
                            tma_load_2d_pair(dst, &tmA, kx, int32_t(a * p.mpad + int64_t(tm) * TMP + rank * TM), full);
                            tma_load_2d_pair(dst + A_BYTES, &tmB, kx,
                                             int32_t(b * p.npad + int64_t(tn) * TN + rank * TNH), full);
                        }
                    }
                }
            }
            // drain: the last use of every stage must have landed before the pair exits (the even
            // CTA's full barriers count the bytes of both)
            if (leader) {
                const uint32_t first = it > STAGES ? it - STAGES : 0;
                for (uint32_t j = first; j < it; ++j)
                    mbar_wait_drain(smem_u32(&bars->full[j % STAGES]), (j / STAGES) & 1, p.limit_ns);
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer (even CTA of the pair) ----------------
        if (lane == 0 && leader) {
            uint32_t it = 0, grp = 0;
            bool ok = true, issued_any = false;
            for (int u = pair; u < units && ok; u += npairs) {
                int tm, tn, seg, Lu;
                unit_coords(p, u, tm, tn, seg, Lu);
                const int kb0 = seg * p.kb_per_seg;
                const int kbn = min(p.kb_per_seg, p.kb_total - kb0);
                {
                    const int L = Lu;
                    const int np = pairs_in_level(mode, L);
                    const int items = np * kbn;
                    const int gsize = (mode == kExact || mode == kCrt) ? GROUP_ITEMS : items;
                    for (int g0 = 0; g0 < items && ok; g0 += gsize, ++grp) {
                        const int buf = grp & 1;
                        if (grp >= 2 && !mbar_wait(smem_u32(&bars->acc_empty[buf]), ((grp >> 1) - 1) & 1, p.status,
                                                   kDevTimeoutAccEmpty, p.limit_ns)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t dcol = tmem + uint32_t(buf * TN);
                        const int gend = min(items, g0 + gsize);
                        for (int x = g0; x < gend; ++x, ++it) {
                            const int s = it % STAGES;
                            if (!mbar_wait(smem_u32(&bars->full[s]), (it / STAGES) & 1, p.status, kDevTimeoutFull,
                                           p.limit_ns)) {
                                ok = false;
                                break;
                            }
                            tc_fence_after();
                            const uint32_t a_addr = smem_u32(smem + s * STAGE_BYTES);
                            const uint64_t adesc = sw128_desc(a_addr);
                            const uint64_t bdesc = sw128_desc(a_addr + A_BYTES);
#pragma unroll
                            for (int j = 0; j < TK / 16; ++j)
                                tc_mma_f16_pair(dcol, adesc + uint64_t(2 * j), bdesc + uint64_t(2 * j), kIdesc,
                                                (x == g0 && j == 0) ? 0u : 1u);
                            tc_commit_pair_mc(smem_u32(&bars->empty[s]), 0x3);
                            issued_any = true;
                        }
                        if (!ok) break;
                        tc_commit_pair_mc(smem_u32(&bars->acc_full[buf]), 0x3);
                    }
                }
            }
            // drain: every issued MMA completes before TMEM is released
            if (issued_any) {
                tc_commit_pair_mc(smem_u32(&bars->drain), 0x1);
                mbar_wait_drain(smem_u32(&bars->drain), 0, p.limit_ns);
            }
        }
    } else {
        // ---------------- epilogue ----------------
        const int q = warp & 3;                 // TMEM lane quarter of this warp
        const int h = (warp - 2) >> 2;          // column half: 0 or 1
        const uint32_t lane_base = uint32_t(32 * q) << 16;
        uint32_t grp = 0;
        bool ok = true;
        // the even CTA's accumulator-empty barriers (the MMA issuer waits for both CTAs' drains)
        const uint32_t acc_empty0 = mapa_shared(smem_u32(&bars->acc_empty[0]), 0);
        const uint32_t acc_empty1 = mapa_shared(smem_u32(&bars->acc_empty[1]), 0);
        for (int u = pair; u < units && ok; u += npairs) {
            int tm, tn, seg, Lu;
            unit_coords(p, u, tm, tn, seg, Lu);
            const int kb0 = seg * p.kb_per_seg;
            const int kbn = min(p.kb_per_seg, p.kb_total - kb0);
            const int64_t row = int64_t(tm) * TMP + int64_t(rank) * TM + 32 * q + lane;
            {
                const int L = Lu;
                const int np = pairs_in_level(mode, L);
                const int items = np * kbn;
                const int gsize = (mode == kExact || mode == kCrt) ? GROUP_ITEMS : items;
                uint32_t acc[128];
#pragma unroll
                for (int c = 0; c < 128; ++c) acc[c] = 0u;
                for (int g0 = 0; g0 < items; g0 += gsize, ++grp) {
                    const int buf = grp & 1;
                    if (!mbar_wait(smem_u32(&bars->acc_full[buf]), (grp >> 1) & 1, p.status, kDevTimeoutMma,
                                   p.limit_ns)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t base = tmem + lane_base + uint32_t(buf * TN + h * 128);
#pragma unroll
                    for (int c4 = 0; c4 < 8; ++c4) {
                        uint32_t v[16];
                        tmem_ld_32x32b_x16(base + uint32_t(c4 * 16), v);
                        tc_wait_ld();
                        if (emode == kExact) {
                            // the group sum is an integer of at most 2^24 in magnitude: exact in
                            // FP32 and exactly converted (adding 1.5 * 2^23 would be exact only
                            // below 2^22, i.e. for groups of 256 products)
#pragma unroll
                            for (int c = 0; c < 16; ++c)
                                acc[c4 * 16 + c] += uint32_t(__float2int_rn(__uint_as_float(v[c])));
                        } else {
#pragma unroll
                            for (int c = 0; c < 16; ++c) acc[c4 * 16 + c] = v[c];
                        }
                    }
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive_cluster(buf ? acc_empty1 : acc_empty0);
                }
                if (!ok) break;
                // level sums -> global level plane (row-major, pitch npad); in the residue (CRT)
                // schedule the sum is reduced modulo the level's modulus and stored as 16 bits
                const int64_t plane_off = ((int64_t(seg) * p.max_levels + L) * p.mpad + row) * p.npad +
                                          int64_t(tn) * TN + h * 128;
                if (emode == kExact && mode == kCrt) {
                    // residues in [0, p) as 16-bit values; two 64-column halves per warp go out
                    // through the warp's staging tile (row = lane, 16-byte chunk j of a row at
                    // j ^ (lane % 8): the TMA 128-byte swizzle) and a TMA store
                    const uint32_t pm = c_mod[L], inv = c_mod_inv32[L];
                    uint8_t* stg = out_stage + (warp - 2) * OUT_WARP_BYTES;
                    const int32_t ytile = int32_t((int64_t(seg) * p.max_levels + L) * p.mpad + int64_t(tm) * TMP +
                                                  int64_t(rank) * TM + 32 * q);
#pragma unroll
                    for (int ch = 0; ch < 2; ++ch) {
                        if (lane == 0) bulk_wait_read0();  // the previous store has read the tile
                        __syncwarp();
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int c = ch * 64 + j * 8;
                            __align__(16) uint16_t rr[8];
#pragma unroll
                            for (int e = 0; e < 8; ++e) {
                                const int32_t t = int32_t(acc[c + e]);
                                const uint32_t mag = t < 0 ? uint32_t(-int64_t(t)) : uint32_t(t);
                                uint32_t rsd = mod_small(mag, pm, inv);
                                if (t < 0 && rsd) rsd = pm - rsd;
                                rr[e] = uint16_t(rsd);
                            }
                            *reinterpret_cast<uint4*>(stg + lane * 128 + ((j ^ (lane & 7)) << 4)) =
                                *reinterpret_cast<const uint4*>(rr);
                        }
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0) {
                            tma_store_2d(&tmC, int32_t(tn * TN + h * 128 + ch * 64), ytile, smem_u32(stg));
                            bulk_commit();
                        }
                    }
                } else {
                    int32_t* dst = p.levels + plane_off;
#pragma unroll
                    for (int c = 0; c < 128; c += 4) {
                        int4 w;
                        w.x = int32_t(acc[c + 0]);
                        w.y = int32_t(acc[c + 1]);
                        w.z = int32_t(acc[c + 2]);
                        w.w = int32_t(acc[c + 3]);
                        *reinterpret_cast<int4*>(dst + c) = w;
                    }
                }
            }
        }
    }

    // the residue stores of this thread have completed
    if (warp >= 2 && lane == 0) bulk_wait0();
    tc_fence_before();
    // neither CTA leaves while the pair MMAs, copies or arrivals may still touch its memory
    cluster_sync();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        tmem_dealloc_pair(tmem, 512);
    }
}

// Round the signed 128-bit integer W to the nearest double and multiply by 2^x, with integer
// operations only whenever the result is a normal number (the usual case); sub- or overflowing
// results take the FP64 ldexp path.
__device__ __forceinline__ double int128_to_double_scaled(__int128 W, int x) {
    if (W == 0) return 0.0;
    const bool neg = W < 0;
    const unsigned __int128 U = neg ? (unsigned __int128)(-W) : (unsigned __int128)W;
    const unsigned long long hi = (unsigned long long)(U >> 64), lo = (unsigned long long)U;
    const int nbits = hi ? 128 - __clzll((long long)hi) : 64 - __clzll((long long)lo);
    unsigned long long mant;
    int shift = 0;
    if (nbits <= 53) {
        mant = lo << (53 - nbits);
        shift = nbits - 53;
    } else {
        shift = nbits - 53;
        const unsigned __int128 m = U >> shift;
        const unsigned __int128 rem = U - (m << shift);
        const unsigned __int128 half = (unsigned __int128)1 << (shift - 1);
        mant = (unsigned long long)m;
        if (rem > half || (rem == half && (mant & 1))) ++mant;
        if (mant == (1ull << 53)) {
            mant >>= 1;
            ++shift;
        }
    }
    // value = mant * 2^(shift + x), mant in [2^52, 2^53)
    const int be = 52 + shift + x + 1023;
    if (be > 0 && be < 2047) {
        const unsigned long long bits =
            (neg ? (1ull << 63) : 0ull) | ((unsigned long long)be << 52) | (mant & 0xfffffffffffffull);
        return __longlong_as_double((long long)bits);
    }
    const double v = ldexp(double(mant), shift + x);
    return neg ? -v : v;
}

// The same for W given as two's-complement 64-bit halves, on 64-bit integer operations: normalize
// the magnitude so that its top bit is bit 127, keep 53 bits, round to nearest even, and write the
// exponent field by adding (be - 1) << 52 to the 53-bit mantissa (a rounding carry into 2^53 then
// moves the exponent up by itself).
__device__ __forceinline__ double i128_to_double_scaled(unsigned long long hi, unsigned long long lo, int x) {
    const bool neg = (long long)hi < 0;
    if (neg) {
        lo = ~lo + 1ull;
        hi = ~hi + (lo == 0ull ? 1ull : 0ull);
    }
    if ((hi | lo) == 0ull) return 0.0;
    int lz;
    unsigned long long t, sticky;
    if (hi) {
        lz = __clzll((long long)hi);
        t = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;
        sticky = lo << lz;
    } else {
        const int l2 = __clzll((long long)lo);
        lz = 64 + l2;
        t = lo << l2;
        sticky = 0ull;
    }
    // |W| = (t + sticky 2^-64) 2^(64 - lz); mantissa bits 63..11 of t, bit 10 the rounding bit
    unsigned long long mant = t >> 11;
    if ((t & 0x400ull) && ((t & 0x3ffull) || sticky || (mant & 1ull))) ++mant;
    // |W| 2^x ~= mant 2^(75 - lz + x), leading bit 2^(127 - lz + x)
    const int be = 127 - lz + x + 1023;
    if (be >= 1 && be + int(mant >> 53) <= 2046) {
        const unsigned long long bits = ((unsigned long long)(be - 1) << 52) + mant;
        return __longlong_as_double((long long)(bits | (neg ? (1ull << 63) : 0ull)));
    }
    const double v = ldexp(double(mant), 75 - lz + x);
    return neg ? -v : v;
}

// C = alpha * 2^(e_i + f_j) * sum_L 2^(-14-8L) * sum_seg T[seg][L] + beta * C   (exact mode)
// C = alpha * sum_seg P[seg] + beta * C                                         (float modes)
// Exact mode forms W = sum_L T_L * 2^(8(S-1-L)) exactly in 128-bit integers, so the only roundings
// are the conversion of W to double and the alpha/beta update (skipped when alpha == 1, beta == 0).
// Grid: x over groups of 4 consecutive columns (one 16-byte load per level plane), y over rows.
constexpr int COMBINE_COLS = 4;

// Residue (CRT) reconstruction of CC consecutive outputs of one row for N moduli, all constants
// compile-time (crt_tables.h).  u_s = (c_p A_s + c_q B_s) mod P_s per super modulus (< 2^26 before
// the reduction), W = sum_s u_s (P / P_s) in signed 64-bit sums of 32-bit limb products (each below
// 2^48, at most 8 per limb), and the symmetric residue W - round(W / P) P with the quotient from an
// FP32 estimate of sum_s u_s / P_s: the product of the scaled integers has |value| < P / 2.125, so
// W / P lies at least 0.029 from a half integer and an estimate off by less than 0.01 picks the
// right multiple of P.
// Residues of CC consecutive columns (CC / 2 words of two 16-bit residues).
template <int CC>
__device__ __forceinline__ void load_res(const uint16_t* __restrict__ p, uint32_t (&w)[CC / 2]) {
    if constexpr (CC == 4) {
        const uint2 v = *reinterpret_cast<const uint2*>(p);
        w[0] = v.x;
        w[1] = v.y;
    } else {
        w[0] = *reinterpret_cast<const uint32_t*>(p);
    }
}

template <int N, int CC>
__device__ __forceinline__ void crt_cols(const uint16_t* __restrict__ res16, int64_t plane, int64_t off, int nseg,
                                         int max_levels, int scale, int ei, const int (&fj)[CC], double (&v)[CC]) {
    constexpr CrtTable T = kCrtTables[N - 2];
    constexpr int NS = T.nsup, LB = T.limbs;
    uint32_t rq[2 * NS][CC / 2];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int t = h ? T.sup[s].ib : T.sup[s].ia;
            if (t < 0) continue;
            load_res<CC>(res16 + int64_t(t) * plane + off, rq[2 * s + h]);
            for (int g = 1; g < nseg; ++g) {
                // segment residues add up: each < p, words hold two 16-bit residues and no carry
                // crosses for nseg < 256
                uint32_t b[CC / 2];
                load_res<CC>(res16 + (int64_t(g) * max_levels + t) * plane + off, b);
#pragma unroll
                for (int w = 0; w < CC / 2; ++w) rq[2 * s + h][w] += b[w];
            }
        }
    }
    long long acc[CC][4];
    float fq[CC];
#pragma unroll
    for (int cc = 0; cc < CC; ++cc) {
        fq[cc] = -T.fbias;
#pragma unroll
        for (int l = 0; l < 4; ++l) acc[cc][l] = 0;
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        constexpr uint32_t one = 1u;
        const CrtSuper& S = T.sup[s];
#pragma unroll
        for (int cc = 0; cc < CC; ++cc) {
            const uint32_t ha = rq[2 * s][cc >> 1];
            uint32_t cp = (cc & 1) ? (ha >> 16) : (ha & 0xffffu);
            if (nseg > 1) cp = mod_small(cp, S.p, S.pinv32);
            uint32_t x = cp * S.A;
            if (S.q > one) {
                const uint32_t hb = rq[2 * s + 1][cc >> 1];
                uint32_t cq = (cc & 1) ? (hb >> 16) : (hb & 0xffffu);
                if (nseg > 1) cq = mod_small(cq, S.q, S.qinv32);
                x += cq * S.B;
            }
            uint32_t u = x - __umulhi(x, S.Psinv32) * S.Ps;
            u = min(u, u - S.Ps);
            fq[cc] = fmaf(__uint_as_float(0x4B000000u | u), S.finv, fq[cc]);
#pragma unroll
            for (int l = 0; l < LB; ++l)
                if (S.M[l]) acc[cc][l] += (unsigned long long)u * S.M[l];
        }
    }
#pragma unroll
    for (int cc = 0; cc < CC; ++cc) {
        const uint32_t qm = __float_as_uint(fq[cc] + MAGIC) - MAGIC_BITS;
        long long a[4];
#pragma unroll
        for (int l = 0; l < LB; ++l) {
            a[l] = acc[cc][l] - (long long)((unsigned long long)qm * T.P[l]);
            if (l > 0) a[l] += a[l - 1] >> 32;
        }
        unsigned long long hi, lo;
        if (LB == 1) {
            lo = (unsigned long long)a[0];
            hi = (unsigned long long)(a[0] >> 63);
        } else {
            lo = ((unsigned long long)a[1] << 32) | uint32_t(a[0]);
            if (LB == 2) hi = (unsigned long long)(a[1] >> 32);
            else if (LB == 3) hi = (unsigned long long)a[2];
            else hi = ((unsigned long long)a[LB - 1] << 32) | uint32_t(a[LB - 2]);
        }
        if (ei == kNonFinite || fj[cc] == kNonFinite) v[cc] = __longlong_as_double(0x7ff8000000000000ll);
        else v[cc] = i128_to_double_scaled(hi, lo, ei + fj[cc] - scale);
    }
}

// Residue (CRT) reconstruction and epilogue, CC columns a thread (row i on blockIdx.y, striding by
// gridDim.y; the column exponents are read once): C = alpha * W 2^(e_i + f_j - scale) + beta * C.
// Measured at 2048^3 and 8192^3: 4 columns beat 2 (latency-bound, less work in flight) and 8
// (fewer resident warps); reading the column exponents once took 4 % off the 8192^3 time.
template <int CC>
__global__ void __launch_bounds__(128, 8) crt_combine_kernel(const uint16_t* __restrict__ res16, int nseg,
                                                             int max_levels, int64_t mpad, int64_t npad,
                                                             const SplitInfo* __restrict__ info,
                                                             const int* __restrict__ eA, const int* __restrict__ eB,
                                                             int64_t m, int64_t n, double alpha, double beta,
                                                             double* __restrict__ C, int64_t ldc) {
    const int64_t j0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) * CC;
    if (j0 >= n) return;
    const int64_t plane = mpad * npad;
    const int scale = info->beta + info->beta_b;
    const int N = info->slices;
    int fj[CC];
#pragma unroll
    for (int cc = 0; cc < CC; ++cc) fj[cc] = (j0 + cc < n) ? eB[j0 + cc] : 0;
    const bool plain = (alpha == 1.0 && beta == 0.0);
    for (int64_t i = blockIdx.y; i < m; i += gridDim.y) {
        const int64_t off = i * npad + j0;
        const int ei = eA[i];
        double v[CC];
        switch (N) {
#define GB_CRT_CASE(NN) \
    case NN: crt_cols<NN, CC>(res16, plane, off, nseg, max_levels, scale, ei, fj, v); break;
            GB_CRT_CASE(2) GB_CRT_CASE(3) GB_CRT_CASE(4) GB_CRT_CASE(5) GB_CRT_CASE(6) GB_CRT_CASE(7)
            GB_CRT_CASE(8) GB_CRT_CASE(9) GB_CRT_CASE(10) GB_CRT_CASE(11) GB_CRT_CASE(12) GB_CRT_CASE(13)
            GB_CRT_CASE(14) GB_CRT_CASE(15)
#undef GB_CRT_CASE
            default:
#pragma unroll
                for (int cc = 0; cc < CC; ++cc) v[cc] = __longlong_as_double(0x7ff8000000000000ll);
        }
        double* crow = C + i * ldc;
#pragma unroll
        for (int cc = 0; cc < CC; ++cc) {
            const int64_t j = j0 + cc;
            if (j >= n) break;
            if (plain) crow[j] = v[cc];
            else {
                const double x = alpha * v[cc];
                crow[j] = (beta == 0.0) ? x : fma(beta, crow[j], x);
            }
        }
    }
}

constexpr int CRT_COMBINE_COLS = 4;

__global__ void __launch_bounds__(128, 8) combine_kernel(const int32_t* __restrict__ levels, int nseg, int max_levels, int64_t mpad,
                               int64_t npad, int mode, const SplitInfo* __restrict__ info,
                               const int* __restrict__ eA, const int* __restrict__ eB, int64_t m, int64_t n,
                               double alpha, double beta, double* __restrict__ C, int64_t ldc) {
    const int64_t j0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) * COMBINE_COLS;
    if (j0 >= n) return;
    const int64_t plane = mpad * npad;
    for (int64_t i = blockIdx.y; i < m; i += gridDim.y) {
    const int64_t off = i * npad + j0;
    double v[COMBINE_COLS];
    if (mode == kExact) {
        const int S = info->slices;
        const int ei = eA[i];
        __int128 W[COMBINE_COLS] = {0, 0, 0, 0};
        for (int L = 0; L < S; ++L) {
            long long t[COMBINE_COLS] = {0, 0, 0, 0};
            for (int g = 0; g < nseg; ++g) {
                const int4 q = *reinterpret_cast<const int4*>(levels + (int64_t(g) * max_levels + L) * plane + off);
                t[0] += q.x; t[1] += q.y; t[2] += q.z; t[3] += q.w;
            }
#pragma unroll
            for (int c = 0; c < COMBINE_COLS; ++c) W[c] = (W[c] << 8) + t[c];
        }
#pragma unroll
        for (int c = 0; c < COMBINE_COLS; ++c) {
            const int64_t j = j0 + c;
            const int fj = (j < n) ? eB[j] : 0;
            if (ei == kNonFinite || fj == kNonFinite)
                v[c] = __longlong_as_double(0x7ff8000000000000ll);  // NaN: the inputs were not finite
            else
                v[c] = int128_to_double_scaled(W[c], ei + fj - 14 - 8 * (S - 1));
        }
    } else {
        float acc[COMBINE_COLS] = {0.f, 0.f, 0.f, 0.f};
        double dacc[COMBINE_COLS] = {0.0, 0.0, 0.0, 0.0};
        for (int g = 0; g < nseg; ++g) {
            const int4 q = *reinterpret_cast<const int4*>(levels + int64_t(g) * max_levels * plane + off);
            acc[0] = __int_as_float(q.x); acc[1] = __int_as_float(q.y);
            acc[2] = __int_as_float(q.z); acc[3] = __int_as_float(q.w);
#pragma unroll
            for (int c = 0; c < COMBINE_COLS; ++c) dacc[c] += double(acc[c]);
        }
#pragma unroll
        for (int c = 0; c < COMBINE_COLS; ++c) v[c] = dacc[c];
    }
    const bool plain = (alpha == 1.0 && beta == 0.0);
    double* crow = C + i * ldc;
#pragma unroll
    for (int c = 0; c < COMBINE_COLS; ++c) {
        const int64_t j = j0 + c;
        if (j >= n) break;
        if (plain) crow[j] = v[c];
        else {
            const double x = alpha * v[c];
            crow[j] = (beta == 0.0) ? x : fma(beta, crow[j], x);
        }
    }
    }
}

int64_t round_up(int64_t x, int64_t q) { return (x + q - 1) / q * q; }

}  // namespace

bool split_read_info(const void* info_dev, int* slices, double* bound) {
    SplitInfo h;
    if (cudaMemcpy(&h, info_dev, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return false;
    *slices = h.slices;
    *bound = h.bound;
    return true;
}

size_t split_info_bytes() { return sizeof(SplitInfo); }

void split_decode_info(const void* info_host, int* slices, double* bound) {
    SplitInfo h;
    std::memcpy(&h, info_host, sizeof(h));
    *slices = h.slices;
    *bound = h.bound;
}

namespace {
// dst (rows x cols, pitch ld_d) = src (pitch ld_s), element-wise conversion: rows on blockIdx.y
// (striding by gridDim.y), columns on threads.
template <typename S, typename D>
__global__ void convert_kernel(int64_t rows, int64_t cols, const S* __restrict__ src, int64_t ld_s, D* __restrict__ dst,
                               int64_t ld_d) {
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y)
        for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < cols; c += int64_t(gridDim.x) * blockDim.x)
            dst[r * ld_d + c] = D(src[r * ld_s + c]);
}

template <typename S, typename D>
cudaError_t launch_convert(int64_t rows, int64_t cols, const S* src, int64_t ld_s, D* dst, int64_t ld_d,
                           cudaStream_t st) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    const int64_t x = std::max<int64_t>(1, std::min<int64_t>((cols + 255) / 256, 64));
    const int64_t y = std::max<int64_t>(1, std::min<int64_t>(rows, int64_t(runtime().num_sms) * 16 / x));
    convert_kernel<S, D><<<dim3(unsigned(x), unsigned(y)), 256, 0, st>>>(rows, cols, src, ld_s, dst, ld_d);
    count_launches(1);
    return cudaGetLastError();
}
}  // namespace

// ---- host orchestration ------------------------------------------------------------------------
namespace {

int native_product(const Gemm& g, const LaunchCtl& ctl, cudaStream_t st, Workspace& ws, SplitResult* out,
                   std::string* err) {
    Runtime& r = runtime();
    const int splits = g.k > 0 ? native_choose_splits(g.m, g.n, g.k, 8, r.num_sms) : 1;
    double* w = nullptr;
    if (splits > 1) {
        w = static_cast<double*>(ws.get(kSlotWork, size_t(splits) * size_t(g.m) * size_t(g.n) * 8, err));
        if (!w) return GB300_ERR_NO_MEMORY;
    }
    cudaError_t e = native_gemm<double>(g, splits, w, ctl, st, err);
    if (e != cudaSuccess) {
        if (err && err->empty()) *err = cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    out->method_used = GB300_METHOD_NATIVE;
    out->slices = 0;
    out->error_bound = double(g.k) * 0x1p-53;
    out->info_dev = nullptr;
    return GB300_OK;
}

// The AUTO policy: the split form costs about S(S+1)/2 BF16 products plus operand passes; below a
// few million multiply-adds, or for very short k, the native kernel's single pass wins.
bool auto_uses_native(const Gemm& g) {
    const double work = double(g.m) * double(g.n) * double(g.k);
    return work < 256.0 * 256.0 * 256.0 || g.k < 64;
}

// Moduli the CRT form needs in the worst case for inner dimension k and a normwise target (<= 0:
// k*2^-53): with |a_i| < 2^e_i, ||A||_F >= ||2^e||/2, so rA, rB <= 2 sqrt(k).  Returns a count above
// MAX_MODULI when the target is out of reach (the digit form is used then).
int crt_worst_case_moduli(int64_t k, double target) {
    if (target <= 0) target = double(k) * 0x1p-53;
    const double r = 2.0 * std::sqrt(double(std::max<int64_t>(k, 1)));
    int beta = 1;
    while (beta <= 55 && (std::ldexp(1.0, -beta - 1) * 2 * r + std::ldexp(1.0, -2 * beta - 2) * r * r + 0x1p-52) > target)
        ++beta;
    if (beta > 55) return MAX_MODULI + 1;
    int kbits = 0;
    while ((int64_t(1) << kbits) < std::max<int64_t>(k, 2)) ++kbits;
    const double need = 2.0 + kbits + 2.0 * beta;
    double have = 0;
    int N = 0;
    while (N < MAX_MODULI && have < need) have += kModLog2[N++];
    return have < need ? MAX_MODULI + 1 : N;
}

struct SplitGeometry {
    int mode, m_tiles, n_tiles, nseg, kb_total, max_planes, max_levels;
    int64_t mpad, npad, kpad, kseg;
};

SplitGeometry split_geometry(const Gemm& g, const SplitRequest& req, int num_sms) {
    SplitGeometry G;
    G.mode = kExact;
    if (req.method == GB300_METHOD_BF16) G.mode = kBf16;
    else if (req.method == GB300_METHOD_BF16X3) G.mode = kBf16x3;
    else if (req.method == GB300_METHOD_SPLIT_CRT) G.mode = kCrt;
    else if ((req.method == GB300_METHOD_SPLIT || req.method == GB300_METHOD_AUTO) && req.slices <= 0 &&
             crt_worst_case_moduli(g.k, req.target_error) <= MAX_MODULI)
        G.mode = kCrt;
    G.m_tiles = int((g.m + TMP - 1) / TMP);  // tiles of a CTA pair (256 rows)
    G.n_tiles = int((g.n + TN - 1) / TN);
    G.mpad = int64_t(G.m_tiles) * TMP;
    G.npad = int64_t(G.n_tiles) * TN;
    G.kpad = round_up(g.k, TK);
    G.kb_total = int(G.kpad / TK);
    if (G.mode == kCrt)
        // at least two moduli (the reconstruction tables start at N = 2)
        G.max_planes = req.slices > 0 ? std::max(2, std::min(req.slices, MAX_MODULI))
                                      : std::max(2, std::min(MAX_MODULI, crt_worst_case_moduli(g.k, req.target_error)));
    else
        G.max_planes = (G.mode == kExact) ? (req.slices > 0 ? std::min(req.slices, MAX_SLICES) : MAX_SLICES)
                                          : (G.mode == kBf16 ? 1 : 2);
    G.max_levels = (G.mode == kExact || G.mode == kCrt) ? G.max_planes : 1;
    // k-segments: exactness (int32 level sums) and parallelism for few output tiles; decided from the
    // device's SM count only, so a capped grid computes the same segments (and the same result)
    int64_t kseg = G.kpad;
    if (G.mode == kExact || G.mode == kCrt) {
        // n_L * Kseg products of at most 2^14 each must stay below 2^31 (one pair per level in
        // CRT mode)
        const int64_t cap = (int64_t(511) / (G.mode == kCrt ? 1 : G.max_planes)) * KSEG_UNIT;
        kseg = std::min(kseg, std::max<int64_t>(cap, KSEG_UNIT));
    }
    // Split k only when at most half the CTA pairs would have a tile, and into as many segments as
    // still fit one wave of pairs.  With more tiles a split cannot raise the occupancy (the units
    // spill into a second, partial wave) and it multiplies the residue planes the reconstruction
    // reads; at 64 tiles on 76 pairs two segments made a 512 x 8192 x 512 product 1.6 times slower.
    // A segment keeps at least one TMEM drain group of k (1024): a unit of 256 k has about 1.3 us of
    // products against about 3 us of epilogue (drain, modular reduction, residue store), and every
    // extra segment adds residue planes for the reconstruction; 1024^3 split into four 256-k
    // segments took 59 us in the tensor-core kernel and 55 us in the reconstruction.
    const int tiles = G.m_tiles * G.n_tiles, pairs = std::max(1, num_sms / 2);
    if (2 * tiles <= pairs) {
        const int64_t want = pairs / tiles;
        constexpr int64_t kMinSeg = int64_t(GROUP_ITEMS) * TK;
        kseg = std::min(kseg, std::max<int64_t>(kMinSeg, round_up((G.kpad + want - 1) / want, KSEG_UNIT)));
    }
    // equal segments: persistent CTAs take units in a fixed stride, so unequal segments would give
    // some CTAs only the long ones
    const int64_t nseg = (G.kpad + kseg - 1) / kseg;
    G.kseg = round_up((G.kpad + nseg - 1) / nseg, TK);
    G.nseg = int((G.kpad + G.kseg - 1) / G.kseg);
    return G;
}

// Stored (row-major) shape of the operands of a logical product.
void stored_a(const Gemm& g, int64_t* rows, int64_t* cols) { *rows = g.ta ? g.k : g.m; *cols = g.ta ? g.m : g.k; }
void stored_b(const Gemm& g, int64_t* rows, int64_t* cols) { *rows = g.tb ? g.n : g.k; *cols = g.tb ? g.k : g.n; }
bool tma_ready(const void* p, int64_t ld) { return reinterpret_cast<uintptr_t>(p) % 16 == 0 && (ld * 8) % 16 == 0; }

// Copy operands whose base or pitch TMA cannot address (16-byte alignment) into the workspace.
int realign_operands(Gemm& g, Workspace& ws, cudaStream_t st, std::string* err) {
    if (g.k == 0) return GB300_OK;
    for (int which = 0; which < 2; ++which) {
        const void*& p = which == 0 ? g.A : g.B;
        int64_t& ld = which == 0 ? g.lda : g.ldb;
        if (tma_ready(p, ld)) continue;
        int64_t rows, cols;
        if (which == 0) stored_a(g, &rows, &cols);
        else stored_b(g, &rows, &cols);
        const int64_t ldp = (cols + 1) / 2 * 2;
        void* d = ws.get(which == 0 ? kSlotA : kSlotB, size_t(rows) * size_t(ldp) * 8, err);
        if (!d) return GB300_ERR_NO_MEMORY;
        const cudaError_t e = cudaMemcpy2DAsync(d, size_t(ldp) * 8, p, size_t(ld) * 8, size_t(cols) * 8, size_t(rows),
                                                cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) {
            if (err) *err = std::string("operand realignment: ") + cudaGetErrorString(e);
            return GB300_ERR_CUDA;
        }
        p = d;
        ld = ldp;
    }
    return GB300_OK;
}

}  // namespace

void device_product_slot_needs(const Gemm& g, const SplitRequest& req, size_t need[kSlotCount]) {
    Runtime& r = runtime();
    for (int i = 0; i < kSlotCount; ++i) need[i] = 0;
    auto rounded = [](size_t b) { return b == 0 ? size_t(0) : (b + (size_t(2) << 20) - 1) & ~((size_t(2) << 20) - 1); };
    if (g.k > 0) {
        int64_t rr, cc;
        if (!tma_ready(g.A, g.lda)) { stored_a(g, &rr, &cc); need[kSlotA] = rounded(size_t(rr) * size_t((cc + 1) / 2 * 2) * 8); }
        if (!tma_ready(g.B, g.ldb)) { stored_b(g, &rr, &cc); need[kSlotB] = rounded(size_t(rr) * size_t((cc + 1) / 2 * 2) * 8); }
    }
    if (g.k == 0 || req.method == GB300_METHOD_NATIVE || (req.method == GB300_METHOD_AUTO && auto_uses_native(g))) {
        const int splits = g.k > 0 ? native_choose_splits(g.m, g.n, g.k, 8, r.num_sms) : 1;
        if (splits > 1) need[kSlotWork] = rounded(size_t(splits) * size_t(g.m) * size_t(g.n) * 8);
        return;
    }
    const SplitGeometry G = split_geometry(g, req, r.num_sms);
    need[kSlotSliceA] = rounded(size_t(G.max_planes) * size_t(G.mpad) * size_t(G.kpad) * 2);
    need[kSlotSliceB] = rounded(size_t(G.max_planes) * size_t(G.npad) * size_t(G.kpad) * 2);
    need[kSlotLevels] = rounded(size_t(G.nseg) * G.max_levels * size_t(G.mpad) * size_t(G.npad) * 4);
    const int64_t off_sq = round_up((g.m + g.n) * int64_t(sizeof(int)), 256);
    const int64_t off_info = round_up(off_sq + (g.m + g.n) * int64_t(sizeof(double)), 256);
    const size_t off_part = size_t(off_info) + ((sizeof(SplitInfo) + 255) / 256) * 256;
    need[kSlotScaleA] = rounded(off_part + size_t((g.m + 255) / 256 + (g.n + 255) / 256) * sizeof(RowPartial));
    need[kSlotScaleB] = rounded(size_t(g.m + g.n) * sizeof(RowAcc));
}

size_t device_product_footprint(const Gemm& g, const SplitRequest& req) {
    size_t need[kSlotCount];
    device_product_slot_needs(g, req, need);
    size_t t = 0;
    for (int i = 0; i < kSlotCount; ++i) t += need[i];
    return t;
}

bool split_auto_uses_native(const Gemm& g) { return auto_uses_native(g); }

// A residue product with at least as many pair tiles as SMs runs its tensor-core work as two
// launches over the two halves of C's column tiles, and the first half's reconstruction runs on a
// second stream while the tensor cores work on the second half: a reconstruction block (128
// threads, no shared memory) fits on an SM beside the tensor-core kernel's one CTA.  The second
// stream belongs to the pair (calling host thread, caller's stream) and has the caller's stream
// priority, so concurrent callers (user threads, or the server's slots, launched from its one
// scheduler thread on their own streams) never queue behind one another's reconstructions; the
// ordering events come from a pool.
struct PartEvents {
    cudaStream_t aux = nullptr;
    cudaEvent_t tc0 = nullptr, done0 = nullptr;
};

struct ThreadAuxStreams {
    static constexpr size_t kMax = 32;
    std::vector<std::pair<cudaStream_t, cudaStream_t>> map;  // caller's stream -> second stream
    ~ThreadAuxStreams() {
        for (auto& kv : map) cudaStreamDestroy(kv.second);  // fails harmlessly once the context is gone
    }
};

// The second stream of the calling host thread for the caller's stream `st` (created on first
// use; past kMax callers' streams the last one is shared, which orders more but stays correct).
static cudaStream_t aux_stream_for(cudaStream_t st, std::string* err) {
    static thread_local ThreadAuxStreams ts;
    for (auto& kv : ts.map)
        if (kv.first == st) return kv.second;
    if (ts.map.size() >= ThreadAuxStreams::kMax) return ts.map.back().second;
    int prio = 0;
    if (cudaStreamGetPriority(st, &prio) != cudaSuccess) {
        cudaGetLastError();
        prio = 0;
    }
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio) != cudaSuccess) {
        if (err) *err = "second stream creation failed";
        return nullptr;
    }
    ts.map.emplace_back(st, s);
    return s;
}

static bool part_events_get(cudaStream_t st, PartEvents* pe, std::string* err) {
    cudaStream_t aux = aux_stream_for(st, err);
    if (!aux) return false;
    Runtime& r = runtime();
    std::lock_guard<std::mutex> lk(r.part_mu);
    cudaEvent_t ev[2];
    for (int i = 0; i < 2; ++i) {
        if (!r.part_events.empty()) {
            ev[i] = r.part_events.back();
            r.part_events.pop_back();
        } else if (cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess) {
            if (i == 1) r.part_events.push_back(ev[0]);
            if (err) *err = "part event creation failed";
            return false;
        }
    }
    pe->aux = aux;
    pe->tc0 = ev[0];
    pe->done0 = ev[1];
    return true;
}

// The events go back to the pool once every record and wait on them is enqueued (a wait takes the
// event's state when it is enqueued, so a later record by another product does not affect it).
static void part_events_put(const PartEvents& pe) {
    Runtime& r = runtime();
    std::lock_guard<std::mutex> lk(r.part_mu);
    r.part_events.push_back(pe.tc0);
    r.part_events.push_back(pe.done0);
}

int device_product(const Gemm& g_in, const SplitRequest& req, const LaunchCtl& ctl, cudaStream_t st, Workspace& ws,
                   SplitResult* out, std::string* err) {
    Runtime& r = runtime();
    Gemm g = g_in;
    {
        const int rst = realign_operands(g, ws, st, err);
        if (rst != GB300_OK) return rst;
    }
    if (g.k == 0 || req.method == GB300_METHOD_NATIVE || (req.method == GB300_METHOD_AUTO && auto_uses_native(g)))
        return native_product(g, ctl, st, ws, out, err);

    const SplitGeometry G = split_geometry(g, req, r.num_sms);
    const int mode = G.mode;
    const int64_t m = g.m, n = g.n, k = g.k;
    const int m_tiles = G.m_tiles, n_tiles = G.n_tiles;
    const int64_t mpad = G.mpad, npad = G.npad, kpad = G.kpad;
    const int kb_total = G.kb_total, max_planes = G.max_planes, max_levels = G.max_levels;
    const int64_t kseg = G.kseg;
    const int nseg = G.nseg;

    // device buffers
    const size_t planesA = size_t(max_planes) * size_t(mpad) * size_t(kpad);
    const size_t planesB = size_t(max_planes) * size_t(npad) * size_t(kpad);
    auto* pa = static_cast<__nv_bfloat16*>(ws.get(kSlotSliceA, planesA * 2, err));
    auto* pb = static_cast<__nv_bfloat16*>(ws.get(kSlotSliceB, planesB * 2, err));
    auto* lv = static_cast<int32_t*>(
        ws.get(kSlotLevels, size_t(nseg) * max_levels * size_t(mpad) * size_t(npad) * 4, err));
    // statistics block: exponents (int), relative sums of squares (double), SplitInfo
    const int64_t off_sq = round_up((m + n) * int64_t(sizeof(int)), 256);
    const int64_t off_info = round_up(off_sq + (m + n) * int64_t(sizeof(double)), 256);
    const int64_t off_part = off_info + int64_t((sizeof(SplitInfo) + 255) / 256) * 256;
    const unsigned xb0 = unsigned((m + 255) / 256), xb1 = unsigned((n + 255) / 256);
    const size_t stat_bytes = size_t(off_part) + size_t(xb0 + xb1) * sizeof(RowPartial);
    auto* stats = static_cast<uint8_t*>(ws.get(kSlotScaleA, stat_bytes, err));
    if (!pa || !pb || !lv || !stats) return GB300_ERR_NO_MEMORY;
    int* eA = reinterpret_cast<int*>(stats);
    int* eB = eA + m;
    double* sqA = reinterpret_cast<double*>(stats + off_sq);
    double* sqB = sqA + m;
    auto* info = reinterpret_cast<SplitInfo*>(stats + off_info);
    auto* part = reinterpret_cast<RowPartial*>(stats + off_part);

    // operand strides of the logical R x K views
    const int64_t a_sr = g.ta ? 1 : g.lda, a_sp = g.ta ? g.lda : 1;
    const int64_t b_sr = g.tb ? g.ldb : 1, b_sp = g.tb ? 1 : g.ldb;
    const double* A = static_cast<const double*>(g.A);
    const double* B = static_cast<const double*>(g.B);

    RowAcc* racc = static_cast<RowAcc*>(ws.get(kSlotScaleB, size_t(m + n) * sizeof(RowAcc), err));
    if (!racc) return GB300_ERR_NO_MEMORY;
    cudaMemsetAsync(racc, 0, size_t(m + n) * sizeof(RowAcc), st);
    OperandPair op;
    op.X[0] = A; op.X[1] = B;
    op.R[0] = m; op.R[1] = n;
    op.sr[0] = a_sr; op.sr[1] = b_sr;
    op.sp[0] = a_sp; op.sp[1] = b_sp;
    op.acc[0] = racc; op.acc[1] = racc + m;
    op.rexp[0] = eA; op.rexp[1] = eB;
    op.rsq[0] = sqA; op.rsq[1] = sqB;
    op.planes[0] = pa; op.planes[1] = pb;
    op.rpad[0] = mpad; op.rpad[1] = npad;
    op.yb0 = unsigned((m + 31) / 32);
    {
        dim3 grid(unsigned(((k + 63) / 64 + TILE_KT - 1) / TILE_KT), unsigned((m + 31) / 32 + (n + 31) / 32));
        stats_tile_kernel<<<grid, 256, 0, st>>>(op, k);
        stats_finalize_pair_kernel<<<xb0 + xb1, 256, 0, st>>>(op, k, xb0, part);
    }
    const double target = req.target_error > 0 ? req.target_error : double(k) * 0x1p-53;
    split_info_kernel<<<1, 32, 0, st>>>(part, int(xb0), int(xb1), k, mode, req.slices > 0 ? max_planes : 0,
                                         max_planes, target, info);
    if (cudaError_t le = cudaGetLastError(); le != cudaSuccess) {
        if (err) *err = std::string("split pre-pass launch: ") + cudaGetErrorString(le);
        return GB300_ERR_CUDA;
    }
    {
        OperandPair sp2 = op;
        sp2.yb0 = unsigned(mpad / 32);
        dim3 grid(unsigned((kpad / 64 + TILE_KT - 1) / TILE_KT), unsigned(mpad / 32 + npad / 32));
        auto sk = mode == kCrt ? slice_kernel<kCrt>
                               : (mode == kExact ? slice_kernel<kExact> : (mode == kBf16 ? slice_kernel<kBf16> : slice_kernel<kBf16x3>));
        sk<<<grid, 256, 0, st>>>(sp2, k, info, kpad);
    }
    count_launches(4);
    if (cudaError_t le = cudaGetLastError(); le != cudaSuccess) {
        if (err) *err = std::string("split slicing launch: ") + cudaGetErrorString(le);
        return GB300_ERR_CUDA;
    }

    CUtensorMap tA, tB;
    if (!encode_tmap_2d(&tA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, pa, uint64_t(max_planes) * mpad, kpad, kpad, TM, TK,
                        CU_TENSOR_MAP_SWIZZLE_128B, err) ||
        !encode_tmap_2d(&tB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, pb, uint64_t(max_planes) * npad, kpad, kpad, TNH, TK,
                        CU_TENSOR_MAP_SWIZZLE_128B, err))
        return GB300_ERR_CUDA;

    // residue planes as a 2-D array of 16-bit values for the epilogue's TMA stores
    CUtensorMap tC = tA;
    if (mode == kCrt &&
        !encode_tmap_2d(&tC, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, lv, uint64_t(nseg) * max_levels * mpad, npad, npad, 32,
                        64, CU_TENSOR_MAP_SWIZZLE_128B, err))
        return GB300_ERR_CUDA;

    TcParams p;
    p.mode = mode;
    p.m_tiles = m_tiles;
    p.n_tiles = n_tiles;
    p.nseg = nseg;
    p.kb_per_seg = int(kseg / TK);
    p.kb_total = kb_total;
    p.mpad = mpad;
    p.npad = npad;
    p.levels = lv;
    p.max_levels = max_levels;
    p.info = info;
    p.status = ctl.status;
    p.limit_ns = ctl.wait_limit_ns;
    p.inject_stall = ctl.inject_stall;
    // units: one level of one pair tile and k-segment (the device picks the level count, at most
    // max_levels); CTA pairs (clusters of two): at most one pair per unit, at least one pair
    const int sms = req.max_sms > 0 ? std::min(req.max_sms, r.num_sms) : r.num_sms;
    auto kern = (mode == kExact || mode == kCrt) ? tc_gemm_kernel<kExact>
                                                 : (mode == kBf16 ? tc_gemm_kernel<kBf16> : tc_gemm_kernel<kBf16x3>);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTcSmem));
    if (e != cudaSuccess) {
        if (err) *err = std::string("tc_gemm_kernel smem attribute: ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    auto launch_tc = [&](int tn0, int nt) {
        TcParams q = p;
        q.tn0 = tn0;
        q.n_tiles = nt;
        const int units = m_tiles * nt * nseg * max_levels;
        const int grid = 2 * std::max(1, std::min(units, sms / 2));
        KernelTimer timer("tc_gemm", st);
        kern<<<grid, THREADS, kTcSmem, st>>>(tA, tB, tC, q);
    };
    // reconstruction of C's columns [c0, c0 + nc) on stream s
    auto launch_crt_combine = [&](int64_t c0, int64_t nc, cudaStream_t s) {
        const int64_t colgroups = (nc + CRT_COMBINE_COLS - 1) / CRT_COMBINE_COLS;
        dim3 cgrid(unsigned((colgroups + 127) / 128), unsigned(std::min<int64_t>(m, 65535)));
        crt_combine_kernel<CRT_COMBINE_COLS><<<cgrid, 128, 0, s>>>(
            reinterpret_cast<const uint16_t*>(lv) + c0, nseg, max_levels, mpad, npad, info, eA, eB + c0, m, nc,
            g.alpha, g.beta, static_cast<double*>(g.C) + c0, g.ldc);
    };
    const bool in_parts = mode == kCrt && n_tiles >= 2 && m_tiles * n_tiles >= sms && req.max_sms <= 0;
    if (in_parts) {
        PartEvents pe;
        if (!part_events_get(st, &pe, err)) return GB300_ERR_CUDA;
        const int nt0 = n_tiles / 2;
        const int64_t c0 = int64_t(nt0) * TN;
        launch_tc(0, nt0);
        cudaEventRecord(pe.tc0, st);
        launch_tc(nt0, n_tiles - nt0);
        cudaStreamWaitEvent(pe.aux, pe.tc0, 0);
        launch_crt_combine(0, c0, pe.aux);
        cudaEventRecord(pe.done0, pe.aux);
        launch_crt_combine(c0, n - c0, st);
        cudaStreamWaitEvent(st, pe.done0, 0);
        part_events_put(pe);
        count_launches(2);
    } else {
        launch_tc(0, n_tiles);
        if (mode == kCrt) {
            launch_crt_combine(0, n, st);
        } else {
            const int64_t colgroups = (n + COMBINE_COLS - 1) / COMBINE_COLS;
            dim3 cgrid(unsigned((colgroups + 127) / 128), unsigned(std::min<int64_t>(m, 65535)));
            combine_kernel<<<cgrid, 128, 0, st>>>(lv, nseg, max_levels, mpad, npad, mode, info, eA, eB, m, n,
                                                  g.alpha, g.beta, static_cast<double*>(g.C), g.ldc);
        }
    }
    count_launches(2);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        if (err) *err = std::string("split-precision launch: ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    out->method_used = mode == kCrt ? GB300_METHOD_SPLIT_CRT
                                    : (req.method == GB300_METHOD_AUTO || req.method == GB300_METHOD_SPLIT_CRT)
                                          ? GB300_METHOD_SPLIT
                                          : req.method;
    out->slices = -1;  // filled in by the caller from the device info when synchronous
    out->error_bound = -1.0;
    out->info_dev = info;
    return GB300_OK;
}


// A float product through the FP64-accurate machinery: A and B (device, float, the caller's
// pitches) are widened to double in `conv`'s slots 0 and 1 (exact), C in slot 2 (read only when
// beta != 0), device_product runs at the float target (k 2^-24 unless the request sets one), and
// the double result is rounded once to float into C.  The reported bound adds 2^-24 for that final
// rounding.
int device_product_float(const Gemm& g, const SplitRequest& req_in, const LaunchCtl& ctl, cudaStream_t st,
                         Workspace& ws, Workspace& conv, SplitResult* out, std::string* err) {
    const int64_t a_rows = g.ta ? g.k : g.m, a_cols = g.ta ? g.m : g.k;
    const int64_t b_rows = g.tb ? g.n : g.k, b_cols = g.tb ? g.k : g.n;
    const int64_t pa = (a_cols + 1) / 2 * 2, pb = (b_cols + 1) / 2 * 2, pc = (g.n + 1) / 2 * 2;  // 16-byte pitches
    auto* dA = static_cast<double*>(conv.get(0, size_t(a_rows) * size_t(pa) * 8, err));
    auto* dB = static_cast<double*>(conv.get(1, size_t(b_rows) * size_t(pb) * 8, err));
    auto* dC = static_cast<double*>(conv.get(2, size_t(g.m) * size_t(pc) * 8, err));
    if (!dA || !dB || !dC) return GB300_ERR_NO_MEMORY;
    cudaError_t e = launch_convert(a_rows, a_cols, static_cast<const float*>(g.A), g.lda, dA, pa, st);
    if (e == cudaSuccess) e = launch_convert(b_rows, b_cols, static_cast<const float*>(g.B), g.ldb, dB, pb, st);
    if (e == cudaSuccess && g.beta != 0.0)
        e = launch_convert(g.m, g.n, static_cast<const float*>(g.C), g.ldc, dC, pc, st);
    if (e != cudaSuccess) {
        if (err) *err = std::string("float widening: ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    Gemm g64 = g;
    g64.A = dA; g64.lda = pa;
    g64.B = dB; g64.ldb = pb;
    g64.C = dC; g64.ldc = pc;
    SplitRequest req = req_in;
    if (req.target_error <= 0) req.target_error = double(std::max<int64_t>(g.k, 1)) * 0x1p-24;
    const int st_ = device_product(g64, req, ctl, st, ws, out, err);
    if (st_ != GB300_OK) return st_;
    e = launch_convert(g.m, g.n, static_cast<const double*>(dC), pc, static_cast<float*>(g.C), g.ldc, st);
    if (e != cudaSuccess) {
        if (err) *err = std::string("float rounding: ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    if (out->error_bound >= 0) out->error_bound += 0x1p-24;
    return GB300_OK;
}

namespace {
bool page_locked(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

bool pipe_init(Runtime& r, std::string* err) {
    if (r.pipe_ready) return true;
    if (cudaStreamCreateWithFlags(&r.copy_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&r.copy_out, cudaStreamNonBlocking) != cudaSuccess) {
        if (err) *err = "copy stream creation failed";
        return false;
    }
    for (int i = 0; i < Runtime::kPipeEvents; ++i)
        if (cudaEventCreateWithFlags(&r.pipe_ev[i], cudaEventDisableTiming) != cudaSuccess) {
            if (err) *err = "event creation failed";
            return false;
        }
    r.pipe_ready = true;
    return true;
}
}  // namespace

int device_product_host_panels(const Gemm& g, const SplitRequest& req, const LaunchCtl& ctl, cudaStream_t st,
                               Workspace& ws, SplitResult* out, std::string* err) {
    Runtime& r = runtime();
    const int64_t m = g.m, n = g.n, k = g.k;
    if (k == 0 || req.method == GB300_METHOD_NATIVE || (req.method == GB300_METHOD_AUTO && auto_uses_native(g)) ||
        req.max_sms > 0 || req.slices > 0)
        return GB300_ERR_NOT_SUPPORTED;
    const SplitGeometry G = split_geometry(g, req, r.num_sms);
    if (G.mode != kCrt) return GB300_ERR_NOT_SUPPORTED;
    // blocks: row panels of about a quarter of A (at least 2048 rows) and up to kPipeMaxQ column
    // blocks of B of at least 2048 columns each, whole pair tiles.  Four column blocks at 8192^3
    // start the first block earlier (A_0 and B_0 are 256 MiB instead of 384) but measured the same
    // end to end and 1 % slower with pageable memory; loading A and B alternately in quarters over a
    // 4 x 4 grid measured 6 % slower (the copies of C back then share the link with more of the
    // copies in).
    const bool c_locked = page_locked(g.C);
    const int64_t Mp = std::max<int64_t>(2048, round_up((m + 3) / 4, TMP));
    const int P = int((m + Mp - 1) / Mp);
    const int64_t Q0 = std::max<int64_t>(1, std::min<int64_t>(kPipeMaxQ, n / 2048));
    const int64_t Nq = round_up((n + Q0 - 1) / Q0, TN);
    const int Q = int((n + Nq - 1) / Nq);
    if (P < 2 || P > 16 || Q > kPipeMaxQ) return GB300_ERR_NOT_SUPPORTED;
    if (!pipe_init(r, err)) return GB300_ERR_CUDA;
    Gemm gp = g;
    gp.m = Mp;
    gp.n = Nq;
    const SplitGeometry Gp = split_geometry(gp, req, r.num_sms);
    const int64_t mpad = Gp.mpad, kpad = Gp.kpad;
    // B planes plane-major over the whole width: plane b holds the Q * Nq columns of every column
    // block (block j at rows j * Nq..), so one tensor map addresses all blocks and one launch can
    // cover all blocks of a panel
    const int max_planes = Gp.max_planes, max_levels = Gp.max_levels, nseg = Gp.nseg;
    const int64_t npb = int64_t(Q) * Nq;

    // device copies of the operands in their stored shapes (dense pitch), C, planes, levels, statistics
    const int64_t a_rows = g.ta ? k : m, a_cols = g.ta ? m : k;
    const int64_t b_rows = g.tb ? n : k, b_cols = g.tb ? k : n;
    auto* dA = static_cast<double*>(ws.get(kSlotA, size_t(a_rows) * size_t(a_cols) * 8, err));
    auto* dB = static_cast<double*>(ws.get(kSlotB, size_t(b_rows) * size_t(b_cols) * 8, err));
    auto* dC = static_cast<double*>(ws.get(kSlotC, size_t(m) * size_t(n) * 8, err));
    // A planes of one panel: a panel's blocks all run before the next panel is sliced
    auto* pa = static_cast<__nv_bfloat16*>(ws.get(kSlotSliceA, size_t(max_planes) * size_t(mpad) * size_t(kpad) * 2, err));
    auto* pb = static_cast<__nv_bfloat16*>(ws.get(kSlotSliceB, size_t(max_planes) * size_t(npb) * size_t(kpad) * 2, err));
    // level planes of a launch over the whole width, two buffers: launch L's reconstructions (on the
    // second stream) read buffer L % 2 while launch L + 1's tensor-core work writes the other
    const size_t lv_elems = size_t(nseg) * max_levels * size_t(mpad) * size_t(npb);
    auto* lv = static_cast<int32_t*>(ws.get(kSlotLevels, 2 * lv_elems * 4, err));
    const int64_t off_sq = round_up((m + n) * int64_t(sizeof(int)), 256);
    const int64_t off_info = round_up(off_sq + (m + n) * int64_t(sizeof(double)), 256);
    const int ninfo = P + Q + P * Q + P + 1;
    const size_t info_stride = ((sizeof(SplitInfo) + 255) / 256) * 256;
    auto* stats = static_cast<uint8_t*>(ws.get(kSlotScaleA, size_t(off_info) + size_t(ninfo) * info_stride, err));
    auto* racc = static_cast<RowAcc*>(ws.get(kSlotScaleB, size_t(m + n) * sizeof(RowAcc), err));
    if (!dA || !dB || !dC || !pa || !pb || !lv || !stats || !racc) return GB300_ERR_NO_MEMORY;
    int* eA = reinterpret_cast<int*>(stats);
    int* eB = eA + m;
    double* sqA = reinterpret_cast<double*>(stats + off_sq);
    double* sqB = sqA + m;
    auto info_at = [&](int i) { return reinterpret_cast<SplitInfo*>(stats + off_info + size_t(i) * info_stride); };
    // infos: [0, P) panels of A, [P, P+Q) blocks of B, [P+Q, P+Q+PQ) blocks of C, [P+Q+PQ,
    // P+Q+PQ+P) the launches over a whole panel (the largest level count of its blocks), last: summary
    SplitInfo* info_sum = info_at(ninfo - 1);
    const double target = req.target_error > 0 ? req.target_error : double(k) * 0x1p-53;
    // events: [0, P) A panels in, [P, P+Q) B blocks in, [P+Q, P+Q+PQ) C blocks computed, next:
    // all out, then [P+Q+PQ+1, P+Q+2PQ+1) the launches' tensor-core work done
    cudaEvent_t* ev = r.pipe_ev;
    if (P + Q + 2 * P * Q + 1 > Runtime::kPipeEvents) return GB300_ERR_NOT_SUPPORTED;
    cudaStream_t aux = aux_stream_for(st, err);
    if (!aux) return GB300_ERR_CUDA;
    auto cuda_fail = [&](const char* what, cudaError_t e) {
        if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    };
    const double* hA = static_cast<const double*>(g.A);
    const double* hB = static_cast<const double*>(g.B);
    double* hC = static_cast<double*>(g.C);

    // ---- copies in (issued by `load` below, in its order) ----
    cudaError_t e = cudaSuccess;
    auto copy_a = [&](int i) {
        const int64_t r0 = int64_t(i) * Mp, mi = std::min(Mp, m - r0);
        if (g.ta)  // columns r0.. of the stored k x m operand
            e = cudaMemcpy2DAsync(dA + r0, size_t(a_cols) * 8, hA + r0, size_t(g.lda) * 8, size_t(mi) * 8, size_t(k),
                                  cudaMemcpyHostToDevice, r.copy_in);
        else
            e = cudaMemcpy2DAsync(dA + r0 * a_cols, size_t(a_cols) * 8, hA + r0 * g.lda, size_t(g.lda) * 8,
                                  size_t(k) * 8, size_t(mi), cudaMemcpyHostToDevice, r.copy_in);
        if (e == cudaSuccess && g.beta != 0.0)
            e = cudaMemcpy2DAsync(dC + r0 * n, size_t(n) * 8, hC + r0 * g.ldc, size_t(g.ldc) * 8, size_t(n) * 8,
                                  size_t(mi), cudaMemcpyHostToDevice, r.copy_in);
        cudaEventRecord(ev[i], r.copy_in);
    };
    auto copy_b = [&](int j) {
        const int64_t c0 = int64_t(j) * Nq, nj = std::min(Nq, n - c0);
        if (g.tb)  // rows c0.. of the stored n x k operand
            e = cudaMemcpy2DAsync(dB + c0 * b_cols, size_t(b_cols) * 8, hB + c0 * g.ldb, size_t(g.ldb) * 8,
                                  size_t(k) * 8, size_t(nj), cudaMemcpyHostToDevice, r.copy_in);
        else
            e = cudaMemcpy2DAsync(dB + c0, size_t(b_cols) * 8, hB + c0, size_t(g.ldb) * 8, size_t(nj) * 8, size_t(k),
                                  cudaMemcpyHostToDevice, r.copy_in);
        cudaEventRecord(ev[P + j], r.copy_in);
    };
    cudaMemsetAsync(racc, 0, size_t(m + n) * sizeof(RowAcc), st);
    const unsigned ktiles = unsigned(((k + 63) / 64 + TILE_KT - 1) / TILE_KT);
    const unsigned stiles = unsigned((kpad / 64 + TILE_KT - 1) / TILE_KT);
    const int64_t a_sr = g.ta ? 1 : a_cols, a_sp = g.ta ? a_cols : 1;
    const int64_t b_sr = g.tb ? b_cols : 1, b_sp = g.tb ? 1 : b_cols;
    OperandPair base;
    base.X[0] = dA; base.X[1] = dB;
    base.R[0] = 0; base.R[1] = 0;
    base.sr[0] = a_sr; base.sr[1] = b_sr;
    base.sp[0] = a_sp; base.sp[1] = b_sp;
    base.acc[0] = racc; base.acc[1] = racc + m;
    base.rexp[0] = eA; base.rexp[1] = eB;
    base.rsq[0] = sqA; base.rsq[1] = sqB;
    base.planes[0] = pa; base.planes[1] = pb;
    base.rpad[0] = mpad; base.rpad[1] = npb;
    base.yb0 = 0;
    // statistics, side scaling and planes of A's panel i (into the panel plane buffer)
    auto prep_a = [&](int i) {
        const int64_t r0 = int64_t(i) * Mp, mi = std::min(Mp, m - r0);
        OperandPair o = base;
        o.X[0] = g.ta ? dA + r0 : dA + r0 * a_cols;
        o.R[0] = mi;
        o.acc[0] = racc + r0;
        o.rexp[0] = eA + r0;
        o.rsq[0] = sqA + r0;
        o.yb0 = unsigned((mi + 31) / 32);
        stats_tile_kernel<<<dim3(ktiles, o.yb0), 256, 0, st>>>(o, k);
        const unsigned xb0 = unsigned((mi + 255) / 256);
        stats_finalize_pair_kernel<<<xb0, 256, 0, st>>>(o, k, xb0, nullptr);
        split_side_kernel<<<1, 1024, 0, st>>>(eA + r0, sqA + r0, mi, k, max_planes, target, info_at(i));
        o.yb0 = unsigned(mpad / 32);
        slice_kernel<kCrt><<<dim3(stiles, o.yb0), 256, 0, st>>>(o, k, info_at(i), kpad);
        count_launches(4);
    };
    // statistics, side scaling and planes of B's column block j (rows j*Nq.. of the B planes)
    auto prep_b = [&](int j) {
        const int64_t c0 = int64_t(j) * Nq, nj = std::min(Nq, n - c0);
        OperandPair o = base;
        o.X[1] = g.tb ? dB + c0 * b_cols : dB + c0;
        o.R[1] = nj;
        o.acc[1] = racc + m + c0;
        o.rexp[1] = eB + c0;
        o.rsq[1] = sqB + c0;
        o.planes[1] = pb + size_t(j) * size_t(Nq) * size_t(kpad);
        o.rpad[1] = npb;
        o.yb0 = 0;
        stats_tile_kernel<<<dim3(ktiles, unsigned((nj + 31) / 32)), 256, 0, st>>>(o, k);
        stats_finalize_pair_kernel<<<unsigned((nj + 255) / 256), 256, 0, st>>>(o, k, 0u, nullptr);
        split_side_kernel<<<1, 1024, 0, st>>>(eB + c0, sqB + c0, nj, k, max_planes, target, info_at(P + j));
        slice_kernel<kCrt><<<dim3(stiles, unsigned(Nq / 32)), 256, 0, st>>>(o, k, info_at(P + j), kpad);
        count_launches(4);
    };

    // ---- tensor maps: A panel planes, the B planes, the level planes of a launch ----
    CUtensorMap tA, tB, tC[2];
    if (!encode_tmap_2d(&tA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, pa, uint64_t(max_planes) * mpad, kpad, kpad, TM, TK,
                        CU_TENSOR_MAP_SWIZZLE_128B, err) ||
        !encode_tmap_2d(&tB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, pb, uint64_t(max_planes) * npb, kpad, kpad, TNH, TK,
                        CU_TENSOR_MAP_SWIZZLE_128B, err))
        return GB300_ERR_CUDA;
    for (int b = 0; b < 2; ++b)
        if (!encode_tmap_2d(&tC[b], CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, lv + b * lv_elems,
                            uint64_t(nseg) * max_levels * mpad, npb, npb, 32, 64, CU_TENSOR_MAP_SWIZZLE_128B, err))
            return GB300_ERR_CUDA;
    e = cudaFuncSetAttribute(tc_gemm_kernel<kExact>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTcSmem));
    if (e != cudaSuccess) return cuda_fail("tc_gemm_kernel smem attribute", e);

    // ---- operands in, blocks as their operands arrive, C back ----
    // Load order A_0, B_0 .. B_{Q-1}, A_1 .. A_{P-1}; after each load the blocks it completes are
    // queued (block (i, j) needs A_i and B_j), so panel i's blocks run together on the panel's
    // planes.  With page-locked memory every call returns at once; with pageable memory each copy
    // holds the host thread until it is done, and the order keeps the GPU busy meanwhile: A_i+1
    // goes in and panel i-1 comes out while panel i computes.  C goes back per block as soon as the
    // block is done (page-locked C); a pageable C goes back per panel, one linear copy when its rows
    // are exactly n elements (pitched copies into untouched pageable pages are slow, see
    // copy_to_host), else per block.
    const bool c_per_panel = !c_locked && Q > 1 && g.ldc == n;
    auto block_ev = [&](int i, int j) { return ev[P + Q + i * Q + j]; };
    auto copy_block_out = [&](int i, int j) {
        const int64_t r0 = int64_t(i) * Mp, mi = std::min(Mp, m - r0);
        const int64_t c0 = int64_t(j) * Nq, nj = std::min(Nq, n - c0);
        cudaStreamWaitEvent(r.copy_out, block_ev(i, j), 0);
        e = copy_to_host(hC + r0 * g.ldc + c0, size_t(g.ldc) * 8, dC + r0 * n + c0, size_t(n) * 8, size_t(nj) * 8,
                         size_t(mi), r.copy_out);
    };
    auto copy_panel_out = [&](int i) {
        if (!c_per_panel) {
            for (int j = 0; j < Q && e == cudaSuccess; ++j) copy_block_out(i, j);
            return;
        }
        const int64_t r0 = int64_t(i) * Mp, mi = std::min(Mp, m - r0);
        for (int j = 0; j < Q; ++j) cudaStreamWaitEvent(r.copy_out, block_ev(i, j), 0);
        e = copy_to_host(hC + r0 * g.ldc, size_t(g.ldc) * 8, dC + r0 * n, size_t(n) * 8, size_t(n) * 8, size_t(mi),
                         r.copy_out);
    };
    // Launch L (blocks j0..j1-1 of panel i, one tensor-core launch) writes level buffer L % 2 on st;
    // each block's reconstruction runs on the second stream and records the block's event, which the
    // copies of C wait on; launch L + 2 waits for launch L's reconstructions before it overwrites the
    // buffer.  A panel whose A arrives after all of B runs as one launch (fewer, fuller waves of pair
    // units than a launch per block), except the last: its blocks' copies back then start one block
    // earlier; the first panel's blocks run as their B blocks arrive.
    int nlaunch = 0;
    int launch_i[16 * kPipeMaxQ], launch_j0[16 * kPipeMaxQ], launch_j1[16 * kPipeMaxQ];
    auto tc_done_ev = [&](int l) { return ev[P + Q + P * Q + 1 + l]; };
    auto run_blocks = [&](int i, int j0, int j1) {
        const int64_t r0 = int64_t(i) * Mp, mi = std::min(Mp, m - r0);
        const int64_t c0 = int64_t(j0) * Nq, c1 = std::min(n, int64_t(j1) * Nq);
        const int l = nlaunch++;
        const int buf = l & 1;
        int32_t* lvb = lv + buf * lv_elems;
        if (l >= 2)
            for (int j = launch_j0[l - 2]; j < launch_j1[l - 2]; ++j)
                cudaStreamWaitEvent(st, block_ev(launch_i[l - 2], j), 0);
        launch_i[l] = i;
        launch_j0[l] = j0;
        launch_j1[l] = j1;
        for (int j = j0; j < j1; ++j)
            split_block_kernel<<<1, 32, 0, st>>>(info_at(i), info_at(P + j), k, max_planes, info_at(P + Q + i * Q + j));
        SplitInfo* linfo = info_at(P + Q + i * Q + j0);
        if (j1 - j0 > 1) {
            linfo = info_at(P + Q + P * Q + i);
            split_max_slices_kernel<<<1, 32, 0, st>>>(reinterpret_cast<const uint8_t*>(info_at(P + Q + i * Q + j0)),
                                                      info_stride, j1 - j0, linfo);
            count_launches(1);
        }
        TcParams tp;
        tp.mode = kCrt;
        tp.m_tiles = int((mi + TMP - 1) / TMP);
        tp.tn0 = int(c0 / TN);
        tp.n_tiles = int((c1 - c0 + TN - 1) / TN);
        tp.nseg = nseg;
        tp.kb_per_seg = int(Gp.kseg / TK);
        tp.kb_total = Gp.kb_total;
        tp.mpad = mpad;
        tp.npad = npb;
        tp.levels = lvb;
        tp.max_levels = max_levels;
        tp.info = linfo;
        tp.status = ctl.status;
        tp.limit_ns = ctl.wait_limit_ns;
        tp.inject_stall = ctl.inject_stall;
        const int units = tp.m_tiles * tp.n_tiles * nseg * max_levels;
        const int grid = 2 * std::max(1, std::min(units, r.num_sms / 2));
        {
            KernelTimer timer("tc_gemm", st);
            tc_gemm_kernel<kExact><<<grid, THREADS, kTcSmem, st>>>(tA, tB, tC[buf], tp);
        }
        cudaEventRecord(tc_done_ev(l), st);
        cudaStreamWaitEvent(aux, tc_done_ev(l), 0);
        for (int j = j0; j < j1; ++j) {
            const int64_t cj = int64_t(j) * Nq, nj = std::min(Nq, n - cj);
            const int64_t colgroups = (nj + CRT_COMBINE_COLS - 1) / CRT_COMBINE_COLS;
            crt_combine_kernel<CRT_COMBINE_COLS>
                <<<dim3(unsigned((colgroups + 127) / 128), unsigned(std::min<int64_t>(mi, 65535))), 128, 0, aux>>>(
                    reinterpret_cast<const uint16_t*>(lvb) + cj, nseg, max_levels, mpad, npb,
                    info_at(P + Q + i * Q + j), eA + r0, eB + cj, mi, nj, g.alpha, g.beta, dC + r0 * n + cj, n);
            if ((e = cudaGetLastError()) != cudaSuccess) return;
            cudaEventRecord(block_ev(i, j), aux);
            if (c_locked) copy_block_out(i, j);
        }
        count_launches(1 + 2 * (j1 - j0));
    };
    bool have_a[16] = {}, have_b[kPipeMaxQ] = {};
    int nb = 0;  // B blocks in
    auto load = [&](int side, int idx) {
        if (side == 0) {
            copy_a(idx);
            if (e != cudaSuccess) return;
            cudaStreamWaitEvent(st, ev[idx], 0);
            prep_a(idx);
            have_a[idx] = true;
            if (nb == Q && idx + 1 < P) run_blocks(idx, 0, Q);
            else
                for (int j = 0; j < Q && e == cudaSuccess; ++j)
                    if (have_b[j]) run_blocks(idx, j, j + 1);
        } else {
            copy_b(idx);
            if (e != cudaSuccess) return;
            cudaStreamWaitEvent(st, ev[P + idx], 0);
            prep_b(idx);
            have_b[idx] = true;
            ++nb;
            for (int i = 0; i < P && e == cudaSuccess; ++i)
                if (have_a[i]) run_blocks(i, idx, idx + 1);
        }
    };
    load(0, 0);
    for (int j = 0; j < Q && e == cudaSuccess; ++j) load(1, j);
    for (int i = 1; i < P && e == cudaSuccess; ++i) {
        load(0, i);
        if (e == cudaSuccess && !c_locked) copy_panel_out(i - 1);
    }
    if (e == cudaSuccess && !c_locked) copy_panel_out(P - 1);
    if (e != cudaSuccess) return cuda_fail("block pipeline", e);
    split_panels_summary_kernel<<<1, 32, 0, st>>>(reinterpret_cast<const uint8_t*>(info_at(P + Q)), info_stride,
                                                  P * Q, info_sum);
    count_launches(1);
    cudaEventRecord(ev[P + Q + P * Q], r.copy_out);
    cudaStreamWaitEvent(st, ev[P + Q + P * Q], 0);  // the call's work ends on st
    for (int l = std::max(0, nlaunch - 2); l < nlaunch; ++l)  // and so does the second stream's
        for (int j = launch_j0[l]; j < launch_j1[l]; ++j) cudaStreamWaitEvent(st, block_ev(launch_i[l], j), 0);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail("block pipeline", e);
    out->method_used = GB300_METHOD_SPLIT_CRT;
    out->slices = -1;
    out->error_bound = -1.0;
    out->info_dev = info_sum;
    return GB300_OK;
}

}  // namespace gb
