// grouped.cu — K4: persistent grouped GEMM for many independent, uneven, small products
// (Blaze's StaticMatrix / HybridMatrix sizes), FP64 (DFMA) and FP32 (FFMA), one launch per batch,
// captured in a CUDA graph, with warp-tile shapes picked per size class by an autotuner.
//
// Blaze evaluates every such product separately on the CPU through its small vectorized kernel
// (blaze/math/expressions/DMatDMatMultExpr.h:864-1878, DMatTDMatMultExpr.h:1067+); it has no
// batched product, so this is a new entry point (gb300_?gemm_grouped) with the per-product CBLAS
// argument conventions.
//
// Design:
//   * Every product is brought to the row-major form (as for the single products) and tiled with
//     the warp-tile shape chosen for its (m, n, k) class.  Warp tile = (8*R) x (4*C) outputs, lane
//     (ly, lx) of an 8 x 4 lane grid owning rows ly + 8r and columns lx + 4c, so a warp's B loads
//     are coalesced runs and its A loads are 8 broadcast rows.
//   * One flat tile list, sorted by descending work (longest first), is consumed by persistent
//     warps through a global atomic counter (warp-granular work stealing): uneven products
//     balance across SMs without a per-product launch.
//   * Operands are read through L1 (__ldg): a small product's panels stay cache-resident across the
//     k loop, and on this chip the FP64 pipe (about 2 DFMA/clock/SM) — not the load path — bounds
//     the FP64 form, so the tile shapes exist to avoid multiply-adds on padding.
//   * The launch (counter reset + kernel) is captured once into a CUDA graph owned by the plan;
//     running the plan is one graph launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/gb300_blas.h"
#include "runtime.h"

namespace gb {
namespace {

// Warp-tile shapes: (R, C) -> (8R) x (4C) outputs per warp.
struct Shape {
    int R, C;
};
constexpr Shape kShapes[] = {{1, 2}, {2, 4}, {4, 4}, {2, 8}, {4, 8}, {8, 8}};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);
__host__ __device__ constexpr int shape_rows(int s) { return s == 0 ? 8 : s == 1 ? 16 : s == 2 ? 32 : s == 3 ? 16 : s == 4 ? 32 : 64; }
__host__ __device__ constexpr int shape_cols(int s) { return s == 0 ? 8 : s == 1 ? 16 : s == 2 ? 16 : s == 3 ? 32 : s == 4 ? 32 : 32; }

struct DevProblem {
    const void* A;
    const void* B;
    void* C;
    int64_t lda, ldb, ldc;
    int m, n, k;
    int ta, tb;
    int shape;
    double alpha, beta;
};

struct DevTile {
    int prob;
    int tm, tn;  // tile coordinates in units of the problem's warp tile
    int pad;
};

template <typename T, int R, int C>
__device__ __forceinline__ void warp_tile(const DevProblem& p, int tm, int tn, int lane) {
    const int ly = lane >> 2, lx = lane & 3;
    const int row0 = tm * (8 * R) + ly;
    const int col0 = tn * (4 * C) + lx;
    // A(i, kk) = A[i*a_rs + kk*a_ks], B(kk, j) = B[kk*b_ks + j*b_cs]; one running pointer per operand
    const int64_t a_rs = p.ta ? 1 : p.lda, a_ks = p.ta ? p.lda : 1;
    const int64_t b_cs = p.tb ? p.ldb : 1, b_ks = p.tb ? 1 : p.ldb;
    const int64_t a8 = 8 * a_rs, b4 = 4 * b_cs;
    const T* pa = static_cast<const T*>(p.A) + int64_t(row0) * a_rs;
    const T* pb = static_cast<const T*>(p.B) + int64_t(col0) * b_cs;
    uint32_t rmask = 0, cmask = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) rmask |= (row0 + 8 * r < p.m) ? (1u << r) : 0u;
#pragma unroll
    for (int c = 0; c < C; ++c) cmask |= (col0 + 4 * c < p.n) ? (1u << c) : 0u;
    T acc[R][C];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < C; ++c) acc[r][c] = T(0);
    auto step = [&]() {
        T a0[R], b0[C];
#pragma unroll
        for (int r = 0; r < R; ++r) a0[r] = (rmask >> r) & 1u ? __ldg(pa + r * a8) : T(0);
#pragma unroll
        for (int c = 0; c < C; ++c) b0[c] = (cmask >> c) & 1u ? __ldg(pb + c * b4) : T(0);
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < C; ++c) acc[r][c] = fma(a0[r], b0[c], acc[r][c]);
        pa += a_ks;
        pb += b_ks;
    };
    // FP64: unrolled so that the loads of the next k step issue before this step's multiply-adds
    // retire; FP32: not unrolled, which keeps every shape within the 128 registers that let an SM
    // hold two blocks (latency is hidden by warps instead).  The accumulation order of every output
    // stays k = 0, 1, 2, ... either way.
    if constexpr (sizeof(T) == 8) {
#pragma unroll 2
        for (int kk = 0; kk < p.k; ++kk) step();
    } else {
#pragma unroll 1
        for (int kk = 0; kk < p.k; ++kk) step();
    }
    T* Cp = static_cast<T*>(p.C);
    const T alpha = T(p.alpha), beta = T(p.beta);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (!((rmask >> r) & 1u)) continue;
        T* crow = Cp + int64_t(row0 + 8 * r) * p.ldc;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            if (!((cmask >> c) & 1u)) continue;
            const int j = col0 + 4 * c;
            const T v = alpha * acc[r][c];
            crow[j] = (beta == T(0)) ? v : fma(beta, crow[j], v);
        }
    }
}

// FP32 warp tiles stage their operands through shared memory, KC k-steps at a time: a warp reads
// its A rows and B columns with coalesced loads (the contiguous dimension across lanes) into its own
// region, then every k step reads them back from there.  Read straight from global memory, each k
// step of an A row costs one cache line per row of the tile for one multiply-add per row and
// column, which bounds small FP32 tiles by L1 line traffic rather than by the FFMA pipe.  Lane
// (ly, lx) owns rows ly + 8r and the C contiguous columns lx*C .. lx*C + C-1 of the tile, so a k
// step reads its B values with 16-byte shared loads (8-byte for C = 2), and one 16-byte load of an
// A row serves KV = 4 k steps (2 for the 8 x 8 shape, whose accumulators leave fewer registers).
// Rows of both staging arrays are padded to multiples of 16 bytes; the 16-byte reads of a warp then
// touch distinct banks (A: rows 36 floats apart land 4 banks apart).  Every output still sums k in
// order, so the results are those of the unstaged tile.
constexpr int KC = 32;                                   // k-steps per staged block
constexpr int PA = KC + 4;                               // A row pitch (floats)
constexpr int kStageA = 32 * PA;                         // up to 32 rows (FP32 tiles stop at 32 x 32)
constexpr int kStageB = KC * (32 + 4);                   // up to 32 columns, pitch TC + 4
constexpr int kStageWarp = kStageA + kStageB;            // floats per warp
constexpr int kStageBytes = 8 * kStageWarp * int(sizeof(float));  // per 256-thread block

// C consecutive floats from 16-byte (or, for C = 2, 8-byte) aligned shared memory.
template <int C>
__device__ __forceinline__ void lds_vec(const float* __restrict__ src, float (&v)[C]) {
    if constexpr (C == 2) {
        const float2 t = *reinterpret_cast<const float2*>(src);
        v[0] = t.x; v[1] = t.y;
    } else {
#pragma unroll
        for (int q = 0; q < C / 4; ++q) {
            const float4 t = *reinterpret_cast<const float4*>(src + 4 * q);
            v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
        }
    }
}

template <int R, int C>
__device__ __forceinline__ void warp_tile_staged(const DevProblem& p, int tm, int tn, int lane, float* __restrict__ sw) {
    constexpr int TR = 8 * R, TC = 4 * C, PB = TC + 4;
    constexpr int KV = R >= 8 ? 2 : 4;  // k steps per A load
    float* As = sw;            // As[r * PA + kk]
    float* Bs = sw + kStageA;  // Bs[kk * PB + c]
    const int ly = lane >> 2, lx = lane & 3;
    const int i0 = tm * TR, j0 = tn * TC;
    const float* A = static_cast<const float*>(p.A);
    const float* B = static_cast<const float*>(p.B);
    float acc[R][C];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < C; ++c) acc[r][c] = 0.f;
    for (int k0 = 0; k0 < p.k; k0 += KC) {
        const int kc = min(KC, p.k - k0);
        // A(i, kk) = A[i lda + kk] (k contiguous) or A[kk lda + i] (m contiguous); zeros outside
        if (!p.ta) {
            for (int r = 0; r < TR; ++r) {
                const int i = i0 + r;
                As[r * PA + lane] = (i < p.m && lane < kc) ? __ldg(A + int64_t(i) * p.lda + k0 + lane) : 0.f;
            }
        } else {
            for (int idx = lane; idx < TR * KC; idx += 32) {
                const int r = idx % TR, kk = idx / TR, i = i0 + r;
                As[r * PA + kk] = (i < p.m && kk < kc) ? __ldg(A + int64_t(k0 + kk) * p.lda + i) : 0.f;
            }
        }
        // B(kk, j) = B[kk ldb + j] (n contiguous) or B[j ldb + kk] (k contiguous)
        if (!p.tb) {
            for (int idx = lane; idx < KC * TC; idx += 32) {
                const int c = idx % TC, kk = idx / TC, j = j0 + c;
                Bs[kk * PB + c] = (j < p.n && kk < kc) ? __ldg(B + int64_t(k0 + kk) * p.ldb + j) : 0.f;
            }
        } else {
            for (int c = 0; c < TC; ++c) {
                const int j = j0 + c;
                Bs[lane * PB + c] = (j < p.n && lane < kc) ? __ldg(B + int64_t(j) * p.ldb + k0 + lane) : 0.f;
            }
        }
        __syncwarp();
        const float* arow = As + ly * PA;
        const float* bcol = Bs + lx * C;
        const int kv = kc & ~(KV - 1);
#pragma unroll 1
        for (int kk = 0; kk < kv; kk += KV) {
            float a[R][KV];
#pragma unroll
            for (int r = 0; r < R; ++r) lds_vec<KV>(arow + 8 * r * PA + kk, a[r]);
#pragma unroll
            for (int q = 0; q < KV; ++q) {
                float b[C];
                lds_vec<C>(bcol + (kk + q) * PB, b);
#pragma unroll
                for (int r = 0; r < R; ++r)
#pragma unroll
                    for (int c = 0; c < C; ++c) acc[r][c] = fmaf(a[r][q], b[c], acc[r][c]);
            }
        }
        // the last kc % KV steps one at a time (the staged zeros beyond kc are never added, so an
        // output's sum is exactly that of its k range)
#pragma unroll 1
        for (int kk = kv; kk < kc; ++kk) {
            float b[C];
            lds_vec<C>(bcol + kk * PB, b);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float a = arow[8 * r * PA + kk];
#pragma unroll
                for (int c = 0; c < C; ++c) acc[r][c] = fmaf(a, b[c], acc[r][c]);
            }
        }
        __syncwarp();
    }
    float* Cp = static_cast<float*>(p.C);
    const float alpha = float(p.alpha), beta = float(p.beta);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int i = i0 + ly + 8 * r;
        if (i >= p.m) continue;
        float* crow = Cp + int64_t(i) * p.ldc;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int j = j0 + lx * C + c;
            if (j >= p.n) continue;
            const float v = alpha * acc[r][c];
            crow[j] = (beta == 0.f) ? v : fmaf(beta, crow[j], v);
        }
    }
}

// Shapes available per element type: FP64 stops at 16x32 / 32x16 warp tiles (16 accumulators per
// lane): on the FP64 pipe a larger tile only adds padding, and the smaller register footprint lets an
// SM hold twice the warps.  FP32 stops at 32x32 (32 accumulators per lane), so that an SM holds three
// 256-thread blocks (24 warps) to cover the latency of the staging loads.
template <typename T>
__host__ __device__ constexpr int max_shape() { return sizeof(T) == 8 ? 3 : 4; }

template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 2 : 3)
grouped_kernel(const DevProblem* __restrict__ probs, const DevTile* __restrict__ tiles, int ntiles,
               int* __restrict__ counter) {
    const int lane = threadIdx.x & 31;
    // FP32: the warp's staging region (dynamic shared memory of kStageBytes per block)
    extern __shared__ float stage_smem[];
    float* sw = stage_smem + (threadIdx.x >> 5) * kStageWarp;
    (void)sw;
    int t = 0;
    if (lane == 0) t = atomicAdd(counter, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    while (t < ntiles) {
        // the next tile's ticket is taken now and read after this tile: the atomic's round trip
        // overlaps the tile's work instead of preceding every tile (small tiles are a few hundred
        // clocks of multiply-adds)
        int next = 0;
        if (lane == 0) next = atomicAdd(counter, 1);
        const DevTile tl = tiles[t];
        const DevProblem p = probs[tl.prob];
        if constexpr (sizeof(T) == 4) {
            switch (p.shape) {
                case 0: warp_tile_staged<1, 2>(p, tl.tm, tl.tn, lane, sw); break;
                case 1: warp_tile_staged<2, 4>(p, tl.tm, tl.tn, lane, sw); break;
                case 2: warp_tile_staged<4, 4>(p, tl.tm, tl.tn, lane, sw); break;
                case 3: warp_tile_staged<2, 8>(p, tl.tm, tl.tn, lane, sw); break;
                default: warp_tile_staged<4, 8>(p, tl.tm, tl.tn, lane, sw); break;
            }
        } else {
            switch (p.shape) {
                case 0: warp_tile<T, 1, 2>(p, tl.tm, tl.tn, lane); break;
                case 1: warp_tile<T, 2, 4>(p, tl.tm, tl.tn, lane); break;
                case 2: warp_tile<T, 4, 4>(p, tl.tm, tl.tn, lane); break;
                case 3: warp_tile<T, 2, 8>(p, tl.tm, tl.tn, lane); break;
                case 4:
                    if constexpr (max_shape<T>() >= 4) warp_tile<T, 4, 8>(p, tl.tm, tl.tn, lane);
                    break;
                default:
                    if constexpr (max_shape<T>() >= 5) warp_tile<T, 8, 8>(p, tl.tm, tl.tn, lane);
                    break;
            }
        }
        t = __shfl_sync(0xffffffffu, next, 0);
    }
}

// ---- tuning table ------------------------------------------------------------------------------
// Size classes: m and n bucketed by powers of two (<=8, <=16, <=32, <=64, <=128, >128), k by
// (<=16, <=64, >64).  Entry = warp-tile shape index.
constexpr int kMB = 6, kKB = 3;
int bucket_mn(int x) { return x <= 8 ? 0 : x <= 16 ? 1 : x <= 32 ? 2 : x <= 64 ? 3 : x <= 128 ? 4 : 5; }
int bucket_k(int x) { return x <= 16 ? 0 : x <= 64 ? 1 : 2; }

// How a plan picks a product's shape, per element type:
//   kPickModel   no table: the least padded work for the product's own m and n (model_shape);
//   kPickTable   a loaded table without costs: the shape stored for the product's size class;
//   kPickCost    autotuned (or a table with costs): for the product's own m, n the shape with the
//                least (padded multiply-adds) x (the time per padded multiply-add the autotuner
//                measured for that shape in the product's size class).
enum PickMode : int { kPickModel = 0, kPickTable = 1, kPickCost = 2 };

struct TuneTable {
    int shape[2][kMB][kMB][kKB];  // [dtype: 0 double, 1 float]
    float cost[2][kMB][kMB][kKB][kNumShapes] = {};  // ns per padded multiply-add, 0 = not measured
    int mode[2] = {kPickModel, kPickModel};
    double tile_w[2] = {-1.0, -1.0};  // the model's per-tile weight (the autotuner's choice; -1: default)
    bool tuned_any = false;  // the autotuner ran (or a v2 table was loaded): save as v2
};

std::mutex g_tune_mu;
TuneTable g_tune;
bool g_tune_init = false;

// Default choice (no measurements): the shape with the least padded work, larger tiles on ties.
// tile_w < 0: the cost is the padded area plus 64 a tile (k left out); tile_w >= 0: the padded
// multiply-adds (area x k) plus tile_w multiply-adds' worth of overhead a tile.
int model_shape(int m, int n, int nshapes, int k = 1, double tile_w = -1.0) {
    int best = 0;
    double best_cost = 1e300;
    for (int s = 0; s < nshapes; ++s) {
        const double tr = shape_rows(s), tc = shape_cols(s);
        const double padded = std::ceil(m / tr) * tr * std::ceil(n / tc) * tc;
        const double tiles = std::ceil(m / tr) * std::ceil(n / tc);
        // a small per-tile overhead favours fewer, larger tiles when the padding is equal
        const double cost = tile_w < 0 ? padded + 64.0 * tiles : padded * double(std::max(k, 1)) + tile_w * tiles;
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = s;
        }
    }
    return best;
}

void tune_defaults() {
    if (g_tune_init) return;
    const int rep[kMB] = {6, 12, 24, 48, 96, 192};
    for (int d = 0; d < 2; ++d)
        for (int a = 0; a < kMB; ++a)
            for (int b = 0; b < kMB; ++b)
                for (int c = 0; c < kKB; ++c)
                    g_tune.shape[d][a][b][c] =
                        model_shape(rep[a], rep[b], d == 0 ? max_shape<double>() + 1 : max_shape<float>() + 1);
    g_tune_init = true;
}

int pick_shape(int dtype_idx, int m, int n, int k, int mode_override = -1) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_defaults();
    const int nshapes = dtype_idx == 0 ? max_shape<double>() + 1 : max_shape<float>() + 1;
    const int a = bucket_mn(m), b = bucket_mn(n), c = bucket_k(k);
    switch (mode_override >= 0 ? mode_override : g_tune.mode[dtype_idx]) {
        case kPickTable: return g_tune.shape[dtype_idx][a][b][c];
        case kPickCost: {
            int best = g_tune.shape[dtype_idx][a][b][c];
            double best_cost = 1e300;
            for (int s = 0; s < nshapes; ++s) {
                const float per = g_tune.cost[dtype_idx][a][b][c][s];
                if (per <= 0.f) continue;
                const double tr = shape_rows(s), tc = shape_cols(s);
                const double cost = std::ceil(m / tr) * tr * std::ceil(n / tc) * tc * double(per);
                if (cost < best_cost) {
                    best_cost = cost;
                    best = s;
                }
            }
            return best;
        }
        default: return model_shape(m, n, nshapes, k, g_tune.tile_w[dtype_idx]);
    }
}

}  // namespace

// ---- plan ----------------------------------------------------------------------------------
struct GroupedPlan {
    int elem = 8;
    int64_t count = 0;
    int64_t ntiles = 0;
    DevProblem* d_probs = nullptr;
    DevTile* d_tiles = nullptr;
    int* d_counter = nullptr;
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int grid = 0;
    double useful_flops = 0, padded_flops = 0;
};

namespace {

void plan_free(GroupedPlan* p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
    if (p->d_probs) cudaFree(p->d_probs);
    if (p->d_tiles) cudaFree(p->d_tiles);
    if (p->d_counter) cudaFree(p->d_counter);
    delete p;
}

// The device problem table and the flat tile list of a batch (longest tiles first).  Each
// product's shape depends only on its own (m, n, k) and the tuning state, so a product gets the same
// tiles — and the same result bits — whatever else is in the batch.
template <typename T>
int build_tables(const gb300_gemm_problem* probs, int64_t count, int force_shape, int policy,
                 std::vector<DevProblem>& hp, std::vector<DevTile>& ht, double& useful, double& padded,
                 std::string* err) {
    const int didx = sizeof(T) == 8 ? 0 : 1;
    hp.clear();
    ht.clear();
    hp.reserve(size_t(count));
    useful = padded = 0;
    for (int64_t q = 0; q < count; ++q) {
        const gb300_gemm_problem& x = probs[q];
        const bool rm = x.order == 101;
        if ((x.order != 101 && x.order != 102) || x.m < 0 || x.n < 0 || x.k < 0 || x.m > INT32_MAX ||
            x.n > INT32_MAX || x.k > INT32_MAX) {
            if (err) *err = "problem " + std::to_string(q) + ": invalid order or size";
            return GB300_ERR_INVALID_ARG;
        }
        const bool tA = x.transA != 111, tB = x.transB != 111;
        const int64_t minlda = std::max<int64_t>(1, rm ? (tA ? x.m : x.k) : (tA ? x.k : x.m));
        const int64_t minldb = std::max<int64_t>(1, rm ? (tB ? x.k : x.n) : (tB ? x.n : x.k));
        const int64_t minldc = std::max<int64_t>(1, rm ? x.n : x.m);
        if (x.lda < minlda || x.ldb < minldb || x.ldc < minldc) {
            if (err) *err = "problem " + std::to_string(q) + ": leading dimension too small";
            return GB300_ERR_INVALID_ARG;
        }
        DevProblem d;
        if (rm) {
            d.m = int(x.m); d.n = int(x.n); d.A = x.A; d.lda = x.lda; d.B = x.B; d.ldb = x.ldb;
            d.ta = tA; d.tb = tB;
        } else {
            d.m = int(x.n); d.n = int(x.m); d.A = x.B; d.lda = x.ldb; d.B = x.A; d.ldb = x.lda;
            d.ta = tB; d.tb = tA;
        }
        d.k = int(x.k);
        d.C = x.C;
        d.ldc = x.ldc;
        d.alpha = x.alpha;
        d.beta = x.beta;
        if (d.m == 0 || d.n == 0) continue;
        if (d.k == 0 || x.alpha == 0.0) d.k = 0;  // C = beta*C through the same kernel
        d.shape = force_shape >= 0 ? force_shape : pick_shape(didx, d.m, d.n, d.k, policy);
        const int tr = shape_rows(d.shape), tc = shape_cols(d.shape);
        const int mt = (d.m + tr - 1) / tr, nt = (d.n + tc - 1) / tc;
        const int pid = int(hp.size());
        hp.push_back(d);
        for (int a = 0; a < mt; ++a)
            for (int b = 0; b < nt; ++b) ht.push_back(DevTile{pid, a, b, 0});
        useful += 2.0 * d.m * d.n * d.k;
        padded += 2.0 * double(mt) * tr * double(nt) * tc * d.k;
    }
    // longest first: tiles ordered by their k times tile area (descending)
    std::stable_sort(ht.begin(), ht.end(), [&](const DevTile& a, const DevTile& b) {
        const DevProblem& pa = hp[a.prob];
        const DevProblem& pb = hp[b.prob];
        const double wa = double(pa.k) * shape_rows(pa.shape) * shape_cols(pa.shape);
        const double wb = double(pb.k) * shape_rows(pb.shape) * shape_cols(pb.shape);
        return wa > wb;
    });
    return GB300_OK;
}

// Dynamic shared memory of a block: the FP32 staging regions (none for FP64).
template <typename T>
int grouped_smem() {
    if constexpr (sizeof(T) == 4) {
        static const bool set = [] {
            return cudaFuncSetAttribute(grouped_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kStageBytes) == cudaSuccess;
        }();
        (void)set;
        return kStageBytes;
    }
    return 0;
}

// Persistent grid for `ntiles` warp tiles: every SM's resident blocks, or fewer for a short list.
template <typename T>
int grouped_grid(int64_t ntiles, int num_sms) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grouped_kernel<T>, 256, grouped_smem<T>());
    per_sm = std::max(per_sm, 1);
    return int(std::max<int64_t>(1, std::min<int64_t>(int64_t(num_sms) * per_sm, (ntiles + 7) / 8)));
}

template <typename T>
int plan_create(const gb300_gemm_problem* probs, int64_t count, int force_shape, GroupedPlan** out, std::string* err,
                int policy = -1) {
    Runtime& r = runtime();
    int st = ensure_init(err);
    if (st != GB300_OK) return st;
    std::vector<DevProblem> hp;
    std::vector<DevTile> ht;
    double useful = 0, padded = 0;
    st = build_tables<T>(probs, count, force_shape, policy, hp, ht, useful, padded, err);
    if (st != GB300_OK) return st;
    auto* p = new GroupedPlan();
    p->elem = sizeof(T);
    p->count = count;
    p->ntiles = int64_t(ht.size());
    p->useful_flops = useful;
    p->padded_flops = padded;
    cudaError_t e = cudaSuccess;
    if (!hp.empty()) {
        if ((e = cudaMalloc(&p->d_probs, hp.size() * sizeof(DevProblem))) != cudaSuccess ||
            (e = cudaMalloc(&p->d_tiles, ht.size() * sizeof(DevTile))) != cudaSuccess ||
            (e = cudaMemcpy(p->d_probs, hp.data(), hp.size() * sizeof(DevProblem), cudaMemcpyHostToDevice)) !=
                cudaSuccess ||
            (e = cudaMemcpy(p->d_tiles, ht.data(), ht.size() * sizeof(DevTile), cudaMemcpyHostToDevice)) != cudaSuccess) {
            plan_free(p);
            if (err) *err = std::string("grouped plan upload: ") + cudaGetErrorString(e);
            return GB300_ERR_NO_MEMORY;
        }
    }
    if ((e = cudaMalloc(&p->d_counter, sizeof(int))) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking)) != cudaSuccess) {
        plan_free(p);
        if (err) *err = std::string("grouped plan set-up: ") + cudaGetErrorString(e);
        return GB300_ERR_NO_MEMORY;
    }
    p->grid = grouped_grid<T>(p->ntiles, r.num_sms);
    // capture: counter reset + persistent kernel
    e = cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaMemsetAsync(p->d_counter, 0, sizeof(int), p->cap_stream);
        if (p->ntiles > 0)
            grouped_kernel<T><<<p->grid, 256, grouped_smem<T>(), p->cap_stream>>>(p->d_probs, p->d_tiles,
                                                                              int(p->ntiles), p->d_counter);
        e = cudaStreamEndCapture(p->cap_stream, &p->graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
    if (e != cudaSuccess) {
        plan_free(p);
        if (err) *err = std::string("grouped graph capture: ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    *out = p;
    return GB300_OK;
}

// ---- autotuner -----------------------------------------------------------------------------
// For every size class, time each candidate shape on a synthetic batch of that class (operands
// uniform [-1,1], sizes drawn inside the class) and keep the fastest; results can be saved to and
// loaded from a text cache ("gb300-grouped-tune v1" header, one class per line).
template <typename T>
int autotune(int didx, int effort, std::string* err) {
    const int rep_lo[kMB] = {4, 9, 17, 33, 65, 129};
    const int rep_hi[kMB] = {8, 16, 32, 64, 128, 256};
    const int k_lo[kKB] = {4, 17, 65}, k_hi[kKB] = {16, 64, 256};
    uint64_t rng = 0x9E3779B97F4A7C15ull;
    auto rnd = [&](int lo, int hi) {
        rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17;
        return lo + int(rng % uint64_t(hi - lo + 1));
    };
    // Each class is timed on a batch holding about `work` multiply-adds, so that a plan's run is
    // long against its launch: a batch of a few tiny products would time the launch, not the shape.
    const double work = 1.28e8 * std::max(1, effort) * (sizeof(T) == 4 ? 4.0 : 1.0);  // FP32 runs ~30x faster
    auto class_batch = [&](int a, int b, int c) {
        const double mean = 0.125 * double(rep_lo[a] + rep_hi[a]) * double(rep_lo[b] + rep_hi[b]) *
                            double(k_lo[c] + k_hi[c]);
        // (at most 16384 products: the plan's host-side set-up grows with the count)
        return int(std::max(64.0, std::min(16384.0, work / mean)));
    };
    auto footprint = [&](int a, int b, int c) {  // elements of A, B and C of one product, at most
        return size_t(rep_hi[a]) * k_hi[c] + size_t(k_hi[c]) * rep_hi[b] + size_t(rep_hi[a]) * rep_hi[b];
    };
    size_t pool = 0;
    for (int a = 0; a < kMB; ++a)
        for (int b = 0; b < kMB; ++b)
            for (int c = 0; c < kKB; ++c) pool = std::max(pool, size_t(class_batch(a, b, c)) * footprint(a, b, c));
    T* dP = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&dP, pool * sizeof(T))) != cudaSuccess) {
        if (err) *err = std::string("autotune buffers: ") + cudaGetErrorString(e);
        return GB300_ERR_NO_MEMORY;
    }
    cudaMemset(dP, 0, pool * sizeof(T));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int table[kMB][kMB][kKB];
    float costs[kMB][kMB][kKB][kNumShapes] = {};
    for (int a = 0; a < kMB; ++a)
        for (int b = 0; b < kMB; ++b)
            for (int c = 0; c < kKB; ++c) {
                const int batch = class_batch(a, b, c);
                std::vector<gb300_gemm_problem> ps(static_cast<size_t>(batch));
                size_t off = 0;
                for (int q = 0; q < batch; ++q) {
                    gb300_gemm_problem& x = ps[size_t(q)];
                    std::memset(&x, 0, sizeof(x));
                    x.order = 101; x.transA = 111; x.transB = 111;
                    x.m = rnd(rep_lo[a], rep_hi[a]); x.n = rnd(rep_lo[b], rep_hi[b]); x.k = rnd(k_lo[c], k_hi[c]);
                    x.alpha = 1.0; x.beta = 0.0;
                    x.A = dP + off; x.lda = x.k;
                    off += size_t(x.m) * size_t(x.k);
                    x.B = dP + off; x.ldb = x.n;
                    off += size_t(x.k) * size_t(x.n);
                    x.C = dP + off; x.ldc = x.n;
                    off += size_t(x.m) * size_t(x.n);
                }
                float best_ms = 1e30f;
                int best = 0;
                for (int s = 0; s <= max_shape<T>(); ++s) {
                    GroupedPlan* p = nullptr;
                    costs[a][b][c][s] = 0.f;
                    if (plan_create<T>(ps.data(), batch, s, &p, err) != GB300_OK) continue;
                    cudaGraphLaunch(p->exec, p->cap_stream);  // warm-up
                    cudaEventRecord(e0, p->cap_stream);
                    const int reps = 5;
                    for (int it = 0; it < reps; ++it) cudaGraphLaunch(p->exec, p->cap_stream);
                    cudaEventRecord(e1, p->cap_stream);
                    cudaEventSynchronize(e1);
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    count_launches(reps + 1);
                    // time per padded multiply-add (ns), the shape's efficiency in this class
                    if (p->padded_flops > 0) costs[a][b][c][s] = float(1e6 * ms / reps / (0.5 * p->padded_flops));
                    plan_free(p);
                    if (ms < best_ms) { best_ms = ms; best = s; }
                }
                table[a][b][c] = best;
            }
    cudaFree(dP);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        tune_defaults();
        std::memcpy(g_tune.shape[didx], table, sizeof(table));
        std::memcpy(g_tune.cost[didx], costs, sizeof(costs));
    }
    // Which way of picking shapes is faster on a mixed batch (m, n, k log-uniform over all classes):
    // the measured costs, or the least padded work alone (the better one where one pipe bounds
    // every shape alike, as the FP64 pipe does).
    const int vcount = 2048;
    std::vector<gb300_gemm_problem> vs(static_cast<size_t>(vcount));
    size_t vtotal = 0;
    auto logu = [&](int lo, int hi) {
        const double u = double(rnd(0, 1 << 20)) / double(1 << 20);
        return int(std::lround(std::exp(std::log(double(lo)) + u * (std::log(double(hi)) - std::log(double(lo))))));
    };
    for (auto& x : vs) {
        std::memset(&x, 0, sizeof(x));
        x.order = 101; x.transA = 111; x.transB = 111;
        x.m = logu(4, 256); x.n = logu(4, 256); x.k = logu(4, 256);
        x.alpha = 1.0; x.beta = 0.0;
        vtotal += size_t(x.m) * size_t(x.k) + size_t(x.k) * size_t(x.n) + size_t(x.m) * size_t(x.n);
    }
    int mode = kPickCost;
    double best_w = -1.0;
    T* dV = nullptr;
    if (cudaMalloc(&dV, vtotal * sizeof(T)) == cudaSuccess) {
        cudaMemset(dV, 0, vtotal * sizeof(T));
        size_t off = 0;
        for (auto& x : vs) {
            x.A = dV + off; x.lda = x.k; off += size_t(x.m) * size_t(x.k);
            x.B = dV + off; x.ldb = x.n; off += size_t(x.k) * size_t(x.n);
            x.C = dV + off; x.ldc = x.n; off += size_t(x.m) * size_t(x.n);
        }
        float best_ms = 1e30f;
        // candidates: the measured costs, and the model with per-tile weights from none to large
        const double weights[] = {-1.0, 0.0, 512.0, 2048.0, 8192.0};
        for (int cand = 0; cand < 6; ++cand) {
            const int pol = cand == 0 ? int(kPickCost) : int(kPickModel);
            const double w = cand == 0 ? -1.0 : weights[cand - 1];
            {
                std::lock_guard<std::mutex> lock(g_tune_mu);
                g_tune.tile_w[didx] = w;
            }
            GroupedPlan* p = nullptr;
            if (plan_create<T>(vs.data(), vcount, -1, &p, err, pol) != GB300_OK) continue;
            cudaGraphLaunch(p->exec, p->cap_stream);
            cudaEventRecord(e0, p->cap_stream);
            for (int it = 0; it < 5; ++it) cudaGraphLaunch(p->exec, p->cap_stream);
            cudaEventRecord(e1, p->cap_stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            count_launches(6);
            plan_free(p);
            if (ms < best_ms) {
                best_ms = ms;
                mode = pol;
                best_w = w;
            }
        }
        cudaFree(dV);
    } else {
        cudaGetLastError();
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune.mode[didx] = mode;
    g_tune.tile_w[didx] = mode == kPickModel ? best_w : -1.0;
    g_tune.tuned_any = true;
    return GB300_OK;
}

}  // namespace

// ---- lanes: grouped launches of the serving loop ---------------------------------------------
// A lane owns grow-only page-locked staging and device buffers for the problem table and tile
// list, so that a batch of small requests goes out as one plain launch (copies, counter reset,
// persistent kernel) on the lane's stream without allocating once the buffers have grown.  The
// caller waits for a lane's previous launch to finish before it launches on that lane again.
struct GroupedLane {
    cudaStream_t stream = nullptr;
    void* h_buf = nullptr;
    size_t h_bytes = 0;
    void* d_buf = nullptr;
    size_t d_bytes = 0;
    int* d_counter = nullptr;
    std::vector<void*> retired;  // outgrown staging buffers: cudaFreeHost would wait for the device
    std::vector<DevProblem> hp;
    std::vector<DevTile> ht;
};

GroupedLane* grouped_lane_create(cudaStream_t stream, std::string* err) {
    auto* l = new GroupedLane();
    l->stream = stream;
    if (cudaMalloc(&l->d_counter, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        if (err) *err = "grouped lane: counter allocation failed";
        delete l;
        return nullptr;
    }
    return l;
}

void grouped_lane_destroy(GroupedLane* l) {
    if (!l) return;
    if (l->d_buf) cudaFreeAsync(l->d_buf, l->stream);
    if (l->stream) cudaStreamSynchronize(l->stream);
    if (l->h_buf) cudaFreeHost(l->h_buf);
    for (void* h : l->retired) cudaFreeHost(h);
    if (l->d_counter) cudaFree(l->d_counter);
    delete l;
}

int grouped_lane_launch(GroupedLane* l, const gb300_gemm_problem* probs, int64_t count, double* useful_flops,
                        std::string* err) {
    double useful = 0, padded = 0;
    int st = build_tables<double>(probs, count, -1, -1, l->hp, l->ht, useful, padded, err);
    if (st != GB300_OK) return st;
    if (useful_flops) *useful_flops = useful;
    if (l->ht.empty()) return GB300_OK;
    const size_t pb = l->hp.size() * sizeof(DevProblem), tb = l->ht.size() * sizeof(DevTile);
    const size_t off_t = (pb + 255) / 256 * 256, need = off_t + tb;
    auto grow = [](size_t n) { return (n + (size_t(1) << 20) - 1) & ~((size_t(1) << 20) - 1); };
    if (l->h_bytes < need) {
        if (l->h_buf) l->retired.push_back(l->h_buf);
        l->h_buf = nullptr;
        l->h_bytes = 0;
        if (cudaHostAlloc(&l->h_buf, grow(need), cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            if (err) *err = "grouped lane: staging allocation failed";
            return GB300_ERR_NO_MEMORY;
        }
        l->h_bytes = grow(need);
    }
    if (l->d_bytes < need) {
        // stream-ordered on the lane's stream: growing the table never waits for other streams
        if (l->d_buf) cudaFreeAsync(l->d_buf, l->stream);
        l->d_buf = nullptr;
        l->d_bytes = 0;
        if (cudaMallocAsync(&l->d_buf, grow(need), l->stream) != cudaSuccess) {
            cudaGetLastError();
            if (err) *err = "grouped lane: table allocation failed";
            return GB300_ERR_NO_MEMORY;
        }
        l->d_bytes = grow(need);
    }
    auto* h = static_cast<uint8_t*>(l->h_buf);
    std::memcpy(h, l->hp.data(), pb);
    std::memcpy(h + off_t, l->ht.data(), tb);
    auto* d = static_cast<uint8_t*>(l->d_buf);
    cudaError_t e = cudaMemcpyAsync(d, h, need, cudaMemcpyHostToDevice, l->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(l->d_counter, 0, sizeof(int), l->stream);
    if (e == cudaSuccess) {
        const int grid = grouped_grid<double>(int64_t(l->ht.size()), runtime().num_sms);
        grouped_kernel<double><<<grid, 256, 0, l->stream>>>(reinterpret_cast<const DevProblem*>(d),
                                                            reinterpret_cast<const DevTile*>(d + off_t),
                                                            int(l->ht.size()), l->d_counter);
        count_launches(1);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        if (err) *err = std::string("grouped lane launch: ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    return GB300_OK;
}

}  // namespace gb

// ============================================================================================
//  C-ABI
// ============================================================================================
extern "C" {

int gb300_grouped_plan_create(int elem_bytes, const gb300_gemm_problem* problems, int64_t count,
                              gb300_grouped_plan** plan) {
    if (!plan || (count > 0 && !problems) || count < 0 || (elem_bytes != 8 && elem_bytes != 4)) {
        gb::set_error(GB300_ERR_INVALID_ARG, "gb300_grouped_plan_create: invalid arguments");
        return GB300_ERR_INVALID_ARG;
    }
    gb::Runtime& r = gb::runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    std::string err;
    gb::GroupedPlan* p = nullptr;
    const int st = elem_bytes == 8 ? gb::plan_create<double>(problems, count, -1, &p, &err)
                                   : gb::plan_create<float>(problems, count, -1, &p, &err);
    if (st != GB300_OK) {
        gb::set_error(st, "gb300_grouped_plan_create: " + err);
        return st;
    }
    *plan = reinterpret_cast<gb300_grouped_plan*>(p);
    gb::clear_error();
    return GB300_OK;
}

int gb300_grouped_plan_run(gb300_grouped_plan* plan, void* stream) {
    auto* p = reinterpret_cast<gb::GroupedPlan*>(plan);
    if (!p) {
        gb::set_error(GB300_ERR_INVALID_ARG, "gb300_grouped_plan_run: null plan");
        return GB300_ERR_INVALID_ARG;
    }
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : gb::runtime().stream;
    const cudaError_t e = cudaGraphLaunch(p->exec, s);
    if (e != cudaSuccess) {
        gb::set_error(GB300_ERR_CUDA, std::string("gb300_grouped_plan_run: ") + cudaGetErrorString(e));
        return GB300_ERR_CUDA;
    }
    gb::count_launches(p->ntiles > 0 ? 1 : 0);
    return GB300_OK;
}

int gb300_grouped_plan_info(const gb300_grouped_plan* plan, int64_t* tiles, double* useful_flops,
                            double* padded_flops) {
    auto* p = reinterpret_cast<const gb::GroupedPlan*>(plan);
    if (!p) return GB300_ERR_INVALID_ARG;
    if (tiles) *tiles = p->ntiles;
    if (useful_flops) *useful_flops = p->useful_flops;
    if (padded_flops) *padded_flops = p->padded_flops;
    return GB300_OK;
}

void gb300_grouped_plan_destroy(gb300_grouped_plan* plan) {
    gb::Runtime& r = gb::runtime();
    std::lock_guard<std::mutex> lock(r.mu);
    gb::plan_free(reinterpret_cast<gb::GroupedPlan*>(plan));
}

int gb300_dgemm_grouped(const gb300_gemm_problem* problems, int64_t count, void* stream) {
    gb300_grouped_plan* p = nullptr;
    int st = gb300_grouped_plan_create(8, problems, count, &p);
    if (st != GB300_OK) return st;
    st = gb300_grouped_plan_run(p, stream);
    if (st == GB300_OK) {
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : gb::runtime().stream;
        if (cudaStreamSynchronize(s) != cudaSuccess) st = GB300_ERR_CUDA;
    }
    gb300_grouped_plan_destroy(p);
    return st;
}

int gb300_sgemm_grouped(const gb300_gemm_problem* problems, int64_t count, void* stream) {
    gb300_grouped_plan* p = nullptr;
    int st = gb300_grouped_plan_create(4, problems, count, &p);
    if (st != GB300_OK) return st;
    st = gb300_grouped_plan_run(p, stream);
    if (st == GB300_OK) {
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : gb::runtime().stream;
        if (cudaStreamSynchronize(s) != cudaSuccess) st = GB300_ERR_CUDA;
    }
    gb300_grouped_plan_destroy(p);
    return st;
}

int gb300_grouped_autotune(int elem_bytes, int effort) {
    if (elem_bytes != 8 && elem_bytes != 4) {
        gb::set_error(GB300_ERR_INVALID_ARG, "gb300_grouped_autotune: elem_bytes must be 8 or 4");
        return GB300_ERR_INVALID_ARG;
    }
    gb::Runtime& r = gb::runtime();
    std::string err;
    int st;
    {
        std::lock_guard<std::mutex> lock(r.mu);
        st = gb::ensure_init(&err);
        if (st == GB300_OK)
            st = elem_bytes == 8 ? gb::autotune<double>(0, effort, &err) : gb::autotune<float>(1, effort, &err);
    }
    if (st != GB300_OK) gb::set_error(st, "gb300_grouped_autotune: " + err);
    return st;
}

// Tuning files: "gb300-grouped-tune v1" then one line per class, `dtype m-class n-class k-class
// shape`; an autotuned table is saved as "gb300-grouped-tune v2", each line followed by the measured
// ns per padded multiply-add of every shape (0: not measured).  Loading v1 makes plans use the
// class shapes, loading v2 the measured costs.
int gb300_grouped_tuning_save(const char* path) {
    std::lock_guard<std::mutex> lock(gb::g_tune_mu);
    gb::tune_defaults();
    std::ofstream f(path);
    if (!f) {
        gb::set_error(GB300_ERR_INVALID_ARG, std::string("gb300_grouped_tuning_save: cannot write ") + path);
        return GB300_ERR_INVALID_ARG;
    }
    // untuned defaults and loaded class tables save as v1; an autotuned table as v2 with its costs
    // and the policy the autotuner chose ("mode <double> <float>")
    const bool costs = gb::g_tune.mode[0] == gb::kPickCost || gb::g_tune.mode[1] == gb::kPickCost ||
                       gb::g_tune.tuned_any;
    f << (costs ? "gb300-grouped-tune v2\n" : "gb300-grouped-tune v1\n");
    if (costs)
        f << "mode " << gb::g_tune.mode[0] << ' ' << gb::g_tune.mode[1] << ' ' << gb::g_tune.tile_w[0] << ' '
          << gb::g_tune.tile_w[1] << '\n';
    for (int d = 0; d < 2; ++d)
        for (int a = 0; a < gb::kMB; ++a)
            for (int b = 0; b < gb::kMB; ++b)
                for (int c = 0; c < gb::kKB; ++c) {
                    f << d << ' ' << a << ' ' << b << ' ' << c << ' ' << gb::g_tune.shape[d][a][b][c];
                    if (costs)
                        for (int s = 0; s < gb::kNumShapes; ++s) f << ' ' << gb::g_tune.cost[d][a][b][c][s];
                    f << '\n';
                }
    return GB300_OK;
}

int gb300_grouped_tuning_load(const char* path) {
    std::ifstream f(path);
    std::string head;
    const bool ok_head = f && std::getline(f, head) && (head == "gb300-grouped-tune v1" || head == "gb300-grouped-tune v2");
    if (!ok_head) {
        gb::set_error(GB300_ERR_INVALID_ARG, std::string("gb300_grouped_tuning_load: not a tuning file: ") + path);
        return GB300_ERR_INVALID_ARG;
    }
    const bool v2 = head == "gb300-grouped-tune v2";
    // parse everything first: a malformed file leaves the table as it was
    gb::TuneTable t;
    {
        std::lock_guard<std::mutex> lock(gb::g_tune_mu);
        gb::tune_defaults();
        t = gb::g_tune;
    }
    std::string line;
    int modes[2] = {gb::kPickCost, gb::kPickCost};
    while (std::getline(f, line)) {
        if (line.empty()) continue;
        if (v2 && line.rfind("mode ", 0) == 0) {
            std::istringstream ms(line.substr(5));
            if (!(ms >> modes[0] >> modes[1]) || modes[0] < 0 || modes[0] > 2 || modes[1] < 0 || modes[1] > 2) {
                gb::set_error(GB300_ERR_INVALID_ARG, "gb300_grouped_tuning_load: bad mode line");
                return GB300_ERR_INVALID_ARG;
            }
            double w0 = -1.0, w1 = -1.0;
            if (ms >> w0 >> w1) {  // the model's per-tile weights (absent in older v2 files)
                t.tile_w[0] = w0;
                t.tile_w[1] = w1;
            }
            continue;
        }
        std::istringstream ls(line);
        int d, a, b, c, s;
        if (!(ls >> d >> a >> b >> c >> s) || d < 0 || d > 1 || a < 0 || a >= gb::kMB || b < 0 || b >= gb::kMB ||
            c < 0 || c >= gb::kKB || s < 0 || s > (d == 0 ? gb::max_shape<double>() : gb::max_shape<float>())) {
            gb::set_error(GB300_ERR_INVALID_ARG, "gb300_grouped_tuning_load: bad entry");
            return GB300_ERR_INVALID_ARG;
        }
        t.shape[d][a][b][c] = s;
        if (v2)
            for (int q = 0; q < gb::kNumShapes; ++q) {
                float v = 0.f;
                if (!(ls >> v) || !(v >= 0.f)) {
                    gb::set_error(GB300_ERR_INVALID_ARG, "gb300_grouped_tuning_load: bad cost");
                    return GB300_ERR_INVALID_ARG;
                }
                t.cost[d][a][b][c][q] = v;
            }
    }
    t.mode[0] = v2 ? modes[0] : gb::kPickTable;
    t.mode[1] = v2 ? modes[1] : gb::kPickTable;
    t.tuned_any = v2;
    std::lock_guard<std::mutex> lock(gb::g_tune_mu);
    gb::g_tune = t;
    return GB300_OK;
}

int gb300_grouped_shape_for(int elem_bytes, int64_t m, int64_t n, int64_t k, int* rows, int* cols) {
    const int s = gb::pick_shape(elem_bytes == 8 ? 0 : 1, int(std::min<int64_t>(m, INT32_MAX)),
                                 int(std::min<int64_t>(n, INT32_MAX)), int(std::min<int64_t>(k, INT32_MAX)));
    if (rows) *rows = gb::shape_rows(s);
    if (cols) *cols = gb::shape_cols(s);
    return s;
}

}  // extern "C"
