// native_gemm.cu — K1: native FP64 (DFMA) and FP32 (FFMA) GEMM for sm_103a.
//
// Replaces the CBLAS dgemm/sgemm that Blaze's BLAS path calls (blaze/math/blas/cblas/gemm.h:116-162,
// reached from DMatDMatMultExpr.h:2021-2037 and its three storage-order siblings), i.e. the work
// that Blaze's own large kernel `mmm` (blaze/math/dense/MMM.h:105-600) does on the CPU.
//
// Design (one CTA per 128x128 tile of C — 256x64 when C has at most 64 columns, 64x256 when it has
// at most 64 rows —, 256 threads, 8x8 outputs per thread):
//   * operand tiles are staged in shared memory by TMA (cp.async.bulk.tensor) as 128-byte
//     swizzled boxes, a 4-deep mbarrier pipeline (one "full" barrier with transaction bytes and
//     one "empty" barrier released by the eight warps per stage);
//   * each k-panel is 128 bytes deep (16 doubles / 32 floats): a K-contiguous operand arrives as
//     one 128-row box, an M- or N-contiguous operand as 128-byte-wide boxes of k-rows;
//   * thread (tx,ty) owns rows ty+16r and columns tx+16c, so a warp's B reads are 16 consecutive
//     elements (conflict-free) and its A reads are two broadcast addresses in different banks
//     thanks to the swizzle;
//   * out-of-range parts of edge tiles are zero-filled by TMA, so only the epilogue checks bounds;
//   * optional split-k writes unscaled partial tiles to a workspace that a second kernel reduces
//     in a fixed order (deterministic), then applies alpha and beta.
// beta == 0 never reads C (CBLAS semantics; NaN in C does not propagate).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/gb300_blas.h"

#include "gb300_internal.h"
#include "ptx.cuh"
#include "profile.h"
#include "runtime.h"

namespace gb {
namespace {

constexpr int STAGES = 4;
constexpr int THREADS = 256;
constexpr int PANEL_BYTES = 128;                         // k-panel depth in bytes

// Tile geometry for a tile of BN_ columns: BM = 16384 / BN rows, so that the 256 threads keep
// 8 x 8 outputs each; thread (tx, ty) owns rows ty + TY r and columns tx + TX c.
template <int BN_>
struct NativeTile {
    static constexpr int BN = BN_;
    static constexpr int BM = 16384 / BN_;
    static constexpr int TX = BN_ / 8, TY = THREADS / TX;
    static constexpr int A_BYTES = BM * PANEL_BYTES;     // per stage
    static constexpr int B_BYTES = BN * PANEL_BYTES;
    static constexpr size_t SMEM = size_t(STAGES) * (A_BYTES + B_BYTES) + 2 * STAGES * 8 + 1024;
};

template <typename T>
struct NativeParams {
    int64_t m, n, k;
    int64_t k_per_split;     // multiple of the panel depth
    T alpha, beta;
    T* C;
    int64_t ldc;
    T* ws;                   // split-k partials (splits x m x n) or nullptr
    int* status;
    uint64_t limit_ns;
    int inject_stall;
};

struct __align__(8) NativeBarriers {
    uint64_t full[STAGES];
    uint64_t empty[STAGES];
};

// Shared-memory byte offset of A(m, kk) / B(kk, n) inside one stage's operand tile.
template <typename T, bool TRANS_A>
__device__ __forceinline__ uint32_t a_off(int m, int kk) {
    constexpr int BK = PANEL_BYTES / sizeof(T);
    constexpr int E = PANEL_BYTES / sizeof(T);            // elements per 128-byte row
    if (!TRANS_A) return swz128(uint32_t(m * PANEL_BYTES + kk * sizeof(T)));
    return uint32_t((m / E) * BK * PANEL_BYTES) + swz128(uint32_t(kk * PANEL_BYTES + (m % E) * sizeof(T)));
}

template <typename T, bool TRANS_B>
__device__ __forceinline__ uint32_t b_off(int kk, int n) {
    constexpr int BK = PANEL_BYTES / sizeof(T);
    constexpr int E = PANEL_BYTES / sizeof(T);
    if (TRANS_B) return swz128(uint32_t(n * PANEL_BYTES + kk * sizeof(T)));
    return uint32_t((n / E) * BK * PANEL_BYTES) + swz128(uint32_t(kk * PANEL_BYTES + (n % E) * sizeof(T)));
}

template <typename T, bool TRANS_A, bool TRANS_B, int BN_>
__global__ void __launch_bounds__(THREADS, 1)
native_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const NativeParams<T> p) {
    using Tile = NativeTile<BN_>;
    constexpr int BM = Tile::BM, BN = Tile::BN, TX = Tile::TX, TY = Tile::TY;
    constexpr int BK = PANEL_BYTES / sizeof(T);
    constexpr int E = PANEL_BYTES / sizeof(T);
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte alignment for the swizzle atoms
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* tilesA = smem;
    uint8_t* tilesB = smem + STAGES * Tile::A_BYTES;
    NativeBarriers* bars = reinterpret_cast<NativeBarriers*>(smem + STAGES * (Tile::A_BYTES + Tile::B_BYTES));

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int tx = tid % TX, ty = tid / TX;
    // Float with an n-contiguous B: thread tx owns the 8 consecutive columns 8 tx .. 8 tx + 7, read as
    // two 16-byte swizzle chunks; B's 32-column boxes lie 4 KB apart, on the same banks, so threads
    // in odd boxes read their upper chunk first (their columns rotated by four) and one load
    // instruction spreads over all eight chunk positions.  Otherwise columns tx + TX c.
    constexpr bool VB = sizeof(T) == 4 && !TRANS_B;
    const int vbh = VB ? ((tx * 8 / E) & 1) : 0;
    auto col_of = [&](int c) { return VB ? tx * 8 + ((c + 4 * vbh) & 7) : tx + TX * c; };
    // The same for the rows of a float m-contiguous A: thread ty owns rows 8 ty .. 8 ty + 7.
    constexpr bool VA = sizeof(T) == 4 && TRANS_A;
    const int vah = VA ? ((ty * 8 / E) & 1) : 0;
    auto row_of = [&](int r) { return VA ? ty * 8 + ((r + 4 * vah) & 7) : ty + TY * r; };
    const int64_t m0 = int64_t(blockIdx.y) * BM;
    const int64_t n0 = int64_t(blockIdx.x) * BN;
    const int64_t kbeg = int64_t(blockIdx.z) * p.k_per_split;
    const int64_t kend = min(p.k, kbeg + p.k_per_split);
    const int KT = kend > kbeg ? int((kend - kbeg + BK - 1) / BK) : 0;

    if (tid == 0) {
        tma_prefetch_desc(&tmA);
        tma_prefetch_desc(&tmB);
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(smem_u32(&bars->full[s]), 1);
            mbar_init(smem_u32(&bars->empty[s]), THREADS / 32);
        }
        fence_mbar_init();
    }
    __syncthreads();

    auto issue = [&](int t, int s) {
        const uint32_t full = smem_u32(&bars->full[s]);
        mbar_arrive_expect_tx(full, Tile::A_BYTES + Tile::B_BYTES);
        const int32_t kx = int32_t(kbeg + int64_t(t) * BK);
        const uint32_t dA = smem_u32(tilesA + s * Tile::A_BYTES);
        const uint32_t dB = smem_u32(tilesB + s * Tile::B_BYTES);
        if (!TRANS_A) {
            tma_load_2d(dA, &tmA, kx, int32_t(m0), full);
        } else {
#pragma unroll
            for (int b = 0; b < BM / E; ++b)
                tma_load_2d(dA + b * BK * PANEL_BYTES, &tmA, int32_t(m0 + b * E), kx, full);
        }
        if (TRANS_B) {
            tma_load_2d(dB, &tmB, kx, int32_t(n0), full);
        } else {
#pragma unroll
            for (int b = 0; b < BN / E; ++b)
                tma_load_2d(dB + b * BK * PANEL_BYTES, &tmB, int32_t(n0 + b * E), kx, full);
        }
    };

    int issued = 0;
    if (tid == 0 && !p.inject_stall) {
        for (; issued < min(STAGES, KT); ++issued) issue(issued, issued);
    }

    T acc[8][8];
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[r][c] = T(0);

    bool ok = true;
    int kt = 0;
    for (; kt < KT; ++kt) {
        const int s = kt % STAGES;
        const uint32_t ph = (kt / STAGES) & 1;
        if (!mbar_wait(smem_u32(&bars->full[s]), ph, p.status, kDevTimeoutFull, p.limit_ns)) {
            ok = false;
            break;
        }
        const uint8_t* As = tilesA + s * Tile::A_BYTES;
        const uint8_t* Bs = tilesB + s * Tile::B_BYTES;
        if constexpr (sizeof(T) == 4 && !TRANS_A) {
            // float, k-contiguous A: four consecutive k of a row are one 16-byte swizzle chunk, so
            // one 128-bit load serves four k steps (a quarter of A's shared-memory wavefronts, the
            // FFMA form's limit); every output still accumulates k in order
#pragma unroll 2
            for (int k4 = 0; k4 < BK; k4 += 4) {
                float4 a4[8];
#pragma unroll
                for (int r = 0; r < 8; ++r) a4[r] = *reinterpret_cast<const float4*>(As + a_off<T, TRANS_A>(row_of(r), k4));
                // k-contiguous B: its four k steps of a column are one chunk as well
                float4 b4[TRANS_B ? 8 : 1];
                if constexpr (TRANS_B) {
#pragma unroll
                    for (int c = 0; c < 8; ++c) b4[c] = *reinterpret_cast<const float4*>(Bs + b_off<T, TRANS_B>(k4, col_of(c)));
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    T b[8];
                    if constexpr (TRANS_B) {
#pragma unroll
                        for (int c = 0; c < 8; ++c)
                            b[c] = j == 0 ? b4[c].x : j == 1 ? b4[c].y : j == 2 ? b4[c].z : b4[c].w;
                    } else if constexpr (VB) {
                        const float4 lo = *reinterpret_cast<const float4*>(Bs + b_off<T, TRANS_B>(k4 + j, tx * 8 + 4 * vbh));
                        const float4 hi =
                            *reinterpret_cast<const float4*>(Bs + b_off<T, TRANS_B>(k4 + j, tx * 8 + 4 * (1 - vbh)));
                        b[0] = lo.x; b[1] = lo.y; b[2] = lo.z; b[3] = lo.w;
                        b[4] = hi.x; b[5] = hi.y; b[6] = hi.z; b[7] = hi.w;
                    } else {
#pragma unroll
                        for (int c = 0; c < 8; ++c)
                            b[c] = *reinterpret_cast<const T*>(Bs + b_off<T, TRANS_B>(k4 + j, col_of(c)));
                    }
#pragma unroll
                    for (int r = 0; r < 8; ++r) {
                        const T a = j == 0 ? a4[r].x : j == 1 ? a4[r].y : j == 2 ? a4[r].z : a4[r].w;
#pragma unroll
                        for (int c = 0; c < 8; ++c) acc[r][c] = fma(a, b[c], acc[r][c]);
                    }
                }
            }
        } else if constexpr (VA && TRANS_B) {
            // float, m-contiguous A and k-contiguous B: A's rows as two chunks per k step, B's
            // four k steps of a column as one chunk
#pragma unroll 2
            for (int k4 = 0; k4 < BK; k4 += 4) {
                float4 b4[8];
#pragma unroll
                for (int c = 0; c < 8; ++c) b4[c] = *reinterpret_cast<const float4*>(Bs + b_off<T, TRANS_B>(k4, col_of(c)));
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float4 lo = *reinterpret_cast<const float4*>(As + a_off<T, TRANS_A>(ty * 8 + 4 * vah, k4 + j));
                    const float4 hi =
                        *reinterpret_cast<const float4*>(As + a_off<T, TRANS_A>(ty * 8 + 4 * (1 - vah), k4 + j));
                    const T a[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
                    for (int r = 0; r < 8; ++r)
#pragma unroll
                        for (int c = 0; c < 8; ++c) {
                            const T b = j == 0 ? b4[c].x : j == 1 ? b4[c].y : j == 2 ? b4[c].z : b4[c].w;
                            acc[r][c] = fma(a[r], b, acc[r][c]);
                        }
                }
            }
        } else {
#pragma unroll 4
            for (int kk = 0; kk < BK; ++kk) {
                T a[8], b[8];
                if constexpr (VA) {
                    const float4 lo = *reinterpret_cast<const float4*>(As + a_off<T, TRANS_A>(ty * 8 + 4 * vah, kk));
                    const float4 hi = *reinterpret_cast<const float4*>(As + a_off<T, TRANS_A>(ty * 8 + 4 * (1 - vah), kk));
                    a[0] = lo.x; a[1] = lo.y; a[2] = lo.z; a[3] = lo.w;
                    a[4] = hi.x; a[5] = hi.y; a[6] = hi.z; a[7] = hi.w;
                } else {
#pragma unroll
                    for (int r = 0; r < 8; ++r) a[r] = *reinterpret_cast<const T*>(As + a_off<T, TRANS_A>(row_of(r), kk));
                }
                if constexpr (VB) {
                    const float4 lo = *reinterpret_cast<const float4*>(Bs + b_off<T, TRANS_B>(kk, tx * 8 + 4 * vbh));
                    const float4 hi = *reinterpret_cast<const float4*>(Bs + b_off<T, TRANS_B>(kk, tx * 8 + 4 * (1 - vbh)));
                    b[0] = lo.x; b[1] = lo.y; b[2] = lo.z; b[3] = lo.w;
                    b[4] = hi.x; b[5] = hi.y; b[6] = hi.z; b[7] = hi.w;
                } else {
#pragma unroll
                    for (int c = 0; c < 8; ++c) b[c] = *reinterpret_cast<const T*>(Bs + b_off<T, TRANS_B>(kk, col_of(c)));
                }
#pragma unroll
                for (int r = 0; r < 8; ++r)
#pragma unroll
                    for (int c = 0; c < 8; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&bars->empty[s]));
        if (tid == 0 && issued < KT) {
            // the stage is refilled once all eight warps have released it
            if (!mbar_wait(smem_u32(&bars->empty[s]), ph, p.status, kDevTimeoutEmpty, p.limit_ns)) {
                ok = false;
                ++kt;
                break;
            }
            issue(issued, s);
            ++issued;
        }
    }

    if (!ok) {
        // drain the copies this CTA issued but did not consume, with the same bounded wait
        if (tid == 0) {
            for (int t = kt; t < issued; ++t)
                mbar_wait_drain(smem_u32(&bars->full[t % STAGES]), (t / STAGES) & 1, p.limit_ns);
        }
        return;
    }

    // epilogue
    if (p.ws != nullptr) {
        T* w = p.ws + int64_t(blockIdx.z) * p.m * p.n;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int64_t i = m0 + row_of(r);
            if (i >= p.m) continue;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int64_t j = n0 + col_of(c);
                if (j < p.n) w[i * p.n + j] = acc[r][c];
            }
        }
        return;
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int64_t i = m0 + row_of(r);
        if (i >= p.m) continue;
        T* crow = p.C + i * p.ldc;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int64_t j = n0 + col_of(c);
            if (j >= p.n) continue;
            const T v = p.alpha * acc[r][c];
            crow[j] = (p.beta == T(0)) ? v : fma(p.beta, crow[j], v);
        }
    }
}

// Fixed-order reduction of split-k partials: C = alpha * sum_z W[z] + beta * C.
template <typename T>
__global__ void splitk_reduce_kernel(const T* __restrict__ ws, int splits, int64_t m, int64_t n, T alpha,
                                     T beta, T* __restrict__ C, int64_t ldc) {
    const int64_t total = m * n;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
         e += int64_t(gridDim.x) * blockDim.x) {
        T s = ws[e];
        for (int z = 1; z < splits; ++z) s += ws[int64_t(z) * total + e];
        const int64_t i = e / n, j = e % n;
        T* c = C + i * ldc + j;
        const T v = alpha * s;
        *c = (beta == T(0)) ? v : fma(beta, *c, v);
    }
}

// C = beta * C (k == 0); beta == 0 writes zeros without reading C.
template <typename T>
__global__ void scale_c_kernel(int64_t m, int64_t n, T beta, T* __restrict__ C, int64_t ldc) {
    const int64_t total = m * n;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
         e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i = e / n, j = e % n;
        T* c = C + i * ldc + j;
        *c = (beta == T(0)) ? T(0) : beta * *c;
    }
}

template <typename T>
constexpr CUtensorMapDataType tmap_type() {
    return sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
}

template <typename T, bool TA, bool TB, int BN_>
cudaError_t launch_variant(const CUtensorMap& a, const CUtensorMap& b, const NativeParams<T>& p, dim3 grid,
                           cudaStream_t s) {
    auto kern = native_gemm_kernel<T, TA, TB, BN_>;
    constexpr int smem = int(NativeTile<BN_>::SMEM);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    {
        KernelTimer timer("native_gemm", s);
        kern<<<grid, THREADS, smem, s>>>(a, b, p);
    }
    count_launches(1);
    return cudaGetLastError();
}

// Columns of the CTA tile: 64 (256 x 64 tiles) for products with at most 64 columns and 256
// (64 x 256 tiles) for products with at most 64 rows, where a 128 x 128 tile would compute half of
// its outputs on padding; else 128.
int native_tile_n(int64_t m, int64_t n) { return n <= 64 ? 64 : (m <= 64 ? 256 : 128); }

template <typename T, int BN_>
cudaError_t native_gemm_tiled(const Gemm& g, int splits, T* workspace, const LaunchCtl& ctl, cudaStream_t s,
                              std::string* err) {
    using Tile = NativeTile<BN_>;
    constexpr int BM = Tile::BM, BN = Tile::BN;
    const int64_t BK = PANEL_BYTES / sizeof(T);
    const int E = PANEL_BYTES / sizeof(T);
    CUtensorMap ta, tb;
    const CUtensorMapDataType dt = tmap_type<T>();
    // A: rows x cols as stored (row-major storage, ld = lda)
    bool ok;
    if (!g.ta)
        ok = encode_tmap_2d(&ta, dt, sizeof(T), g.A, g.m, g.k, g.lda, BM, BK, CU_TENSOR_MAP_SWIZZLE_128B, err);
    else
        ok = encode_tmap_2d(&ta, dt, sizeof(T), g.A, g.k, g.m, g.lda, BK, E, CU_TENSOR_MAP_SWIZZLE_128B, err);
    if (!ok) return cudaErrorInvalidValue;
    if (g.tb)
        ok = encode_tmap_2d(&tb, dt, sizeof(T), g.B, g.n, g.k, g.ldb, BN, BK, CU_TENSOR_MAP_SWIZZLE_128B, err);
    else
        ok = encode_tmap_2d(&tb, dt, sizeof(T), g.B, g.k, g.n, g.ldb, BK, E, CU_TENSOR_MAP_SWIZZLE_128B, err);
    if (!ok) return cudaErrorInvalidValue;

    splits = std::max(1, splits);
    int64_t kps = (g.k + splits - 1) / splits;
    kps = (kps + BK - 1) / BK * BK;
    splits = int((g.k + kps - 1) / kps);

    NativeParams<T> p;
    p.m = g.m; p.n = g.n; p.k = g.k;
    p.k_per_split = kps;
    p.alpha = T(g.alpha); p.beta = T(g.beta);
    p.C = static_cast<T*>(g.C); p.ldc = g.ldc;
    p.ws = splits > 1 ? workspace : nullptr;
    p.status = ctl.status;
    p.limit_ns = ctl.wait_limit_ns;
    p.inject_stall = ctl.inject_stall;
    if (splits > 1 && workspace == nullptr) {
        if (err) *err = "split-k needs a workspace";
        return cudaErrorInvalidValue;
    }
    dim3 grid(unsigned((g.n + BN - 1) / BN), unsigned((g.m + BM - 1) / BM), unsigned(splits));
    cudaError_t e;
    if (!g.ta && !g.tb) e = launch_variant<T, false, false, BN_>(ta, tb, p, grid, s);
    else if (!g.ta && g.tb) e = launch_variant<T, false, true, BN_>(ta, tb, p, grid, s);
    else if (g.ta && !g.tb) e = launch_variant<T, true, false, BN_>(ta, tb, p, grid, s);
    else e = launch_variant<T, true, true, BN_>(ta, tb, p, grid, s);
    if (e != cudaSuccess || splits == 1) return e;
    const int64_t total = g.m * g.n;
    const int blocks = int(std::min<int64_t>((total + 255) / 256, 152 * 16));
    splitk_reduce_kernel<T><<<blocks, 256, 0, s>>>(workspace, splits, g.m, g.n, T(g.alpha), T(g.beta),
                                                   static_cast<T*>(g.C), g.ldc);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace

int native_choose_splits(int64_t m, int64_t n, int64_t k, int elem_bytes, int num_sms) {
    const int64_t bk = PANEL_BYTES / elem_bytes;
    const int64_t bn = native_tile_n(m, n), bm = 16384 / bn;
    const int64_t tiles = ((m + bm - 1) / bm) * ((n + bn - 1) / bn);
    if (2 * tiles > num_sms || k < 32 * bk) return 1;
    // as many k-splits as still fit one wave of CTAs (one CTA per SM), each at least 16 panels deep
    // (four times the stage ring, so that filling the ring stays a small part of a split): a split
    // count that spills a few CTAs into a second wave doubles the time
    int64_t splits = num_sms / tiles;
    splits = std::min<int64_t>(splits, k / (16 * bk));
    return int(std::max<int64_t>(splits, 1));
}

template <typename T>
cudaError_t native_gemm(const Gemm& g, int splits, T* workspace, const LaunchCtl& ctl, cudaStream_t s,
                        std::string* err) {
    if (g.m <= 0 || g.n <= 0) return cudaSuccess;
    if (g.k == 0) {
        const int64_t total = g.m * g.n;
        const int blocks = int(std::min<int64_t>((total + 255) / 256, 4096));
        scale_c_kernel<T><<<blocks, 256, 0, s>>>(g.m, g.n, T(g.beta), static_cast<T*>(g.C), g.ldc);
        count_launches(1);
        return cudaGetLastError();
    }
    switch (native_tile_n(g.m, g.n)) {
        case 64: return native_gemm_tiled<T, 64>(g, splits, workspace, ctl, s, err);
        case 256: return native_gemm_tiled<T, 256>(g, splits, workspace, ctl, s, err);
        default: return native_gemm_tiled<T, 128>(g, splits, workspace, ctl, s, err);
    }
}

template cudaError_t native_gemm<double>(const Gemm&, int, double*, const LaunchCtl&, cudaStream_t, std::string*);
template cudaError_t native_gemm<float>(const Gemm&, int, float*, const LaunchCtl&, cudaStream_t, std::string*);

}  // namespace gb

// =============================================================================================
//  Allocation-free entry point (gb300_dgemm_native_noalloc)
// =============================================================================================
// Some callers must not allocate device memory on their own: a host framework that owns every
// byte of device memory through its own pool or budget, a latency-critical loop in which
// cudaMalloc/cudaFree (which can synchronize the device) is not allowed, or a plugin host that
// forbids allocations after start-up.  For them this entry point runs the native kernel with its
// split-k scratch taken from a fixed array compiled into the library instead of the device pool.
//
//   * The array is a file-scope static __device__ variable of kNoAllocScratchBytes (16 MiB).
//     Every GPU on which the library's device code is loaded holds it until the process exits.
//   * Its device address is looked up with cudaGetSymbolAddress on every call, with the call's
//     device current (a lookup, no allocation), so an address never outlives a context that a
//     cudaDeviceReset tore down.  The first call on a device also loads this file's device code
//     there; that first call should therefore come before any stream capture.  Host code must
//     never pass the symbol itself to a kernel: on the host it is only a stand-in, not a device
//     address.
//   * The first 256 bytes hold the kernel status word (cleared before every launch); the rest
//     holds split-k partial tiles, which the kernel writes in full before reading them.
//   * All calls share the array, so two calls whose kernels overlapped on the GPU would race on
//     it.  The entry point therefore serializes its callers with a process-wide lock and returns
//     only after its kernels have finished on `stream`, on the error paths too.
//   * Products whose split-k partials do not fit are rejected with GB300_ERR_INVALID_ARG before
//     anything is queued (C is left as it was); nothing is allocated, including by the CUDA
//     runtime calls made here.
//   * A, B, C and the stream must belong to the current device (managed memory is accepted).
namespace gb {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
constexpr size_t kNoAllocStatusBytes = 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;

// Device address of g_noalloc_scratch on the current device.
int noalloc_scratch(void** out, std::string* err) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        *err = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e);
        return GB300_ERR_CUDA;
    }
    *out = p;
    return GB300_OK;
}

// Whether p is device memory of device `dev`, or managed memory.
bool resident_on(const void* p, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace
}  // namespace gb

extern "C" int gb300_dgemm_native_noalloc(int order, int transA, int transB, int64_t m, int64_t n, int64_t k,
                                          double alpha, const double* A, int64_t lda, const double* B, int64_t ldb,
                                          double beta, double* C, int64_t ldc, void* stream) {
    using namespace gb;
    auto fail = [](int st, const std::string& msg) {
        set_error(st, "gb300_dgemm_native_noalloc: " + msg);
        return st;
    };
    if (order != 101 && order != 102) return fail(GB300_ERR_INVALID_ARG, "parameter 1 (order) is invalid");
    auto valid_trans = [](int t) { return t == 111 || t == 112 || t == 113; };
    if (!valid_trans(transA)) return fail(GB300_ERR_INVALID_ARG, "parameter 2 (transA) is invalid");
    if (!valid_trans(transB)) return fail(GB300_ERR_INVALID_ARG, "parameter 3 (transB) is invalid");
    if (m < 0 || n < 0 || k < 0) return fail(GB300_ERR_INVALID_ARG, "negative dimension");
    const bool tA = transA != 111, tB = transB != 111, rm = order == 101;
    if (lda < std::max<int64_t>(1, rm ? (tA ? m : k) : (tA ? k : m)))
        return fail(GB300_ERR_INVALID_ARG, "parameter 9 (lda) is too small");
    if (ldb < std::max<int64_t>(1, rm ? (tB ? k : n) : (tB ? n : k)))
        return fail(GB300_ERR_INVALID_ARG, "parameter 11 (ldb) is too small");
    if (ldc < std::max<int64_t>(1, rm ? n : m)) return fail(GB300_ERR_INVALID_ARG, "parameter 14 (ldc) is too small");
    clear_error();
    if (m == 0 || n == 0) return GB300_OK;
    if ((alpha == 0.0 || k == 0) && beta == 1.0) return GB300_OK;
    const bool product = alpha != 0.0 && k > 0;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return fail(GB300_ERR_NO_DEVICE, "no current device");
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (s != nullptr) {
        int sdev = -1;
        if (cudaStreamGetDevice(s, &sdev) != cudaSuccess) {
            cudaGetLastError();
            return fail(GB300_ERR_INVALID_ARG, "parameter 15 (stream) is not a valid stream");
        }
        if (sdev != dev)
            return fail(GB300_ERR_INVALID_ARG, "the stream belongs to device " + std::to_string(sdev) +
                                                   ", not the current device " + std::to_string(dev));
    }
    if (product && (!resident_on(A, dev) || !resident_on(B, dev)))
        return fail(GB300_ERR_INVALID_ARG, "A and B must be device memory of the current device (or managed memory)");
    if (!resident_on(C, dev))
        return fail(GB300_ERR_INVALID_ARG, "C must be device memory of the current device (or managed memory)");

    Gemm g;
    if (rm) {
        g.m = m; g.n = n; g.k = k; g.ta = tA; g.tb = tB;
        g.A = A; g.lda = lda; g.B = B; g.ldb = ldb;
    } else {
        g.m = n; g.n = m; g.k = k; g.ta = tB; g.tb = tA;
        g.A = B; g.lda = ldb; g.B = A; g.ldb = lda;
    }
    g.C = C; g.ldc = ldc;
    if (!product) g.k = 0;
    g.alpha = alpha;
    g.beta = beta;
    auto tma_ok = [](const void* p, int64_t ld) {
        return reinterpret_cast<uintptr_t>(p) % 16 == 0 && (ld * 8) % 16 == 0;
    };
    if (product && (!tma_ok(g.A, g.lda) || !tma_ok(g.B, g.ldb)))
        return fail(GB300_ERR_INVALID_ARG,
                    "A and B need 16-byte aligned bases and even leading dimensions (realigning them would "
                    "need device memory; use gb300_dgemm_ex)");

    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    std::string err;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        return fail(GB300_ERR_NO_DEVICE, "cannot query the SM count");
    }
    int splits = g.k > 0 ? native_choose_splits(g.m, g.n, g.k, 8, sms) : 1;
    const size_t need = splits > 1 ? size_t(splits) * size_t(g.m) * size_t(g.n) * sizeof(double) : 0;
    if (need > kNoAllocScratchBytes - kNoAllocStatusBytes)
        return fail(GB300_ERR_INVALID_ARG,
                    "the product needs " + std::to_string(need) + " bytes of split-k scratch; the allocation-free "
                    "entry point holds " + std::to_string(kNoAllocScratchBytes - kNoAllocStatusBytes) +
                    " (use gb300_dgemm_ex)");
    void* scratch = nullptr;
    int st = noalloc_scratch(&scratch, &err);
    if (st != GB300_OK) return fail(st, err);
    auto* status = static_cast<int*>(scratch);
    auto* ws = reinterpret_cast<double*>(static_cast<unsigned char*>(scratch) + kNoAllocStatusBytes);

    // the failure-detection test hook of the other entry points (gb300_debug_inject_stall)
    LaunchCtl ctl;
    ctl.status = status;
    {
        Runtime& r = runtime();
        std::lock_guard<std::mutex> hook(r.mu);
        if (r.inject_stall_count > 0) {
            --r.inject_stall_count;
            ctl.inject_stall = 1;
            ctl.wait_limit_ns = r.inject_limit_ns;
        }
    }
    // from here on work may be queued: every return waits for the stream first, so that no kernel
    // of this call still touches the shared array once the lock is released
    auto fail_after_queue = [&](int st_, const std::string& msg) {
        cudaStreamSynchronize(s);
        cudaGetLastError();
        return fail(st_, msg);
    };
    cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), s);
    if (e != cudaSuccess) return fail_after_queue(GB300_ERR_CUDA, std::string("status reset: ") + cudaGetErrorString(e));
    e = native_gemm<double>(g, splits, splits > 1 ? ws : nullptr, ctl, s, &err);
    if (e != cudaSuccess) return fail_after_queue(GB300_ERR_CUDA, err.empty() ? cudaGetErrorString(e) : err);
    int h = 0;
    e = cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return fail_after_queue(GB300_ERR_CUDA, std::string("kernel failed: ") + cudaGetErrorString(e));
    if (h != 0) return fail(GB300_ERR_DEVICE_TIMEOUT, "a device-side wait ran out (code " + std::to_string(h) + ")");
    return GB300_OK;
}
