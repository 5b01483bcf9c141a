// trsm.cu — kernels of the triangular solve ?trsm on Blaze's seam (blaze/math/blas/cblas/trsm.h):
// the scaling of the right-hand sides by alpha and the inverses of the triangle's diagonal blocks.
// The host side (api_next.cpp) solves recursively.  It halves the triangle, solves one half,
// updates the other half's right-hand sides with one product, and solves that half.  The products
// run through the library's real or complex product, so a double solve does nearly all of its
// work on the tensor cores.  A block of at most solve_block() rows is multiplied by its inverse from
// here.  That leaf product costs 2 nb / ka of the solve's own work.  The inverses are what makes
// the leaves products.  Using them changes the rounding from that of substitution: a leaf's error
// grows with the condition number of its diagonal block, as in other blocked GPU solvers.
//
// Matrices are in row-major storage (a column-major operand is the transpose of its storage; the
// host folds that into the side, the triangle and the transposition).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "cplx.cuh"
#include "gb300_internal.h"
#include "level23.h"
#include "runtime.h"

namespace gb {
namespace {

// X (rows x cols, pitch ld) = alpha X.
template <typename V>
__global__ void scale_kernel(int64_t rows, int64_t cols, V alpha, V* __restrict__ X, int64_t ld) {
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y)
        for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < cols; c += int64_t(gridDim.x) * blockDim.x)
            X[r * ld + c] = Ar<V>::mul(alpha, X[r * ld + c]);
}

// Inverse of every diagonal block of the triangular matrix op(SA).  SA is ka x ka in row-major
// storage with pitch lda, and op transposes it (trans) and conjugates it (conj).  Block b covers
// rows and columns [b nb, min(ka, (b + 1) nb)).  Its inverse is written densely to inv + b nb nb
// with pitch nb, zeros outside the triangle included.
//
// Each block is brought to lower-triangular form L'.  L' is the block itself when op(SA) is lower;
// when it is upper (`upper`), L' is the block with its rows and columns reversed.  L' is inverted
// by forward substitution, Y[r][c] = (delta_rc - sum_{j<r} L'[r][j] Y[j][c]) / L'[r][r].
// blockIdx.x picks a group of 32 columns c, one per lane, and blockIdx.y the block.  The loops are
// the same for every lane: Y[j][c] = 0 for j < c comes out of the recurrence itself, and a group
// starts at its first column r0.  So every L' element is one load broadcast to the warp.
//
// Row r's sum is split over the kInvWarps warps of the block (warp w takes j = r0 + w, + kInvWarps,
// ...), which shortens the dependent FMA chain that bounds the kernel kInvWarps-fold.  Warp 0 adds
// the partial sums in warp order (a fixed order), divides and publishes Y[r] in shared memory
// ([nb][32], conflict-free) before the next row starts.  A unit diagonal is not read.
constexpr int kInvWarps = 8;

template <typename V>
__global__ void __launch_bounds__(32 * kInvWarps) tri_inverse_kernel(int64_t ka, int nb, const V* __restrict__ SA,
                                                                     int64_t lda, int trans, int conj, int upper,
                                                                     int unit, V* __restrict__ inv) {
    extern __shared__ __align__(16) unsigned char tri_smem[];
    V* ycol = reinterpret_cast<V*>(tri_smem);  // [nb][32]
    V* part = ycol + int64_t(nb) * 32;          // [kInvWarps][32]
    using A = Ar<V>;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t b0 = int64_t(blockIdx.y) * nb;
    const int nbk = int(min(int64_t(nb), ka - b0));
    const int r0 = int(blockIdx.x) * 32;
    if (r0 >= nbk) return;
    const int c = r0 + lane;
    // L'[r][j] sits at P + r * sr + j * sj
    int64_t sr = trans ? 1 : lda, sj = trans ? lda : 1;
    const V* P = SA + b0 * lda + b0;
    if (upper) {
        P += int64_t(nbk - 1) * (lda + 1);
        sr = -sr;
        sj = -sj;
    }
    V* out = inv + int64_t(blockIdx.y) * nb * nb;
    // Y[r][c] lands at out[r][c], or at out[nbk-1-r][nbk-1-c] for a reversed (upper) block
    const int64_t o0 = upper ? int64_t(nbk - 1) * (nb + 1) : 0, orow = upper ? -int64_t(nb) : int64_t(nb),
                  ocol = upper ? -1 : 1;
    if (c < nbk)
        for (int r = warp; r < r0; r += kInvWarps) out[o0 + r * orow + c * ocol] = A::zero();
    for (int r = r0; r < nbk; ++r) {
        // this warp's share of the sum, two chains to overlap the loads
        V s0 = A::zero(), s1 = A::zero();
        int j = r0 + warp;
        const V* lp = P + r * sr + j * sj;
        const V* yp = ycol + (j - r0) * 32 + lane;
        const int64_t lstep = int64_t(kInvWarps) * sj;
        for (; j + kInvWarps < r; j += 2 * kInvWarps, lp += 2 * lstep, yp += 64 * kInvWarps) {
            const V l0 = conj ? A::conj(lp[0]) : lp[0];
            const V l1 = conj ? A::conj(lp[lstep]) : lp[lstep];
            s0 = A::fmadd(l0, yp[0], s0);
            s1 = A::fmadd(l1, yp[32 * kInvWarps], s1);
        }
        if (j < r) {
            const V l0 = conj ? A::conj(lp[0]) : lp[0];
            s0 = A::fmadd(l0, yp[0], s0);
        }
        part[warp * 32 + lane] = A::add(s0, s1);
        __syncthreads();
        if (warp == 0) {
            V sum = part[lane];
#pragma unroll
            for (int w = 1; w < kInvWarps; ++w) sum = A::add(sum, part[w * 32 + lane]);
            V acc = A::fnmadd(A::one(), sum, (r == c) ? A::one() : A::zero());  // delta_rc - sum
            if (!unit) {
                const V* dp = P + r * (sr + sj);
                acc = A::div(acc, conj ? A::conj(*dp) : *dp);
            }
            ycol[(r - r0) * 32 + lane] = acc;
            if (c < nbk) out[o0 + r * orow + c * ocol] = acc;
        }
        __syncthreads();
    }
}

}  // namespace

template <typename T, bool CPLX>
cudaError_t launch_scale(int64_t rows, int64_t cols, const T* alpha, T* X, int64_t ld, cudaStream_t st) {
    using V = typename std::conditional<CPLX, Cx<T>, T>::type;
    V al;
    std::memcpy(&al, alpha, sizeof(V));
    const int64_t x = std::max<int64_t>(1, std::min<int64_t>((cols + 255) / 256, 64));
    const int64_t y = std::max<int64_t>(1, std::min<int64_t>(rows, int64_t(runtime().num_sms) * 16 / x));
    scale_kernel<V><<<dim3(unsigned(x), unsigned(y)), 256, 0, st>>>(rows, cols, al, reinterpret_cast<V*>(X), ld);
    count_launches(1);
    return cudaGetLastError();
}

template <typename T, bool CPLX>
cudaError_t launch_tri_inverse(int64_t ka, int nb, const T* SA, int64_t lda, bool trans, bool conj, bool upper,
                               bool unit, T* inv, cudaStream_t st) {
    using V = typename std::conditional<CPLX, Cx<T>, T>::type;
    const size_t smem = size_t(nb + kInvWarps) * 32 * sizeof(V);  // Y columns and the partial sums
    constexpr int nb_max = solve_block(sizeof(V));
    static const cudaError_t attr = cudaFuncSetAttribute(tri_inverse_kernel<V>,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         int((nb_max + kInvWarps) * 32 * sizeof(V)));
    if (attr != cudaSuccess) return attr;
    if (nb > nb_max || nb % 32 != 0) return cudaErrorInvalidValue;
    const int64_t blocks = (ka + nb - 1) / nb;
    tri_inverse_kernel<V><<<dim3(unsigned(nb / 32), unsigned(blocks)), 32 * kInvWarps, smem, st>>>(
        ka, nb, reinterpret_cast<const V*>(SA), lda, trans ? 1 : 0, conj ? 1 : 0, upper ? 1 : 0, unit ? 1 : 0,
        reinterpret_cast<V*>(inv));
    count_launches(1);
    return cudaGetLastError();
}

#define GB_TRSM(T, C)                                                                                             \
    template cudaError_t launch_scale<T, C>(int64_t, int64_t, const T*, T*, int64_t, cudaStream_t);               \
    template cudaError_t launch_tri_inverse<T, C>(int64_t, int, const T*, int64_t, bool, bool, bool, bool, T*, \
                                                  cudaStream_t);
GB_TRSM(double, false)
GB_TRSM(double, true)
GB_TRSM(float, false)
GB_TRSM(float, true)
#undef GB_TRSM

}  // namespace gb
