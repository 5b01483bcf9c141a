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
//
// The work is FP64 FMAs and column c needs about (nb - c)^2 / 2 of them, so the first columns set
// the kernel's time: on GB300 one SM retires about two FP64 FMAs per clock.  A block of the grid
// therefore takes only kInvCols columns (blockIdx.x picks the group, blockIdx.y the diagonal block)
// and spreads each column's sums over kInvChains chains: lane = column + kInvCols * slice, and warp
// w with slice s takes j = r0 + kInvSlices w + s, then every kInvChains-th.  The shuffles and then
// warp 0 add the chains in a fixed order.  Those adds cost FP64 instructions every row: with 8
// warps (32 chains) they were 40 % of the kernel's 18.9 M FP64 instructions at 8192 rows (1.71 ms,
// FP64 pipe 80 % active).  4 warps (16 chains) measured 1.44-1.53 ms and 2 warps 1.79-1.84 ms;
// 16-column groups measured 1.77-1.87 ms (the heaviest group then does twice the FMAs on one SM).  Warp 0 scales by the diagonal's reciprocal (computed for all rows up front, so the
// serial step per row is a multiply) and publishes Y[r] in shared memory before the next row.
// Y[j][c] = 0 for j < c comes out of the recurrence itself, so the loops are the same for every
// column of a group, which starts at its first column r0.  A unit diagonal is not read.
constexpr int kInvWarps = 4;
constexpr int kInvCols = 8;                      // columns per grid block
constexpr int kInvSlices = 32 / kInvCols;        // lanes per column in a warp
constexpr int kInvChains = kInvWarps * kInvSlices;  // FMA chains per column

template <typename V>
__global__ void __launch_bounds__(32 * kInvWarps) tri_inverse_kernel(int64_t ka, int nb, const V* __restrict__ SA,
                                                                     int64_t lda, int trans, int conj, int upper,
                                                                     int unit, V* __restrict__ inv) {
    extern __shared__ __align__(16) unsigned char tri_smem[];
    V* ycol = reinterpret_cast<V*>(tri_smem);              // [nb][kInvCols]
    V* rdiag = ycol + int64_t(nb) * kInvCols;                // [nb]
    V* part = rdiag + nb;                                    // [kInvWarps][kInvCols]
    using A = Ar<V>;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int cl = lane % kInvCols, slice = lane / kInvCols;
    const int64_t b0 = int64_t(blockIdx.y) * nb;
    const int nbk = int(min(int64_t(nb), ka - b0));
    const int r0 = int(blockIdx.x) * kInvCols;
    if (r0 >= nbk) return;
    const int c = r0 + cl;
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
    for (int r = r0 + threadIdx.x; r < nbk; r += blockDim.x) {
        const V d = unit ? A::one() : (conj ? A::conj(P[r * (sr + sj)]) : P[r * (sr + sj)]);
        rdiag[r - r0] = A::div(A::one(), d);
    }
    // rows above the group: zero (the inverse of a lower triangle is lower)
    for (int i = threadIdx.x; i < r0 * kInvCols; i += blockDim.x) {
        const int r = i / kInvCols, cc = r0 + i % kInvCols;
        if (cc < nbk) out[o0 + r * orow + cc * ocol] = A::zero();
    }
    __syncthreads();
    const int chain = warp * kInvSlices + slice;
    const int64_t lstep = kInvChains * sj;
    for (int r = r0; r < nbk; ++r) {
        V s = A::zero();
        int j = r0 + chain;
        const V* lp = P + r * sr + j * sj;
        const V* yp = ycol + (j - r0) * kInvCols + cl;
        for (; j < r; j += kInvChains, lp += lstep, yp += kInvChains * kInvCols)
            s = A::fmadd(conj ? A::conj(*lp) : *lp, *yp, s);
        // the slices of this warp (lanes cl, cl + kInvCols, ...), then the warps
#pragma unroll
        for (int o = kInvCols; o < 32; o *= 2) s = A::add(s, A::shfl_xor(s, o));
        if (slice == 0) part[warp * kInvCols + cl] = s;
        __syncthreads();
        if (warp == 0 && slice == 0) {
            V sum = part[cl];
#pragma unroll
            for (int w = 1; w < kInvWarps; ++w) sum = A::add(sum, part[w * kInvCols + cl]);
            const V acc = A::mul(A::fnmadd(A::one(), sum, (r == c) ? A::one() : A::zero()), rdiag[r - r0]);
            ycol[(r - r0) * kInvCols + cl] = acc;
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
    // Y's columns, the diagonal's reciprocals and the partial sums
    auto smem_for = [](int rows) { return (size_t(rows) * (kInvCols + 1) + kInvWarps * kInvCols) * sizeof(V); };
    constexpr int nb_max = solve_block(sizeof(V));
    static const cudaError_t attr = cudaFuncSetAttribute(tri_inverse_kernel<V>,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         int(smem_for(nb_max)));
    if (attr != cudaSuccess) return attr;
    if (nb > nb_max || nb % 32 != 0) return cudaErrorInvalidValue;
    const int64_t blocks = (ka + nb - 1) / nb;
    tri_inverse_kernel<V><<<dim3(unsigned(nb / kInvCols), unsigned(blocks)), 32 * kInvWarps, smem_for(nb), st>>>(
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
