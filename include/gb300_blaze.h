/* gb300_blaze.h — Blaze-side interception of the dense products that Blaze's kernel selection
 * keeps on the CPU, so that `C = A * B` of such shapes reaches libgb300blas as well.
 *
 * Blaze in BLAS mode calls blaze::gemm() only from selectBlasAssignKernel; before that,
 * selectAssignKernel (blaze/math/expressions/DMatDMatMultExpr.h:561-569, DMatTDMatMultExpr.h:
 * 538-545, TDMatDMatMultExpr.h:540-548, TDMatTDMatMultExpr.h:559-566) sends a product to its own
 * small SIMD kernel when the result has fewer than DMATDMATMULT_THRESHOLD (4900) elements, or —
 * for the row-major operand classes, outside debug mode — when B has at most 10 SIMD widths of
 * columns (80 doubles with AVX-512).  Those gates suit a CPU BLAS; on a GPU a (4096 x 4096) x
 * (4096 x 64) product is 2 GFLOP of work, and a small product is best sent here with the rest.
 *
 * Including this header after Blaze adds overloads of smpAssign / smpAddAssign / smpSubAssign
 * for the four dense product expressions (and for s * (A * B) under assignment).  Blaze's
 * DynamicMatrix / CustomMatrix assignment operators call these functions for `C = A*B`,
 * `C += A*B`, `C -= A*B` and `C = s*(A*B)` (DynamicMatrix.h:1613-1640 and the add / subtract
 * operators next to it); argument-dependent lookup finds the overloads here, which match the
 * product expression exactly and therefore win over Blaze's generic SMP assignment.  An
 * intercepted product goes straight to blaze::gemm (blaze/math/blas/gemm.h:105-131), i.e. the
 * same cblas_?gemm call with the same order / transposition / leading-dimension mapping that
 * Blaze's own BLAS kernel would make, whatever its shape.
 *
 * A product is intercepted only when Blaze's own BLAS kernel could take it
 * (DMatDMatMultExpr.h:213-225, UseBlasKernel_v): the target and both operands are contiguous
 * dense matrices with data access (not expressions, views without data access, adaptors or
 * diagonal / triangular / symmetric / Hermitian types), all of one BLAS element type, and the
 * expression carries no symmetry / triangle declaration.  Everything else keeps Blaze's own
 * evaluation.  Products with fewer than GB300_BLAZE_MIN_WORK multiply-adds (m*n*k; default 0:
 * every eligible product) also keep Blaze's kernel selection: a single GPU call costs tens of
 * microseconds, so hosts that evaluate many tiny products one by one may prefer to leave them to
 * the CPU (or send them together through gb300_dgemm_grouped).
 *
 * Use: compile with -DBLAZE_BLAS_MODE=1 -DBLAZE_BLAS_INCLUDE_FILE="<gb300_cblas.h>" (as for the
 * plain drop-in) and include this header after <blaze/Math.h> in every translation unit that
 * evaluates products.  Errors surface as they do for any BLAS call (GB300_BLAS_THROW turns a
 * failing call into std::runtime_error).
 */
#ifndef GB300_BLAZE_H
#define GB300_BLAZE_H

#include <blaze/Math.h>

#if !BLAZE_BLAS_MODE
#error "gb300_blaze.h needs Blaze's BLAS mode (-DBLAZE_BLAS_MODE=1 with gb300_cblas.h as its BLAS header)"
#endif

#ifndef GB300_BLAZE_MIN_WORK
#define GB300_BLAZE_MIN_WORK 0
#endif

namespace blaze {

namespace gb300_detail {

/* Blaze's dense x dense product expression class templates (row x row, row x column, column x
 * row, column x column operands). */
template <template <typename, typename, bool, bool, bool, bool> class E>
struct IsDenseProduct : FalseType {};
template <>
struct IsDenseProduct<DMatDMatMultExpr> : TrueType {};
template <>
struct IsDenseProduct<DMatTDMatMultExpr> : TrueType {};
template <>
struct IsDenseProduct<TDMatDMatMultExpr> : TrueType {};
template <>
struct IsDenseProduct<TDMatTDMatMultExpr> : TrueType {};

/* A plain stored operand: contiguous, readable through data(), no structure Blaze exploits. */
template <typename T>
constexpr bool PlainOperand_v = IsDenseMatrix_v<T> && !IsExpression_v<T> && IsContiguous_v<T> &&
                                HasConstDataAccess_v<T> && !IsAdaptor_v<T> && !IsDiagonal_v<T> &&
                                !IsTriangular_v<T> && !IsSymmetric_v<T> && !IsHermitian_v<T>;

/* Whether C = op(A * B) with target MT and operands MT1, MT2 goes to blaze::gemm here. */
template <typename MT, typename MT1, typename MT2>
constexpr bool Intercepts_v = BLAZE_USE_BLAS_MATRIX_MATRIX_MULTIPLICATION && PlainOperand_v<MT1> &&
                              PlainOperand_v<MT2> && IsContiguous_v<MT> && HasMutableDataAccess_v<MT> &&
                              !IsAdaptor_v<MT> && !IsExpression_v<MT> &&
                              IsBLASCompatible_v<ElementType_t<MT>> &&
                              IsSame_v<ElementType_t<MT>, ElementType_t<MT1>> &&
                              IsSame_v<ElementType_t<MT>, ElementType_t<MT2>>;

/* Enough work for the GPU (GB300_BLAZE_MIN_WORK multiply-adds); the sizes Blaze checked already
 * agree (the expression was built by operator*). */
template <typename MA, typename MB>
inline bool worth_it(const MA& A, const MB& B) {
    return double(A.rows()) * double(B.columns()) * double(A.columns()) >= double(GB300_BLAZE_MIN_WORK);
}

/* C = alpha * A * B + beta * C through Blaze's own BLAS wrapper; k == 0 leaves beta * C. */
template <typename MT, bool SO, typename MA, typename MB, typename ET>
inline void product(DenseMatrix<MT, SO>& C, const MA& A, const MB& B, ET alpha, ET beta) {
    if ((*C).rows() == 0UL || (*C).columns() == 0UL) return;
    if (A.columns() == 0UL) {
        if (beta == ET(0)) reset(*C);
        return;
    }
    gemm(*C, A, B, alpha, beta);
}

}  // namespace gb300_detail

/* C = A * B */
template <typename MT, bool SO, template <typename, typename, bool, bool, bool, bool> class E, typename MT1,
          typename MT2>
inline auto smpAssign(DenseMatrix<MT, SO>& lhs, const E<MT1, MT2, false, false, false, false>& rhs)
    -> EnableIf_t<gb300_detail::IsDenseProduct<E>::value && gb300_detail::Intercepts_v<MT, MT1, MT2>> {
    using ET = ElementType_t<MT>;
    const auto& A = rhs.leftOperand();
    const auto& B = rhs.rightOperand();
    if (!gb300_detail::worth_it(A, B)) {
        assign(*lhs, rhs);  // Blaze's own kernel selection
        return;
    }
    gb300_detail::product(lhs, A, B, ET(1), ET(0));
}

/* C += A * B */
template <typename MT, bool SO, template <typename, typename, bool, bool, bool, bool> class E, typename MT1,
          typename MT2>
inline auto smpAddAssign(DenseMatrix<MT, SO>& lhs, const E<MT1, MT2, false, false, false, false>& rhs)
    -> EnableIf_t<gb300_detail::IsDenseProduct<E>::value && gb300_detail::Intercepts_v<MT, MT1, MT2>> {
    using ET = ElementType_t<MT>;
    const auto& A = rhs.leftOperand();
    const auto& B = rhs.rightOperand();
    if (!gb300_detail::worth_it(A, B)) {
        addAssign(*lhs, rhs);
        return;
    }
    gb300_detail::product(lhs, A, B, ET(1), ET(1));
}

/* C -= A * B */
template <typename MT, bool SO, template <typename, typename, bool, bool, bool, bool> class E, typename MT1,
          typename MT2>
inline auto smpSubAssign(DenseMatrix<MT, SO>& lhs, const E<MT1, MT2, false, false, false, false>& rhs)
    -> EnableIf_t<gb300_detail::IsDenseProduct<E>::value && gb300_detail::Intercepts_v<MT, MT1, MT2>> {
    using ET = ElementType_t<MT>;
    const auto& A = rhs.leftOperand();
    const auto& B = rhs.rightOperand();
    if (!gb300_detail::worth_it(A, B)) {
        subAssign(*lhs, rhs);
        return;
    }
    gb300_detail::product(lhs, A, B, ET(-1), ET(1));
}

/* C = s * (A * B) */
template <typename MT, bool SO, template <typename, typename, bool, bool, bool, bool> class E, typename MT1,
          typename MT2, typename ST, bool SO2>
inline auto smpAssign(DenseMatrix<MT, SO>& lhs,
                      const DMatScalarMultExpr<E<MT1, MT2, false, false, false, false>, ST, SO2>& rhs)
    -> EnableIf_t<gb300_detail::IsDenseProduct<E>::value && gb300_detail::Intercepts_v<MT, MT1, MT2> &&
                  IsNumeric_v<ST>> {
    using ET = ElementType_t<MT>;
    const auto& AB = rhs.leftOperand();
    const auto& A = AB.leftOperand();
    const auto& B = AB.rightOperand();
    if (!gb300_detail::worth_it(A, B)) {
        assign(*lhs, rhs);
        return;
    }
    gb300_detail::product(lhs, A, B, ET(rhs.rightOperand()), ET(0));
}

}  // namespace blaze

#endif /* GB300_BLAZE_H */
