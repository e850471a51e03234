// Minimal BLAS++-compatible shim (written for this project) so that the reference's
// CPU sources compile against OpenBLAS's Fortran/C symbols.  Only the subset of the
// BLAS++ v2023.01.00 API that the TLR-GEMM CPU path calls is provided: the enums,
// real_type, conj, scal, gemm, trmm, trsm, syrk.  Test infrastructure only.
#ifndef HCGB_SHIM_BLAS_HH
#define HCGB_SHIM_BLAS_HH

#include <cstdint>
#include <cstddef>
#include <stdexcept>
#include <complex>
#include <vector>
#include <string>
#include <cmath>
#include <algorithm>
#include "hcgb_fortran.h"

namespace blas {

enum class Layout : char { ColMajor = 'C', RowMajor = 'R' };
enum class Op : char { NoTrans = 'N', Trans = 'T', ConjTrans = 'C' };
enum class Uplo : char { Upper = 'U', Lower = 'L', General = 'G' };
enum class Diag : char { NonUnit = 'N', Unit = 'U' };
enum class Side : char { Left = 'L', Right = 'R' };

template <typename T> struct real_type_traits { using type = T; };
template <typename T> struct real_type_traits<std::complex<T>> { using type = T; };
template <typename T> using real_type = typename real_type_traits<T>::type;

template <typename T> struct is_complex { static constexpr bool value = false; };
template <typename T> struct is_complex<std::complex<T>> { static constexpr bool value = true; };

inline float conj(float x) { return x; }
inline double conj(double x) { return x; }

namespace detail {
inline char op_char(Op op) { return static_cast<char>(op); }
inline Op flip(Op op) { return op == Op::NoTrans ? Op::Trans : Op::NoTrans; }
inline Uplo flip(Uplo u) { return u == Uplo::Upper ? Uplo::Lower : (u == Uplo::Lower ? Uplo::Upper : u); }
inline Side flip(Side s) { return s == Side::Left ? Side::Right : Side::Left; }
}

#define HCGB_SHIM_BLAS_REAL(T, P)                                                                   \
inline void scal(int64_t n, T alpha, T *x, int64_t incx) {                                        \
    hcgb_blas_int nn = n, inc = incx;                                                               \
    HCGB_F77(P##scal)(&nn, &alpha, x, &inc);                                                        \
}                                                                                                   \
inline void gemm(Layout layout, Op ta, Op tb, int64_t m, int64_t n, int64_t k, T alpha,             \
                 const T *A, int64_t lda, const T *B, int64_t ldb, T beta, T *C, int64_t ldc) {     \
    if (layout == Layout::RowMajor) {                                                               \
        gemm(Layout::ColMajor, tb, ta, n, m, k, alpha, B, ldb, A, lda, beta, C, ldc);               \
        return;                                                                                     \
    }                                                                                               \
    if (m == 0 || n == 0) return;                                                                   \
    char a = detail::op_char(ta), b = detail::op_char(tb);                                          \
    hcgb_blas_int mm = m, nn = n, kk = k, la = lda < 1 ? 1 : lda, lb = ldb < 1 ? 1 : ldb, lc = ldc; \
    HCGB_F77(P##gemm)(&a, &b, &mm, &nn, &kk, &alpha, A, &la, B, &lb, &beta, C, &lc, 1, 1);          \
}                                                                                                   \
inline void trmm(Layout layout, Side side, Uplo uplo, Op trans, Diag diag, int64_t m, int64_t n,   \
                 T alpha, const T *A, int64_t lda, T *B, int64_t ldb) {                             \
    if (layout == Layout::RowMajor) {                                                               \
        trmm(Layout::ColMajor, detail::flip(side), detail::flip(uplo), trans, diag, n, m, alpha,    \
             A, lda, B, ldb);                                                                       \
        return;                                                                                     \
    }                                                                                               \
    char s = (char) side, u = (char) uplo, t = (char) trans, d = (char) diag;                       \
    hcgb_blas_int mm = m, nn = n, la = lda, lb = ldb;                                               \
    HCGB_F77(P##trmm)(&s, &u, &t, &d, &mm, &nn, &alpha, A, &la, B, &lb, 1, 1, 1, 1);                \
}                                                                                                   \
inline void trsm(Layout layout, Side side, Uplo uplo, Op trans, Diag diag, int64_t m, int64_t n,   \
                 T alpha, const T *A, int64_t lda, T *B, int64_t ldb) {                             \
    if (layout == Layout::RowMajor) {                                                               \
        trsm(Layout::ColMajor, detail::flip(side), detail::flip(uplo), trans, diag, n, m, alpha,    \
             A, lda, B, ldb);                                                                       \
        return;                                                                                     \
    }                                                                                               \
    char s = (char) side, u = (char) uplo, t = (char) trans, d = (char) diag;                       \
    hcgb_blas_int mm = m, nn = n, la = lda, lb = ldb;                                               \
    HCGB_F77(P##trsm)(&s, &u, &t, &d, &mm, &nn, &alpha, A, &la, B, &lb, 1, 1, 1, 1);                \
}                                                                                                   \
inline void syrk_impl(Layout layout, Uplo uplo, Op trans, int64_t n, int64_t k, T alpha,            \
                      const T *A, int64_t lda, T beta, T *C, int64_t ldc, T) {                      \
    if (layout == Layout::RowMajor) {                                                               \
        syrk_impl(Layout::ColMajor, detail::flip(uplo), detail::flip(trans), n, k, alpha, A, lda,   \
                  beta, C, ldc, T());                                                               \
        return;                                                                                     \
    }                                                                                               \
    char u = (char) uplo, t = (char) trans;                                                         \
    hcgb_blas_int nn = n, kk = k, la = lda, lc = ldc;                                               \
    HCGB_F77(P##syrk)(&u, &t, &nn, &kk, &alpha, A, &la, &beta, C, &lc, 1, 1);                      \
}

HCGB_SHIM_BLAS_REAL(float, s)
HCGB_SHIM_BLAS_REAL(double, d)
#undef HCGB_SHIM_BLAS_REAL

template <typename T>
void syrk(Layout layout, Uplo uplo, Op trans, int64_t n, int64_t k, T alpha, const T *A, int64_t lda,
          T beta, T *C, int64_t ldc) {
    syrk_impl(layout, uplo, trans, n, k, alpha, A, lda, beta, C, ldc, T());
}

}  // namespace blas

#endif
