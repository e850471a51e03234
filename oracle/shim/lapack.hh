// Minimal LAPACK++-compatible shim (written for this project): the enums and the
// routines the reference's CPU path calls (geqrf, gesvd, gesdd, ungqr, unmqr, lacpy,
// laset, potrf), forwarding to OpenBLAS's LAPACK with workspace queries.
// Test infrastructure only.
#ifndef HCGB_SHIM_LAPACK_HH
#define HCGB_SHIM_LAPACK_HH

#include <vector>
#include <algorithm>
#include <stdexcept>
#include "blas.hh"

namespace lapack {

using blas::Op;
using blas::Uplo;
using blas::Side;
using blas::Diag;
using blas::Layout;

enum class Job : char {
    NoVec = 'N', Vec = 'V', UpdateVec = 'U', AllVec = 'A', SomeVec = 'S', OverwriteVec = 'O',
    CompactVec = 'P', SomeVecTol = 'C', VecJacobi = 'J', Workspace = 'W'
};
enum class MatrixType : char {
    General = 'G', Lower = 'L', Upper = 'U', Hessenberg = 'H', LowerBand = 'B', UpperBand = 'Q', Band = 'Z'
};

namespace detail {
inline void check(hcgb_blas_int info, const char *who) {
    if (info < 0) throw std::invalid_argument(who);
}
}

#define HCGB_SHIM_LAPACK_REAL(T, P)                                                                  \
inline int64_t geqrf(int64_t m, int64_t n, T *A, int64_t lda, T *tau) {                             \
    hcgb_blas_int mm = m, nn = n, la = lda, lw = -1, info = 0; T q = 0;                             \
    HCGB_F77(P##geqrf)(&mm, &nn, A, &la, tau, &q, &lw, &info);                                      \
    lw = std::max<hcgb_blas_int>(1, (hcgb_blas_int) q); std::vector<T> w(lw);                      \
    HCGB_F77(P##geqrf)(&mm, &nn, A, &la, tau, w.data(), &lw, &info);                                \
    detail::check(info, "geqrf"); return info;                                                      \
}                                                                                                   \
inline int64_t ungqr(int64_t m, int64_t n, int64_t k, T *A, int64_t lda, const T *tau) {           \
    hcgb_blas_int mm = m, nn = n, kk = k, la = lda, lw = -1, info = 0; T q = 0;                     \
    HCGB_F77(P##orgqr)(&mm, &nn, &kk, A, &la, tau, &q, &lw, &info);                                 \
    lw = std::max<hcgb_blas_int>(1, (hcgb_blas_int) q); std::vector<T> w(lw);                      \
    HCGB_F77(P##orgqr)(&mm, &nn, &kk, A, &la, tau, w.data(), &lw, &info);                           \
    detail::check(info, "ungqr"); return info;                                                      \
}                                                                                                   \
inline int64_t unmqr(Side side, Op trans, int64_t m, int64_t n, int64_t k, const T *A,              \
                     int64_t lda, const T *tau, T *C, int64_t ldc) {                                \
    char s = (char) side, t = trans == Op::NoTrans ? 'N' : 'T';                                     \
    hcgb_blas_int mm = m, nn = n, kk = k, la = lda, lc = ldc, lw = -1, info = 0; T q = 0;           \
    HCGB_F77(P##ormqr)(&s, &t, &mm, &nn, &kk, A, &la, tau, C, &lc, &q, &lw, &info, 1, 1);           \
    lw = std::max<hcgb_blas_int>(1, (hcgb_blas_int) q); std::vector<T> w(lw);                      \
    HCGB_F77(P##ormqr)(&s, &t, &mm, &nn, &kk, A, &la, tau, C, &lc, w.data(), &lw, &info, 1, 1);     \
    detail::check(info, "unmqr"); return info;                                                      \
}                                                                                                   \
inline int64_t gesvd(Job ju, Job jvt, int64_t m, int64_t n, T *A, int64_t lda, T *S, T *U,          \
                     int64_t ldu, T *VT, int64_t ldvt) {                                            \
    char a = (char) ju, b = (char) jvt;                                                             \
    hcgb_blas_int mm = m, nn = n, la = lda, lu = std::max<int64_t>(1, ldu),                         \
                  lv = std::max<int64_t>(1, ldvt), lw = -1, info = 0; T q = 0;                      \
    HCGB_F77(P##gesvd)(&a, &b, &mm, &nn, A, &la, S, U, &lu, VT, &lv, &q, &lw, &info, 1, 1);         \
    lw = std::max<hcgb_blas_int>(1, (hcgb_blas_int) q); std::vector<T> w(lw);                      \
    HCGB_F77(P##gesvd)(&a, &b, &mm, &nn, A, &la, S, U, &lu, VT, &lv, w.data(), &lw, &info, 1, 1);   \
    detail::check(info, "gesvd"); return info;                                                      \
}                                                                                                   \
inline int64_t gesdd(Job jz, int64_t m, int64_t n, T *A, int64_t lda, T *S, T *U, int64_t ldu,      \
                     T *VT, int64_t ldvt) {                                                         \
    char a = (char) jz;                                                                             \
    hcgb_blas_int mm = m, nn = n, la = lda, lu = std::max<int64_t>(1, ldu),                         \
                  lv = std::max<int64_t>(1, ldvt), lw = -1, info = 0; T q = 0;                      \
    std::vector<hcgb_blas_int> iw(8 * std::max<int64_t>(1, std::min(m, n)));                        \
    HCGB_F77(P##gesdd)(&a, &mm, &nn, A, &la, S, U, &lu, VT, &lv, &q, &lw, iw.data(), &info, 1);     \
    lw = std::max<hcgb_blas_int>(1, (hcgb_blas_int) q); std::vector<T> w(lw);                      \
    HCGB_F77(P##gesdd)(&a, &mm, &nn, A, &la, S, U, &lu, VT, &lv, w.data(), &lw, iw.data(), &info,  \
                       1);                                                                          \
    detail::check(info, "gesdd"); return info;                                                      \
}                                                                                                   \
inline void lacpy(MatrixType type, int64_t m, int64_t n, const T *A, int64_t lda, T *B,             \
                  int64_t ldb) {                                                                    \
    char u = (char) type; hcgb_blas_int mm = m, nn = n, la = lda, lb = ldb;                         \
    HCGB_F77(P##lacpy)(&u, &mm, &nn, A, &la, B, &lb, 1);                                            \
}                                                                                                   \
inline void laset(MatrixType type, int64_t m, int64_t n, T offdiag, T diag, T *A, int64_t lda) {    \
    char u = (char) type; hcgb_blas_int mm = m, nn = n, la = lda;                                   \
    HCGB_F77(P##laset)(&u, &mm, &nn, &offdiag, &diag, A, &la, 1);                                   \
}                                                                                                   \
inline int64_t potrf(Uplo uplo, int64_t n, T *A, int64_t lda) {                                     \
    char u = (char) uplo; hcgb_blas_int nn = n, la = lda, info = 0;                                 \
    HCGB_F77(P##potrf)(&u, &nn, A, &la, &info, 1);                                                  \
    detail::check(info, "potrf"); return info;                                                      \
}

HCGB_SHIM_LAPACK_REAL(float, s)
HCGB_SHIM_LAPACK_REAL(double, d)
#undef HCGB_SHIM_LAPACK_REAL

}  // namespace lapack

#endif
