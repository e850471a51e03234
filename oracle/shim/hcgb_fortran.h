// Fortran-ABI declarations of the BLAS/LAPACK routines the shim forwards to.
// The library is SciPy's bundled OpenBLAS (LP64), whose symbols carry a "scipy_"
// prefix.  Character arguments take gfortran's hidden length arguments at the end.
#ifndef HCGB_SHIM_FORTRAN_H
#define HCGB_SHIM_FORTRAN_H
#include <cstddef>

typedef int hcgb_blas_int;

#ifndef HCGB_F77_PREFIX
#define HCGB_F77_PREFIX scipy_
#endif
#define HCGB_CAT3_(a, b, c) a##b##c
#define HCGB_CAT3(a, b, c) HCGB_CAT3_(a, b, c)
#define HCGB_F77(name) HCGB_CAT3(HCGB_F77_PREFIX, name, _)

#define HCGB_DECL(T, P)                                                                              \
void HCGB_F77(P##scal)(const hcgb_blas_int *, const T *, T *, const hcgb_blas_int *);               \
void HCGB_F77(P##gemm)(const char *, const char *, const hcgb_blas_int *, const hcgb_blas_int *,     \
                       const hcgb_blas_int *, const T *, const T *, const hcgb_blas_int *, const T *, \
                       const hcgb_blas_int *, const T *, T *, const hcgb_blas_int *, size_t, size_t);\
void HCGB_F77(P##trmm)(const char *, const char *, const char *, const char *, const hcgb_blas_int *,\
                       const hcgb_blas_int *, const T *, const T *, const hcgb_blas_int *, T *,      \
                       const hcgb_blas_int *, size_t, size_t, size_t, size_t);                      \
void HCGB_F77(P##trsm)(const char *, const char *, const char *, const char *, const hcgb_blas_int *,\
                       const hcgb_blas_int *, const T *, const T *, const hcgb_blas_int *, T *,      \
                       const hcgb_blas_int *, size_t, size_t, size_t, size_t);                      \
void HCGB_F77(P##syrk)(const char *, const char *, const hcgb_blas_int *, const hcgb_blas_int *,     \
                       const T *, const T *, const hcgb_blas_int *, const T *, T *,                 \
                       const hcgb_blas_int *, size_t, size_t);                                      \
void HCGB_F77(P##geqrf)(const hcgb_blas_int *, const hcgb_blas_int *, T *, const hcgb_blas_int *,   \
                        T *, T *, const hcgb_blas_int *, hcgb_blas_int *);                          \
void HCGB_F77(P##orgqr)(const hcgb_blas_int *, const hcgb_blas_int *, const hcgb_blas_int *, T *,   \
                        const hcgb_blas_int *, const T *, T *, const hcgb_blas_int *,               \
                        hcgb_blas_int *);                                                           \
void HCGB_F77(P##ormqr)(const char *, const char *, const hcgb_blas_int *, const hcgb_blas_int *,   \
                        const hcgb_blas_int *, const T *, const hcgb_blas_int *, const T *, T *,    \
                        const hcgb_blas_int *, T *, const hcgb_blas_int *, hcgb_blas_int *, size_t, \
                        size_t);                                                                    \
void HCGB_F77(P##gesvd)(const char *, const char *, const hcgb_blas_int *, const hcgb_blas_int *,   \
                        T *, const hcgb_blas_int *, T *, T *, const hcgb_blas_int *, T *,           \
                        const hcgb_blas_int *, T *, const hcgb_blas_int *, hcgb_blas_int *, size_t, \
                        size_t);                                                                    \
void HCGB_F77(P##gesdd)(const char *, const hcgb_blas_int *, const hcgb_blas_int *, T *,            \
                        const hcgb_blas_int *, T *, T *, const hcgb_blas_int *, T *,                \
                        const hcgb_blas_int *, T *, const hcgb_blas_int *, hcgb_blas_int *,         \
                        hcgb_blas_int *, size_t);                                                   \
void HCGB_F77(P##lacpy)(const char *, const hcgb_blas_int *, const hcgb_blas_int *, const T *,      \
                        const hcgb_blas_int *, T *, const hcgb_blas_int *, size_t);                 \
void HCGB_F77(P##laset)(const char *, const hcgb_blas_int *, const hcgb_blas_int *, const T *,      \
                        const T *, T *, const hcgb_blas_int *, size_t);                             \
void HCGB_F77(P##potrf)(const char *, const hcgb_blas_int *, T *, const hcgb_blas_int *,            \
                        hcgb_blas_int *, size_t);

extern "C" {
HCGB_DECL(float, s)
HCGB_DECL(double, d)
void HCGB_CAT3(HCGB_F77_PREFIX, openblas_set_num_threads, )(int);
}
#undef HCGB_DECL

#endif
