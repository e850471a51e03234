// Shim: BLAS++ flop counts used by the reference's tests (gemm only).
#ifndef HCGB_SHIM_BLAS_FLOPS_HH
#define HCGB_SHIM_BLAS_FLOPS_HH
#include "../blas.hh"
namespace blas {
template <typename T> struct Gflop {
    static double gemm(double m, double n, double k) { return 2.0 * m * n * k * 1e-9; }
};
}
#endif
