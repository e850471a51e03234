// Dense per-tile building blocks of a tile Cholesky: potrf, trsm, syrk (FP64).
//
// Replace HCoreKernels<T>::potrf / trsm / syrk on the GPU (src/kernels/cuda/kernels.cpp:290-306,
// src/kernels/cuda/CudaKernels.cu:1019-1049: cuSOLVER Xpotrf, cuBLAS trsm/syrk) with the
// semantics of LAPACK dpotrf and BLAS dtrsm / dsyrk (column-major), which the CPU backend calls
// (src/kernels/omp/kernels.cpp:234-282).  One CTA per call: these operate on one tile (nb <= 1024)
// and sit off the GEMM hot path.
#include "internal.cuh"

namespace hcgb {

namespace {

constexpr int CT = 1024;

__device__ double block_reduce_sum(double v, double *red) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double t = lane < nw ? red[lane] : 0.0;
        t = warp_sum(t);
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

// Left-looking Cholesky of the lower (uplo 0) or upper (uplo 1) triangle of A (n x n, ld lda).
// info: 0, or j + 1 when the leading minor of order j + 1 is not positive (dpotrf's convention;
// the factorisation stops there).  The other triangle is not referenced.
__global__ void __launch_bounds__(CT) potrf_kernel(double *A, int n, int lda, int uplo, int *info) {
    __shared__ double red[40];
    __shared__ int s_info;
    if (threadIdx.x == 0) s_info = 0;
    __syncthreads();
    // L(i, k) for the lower case; the upper case stores U(k, i) = L(i, k).
    auto L = [&](int i, int k) -> double & { return uplo == 0 ? A[i + (size_t) k * lda] : A[k + (size_t) i * lda]; };
    for (int j = 0; j < n; j++) {
        double part = 0.0;
        for (int k = threadIdx.x; k < j; k += blockDim.x) part = fma(L(j, k), L(j, k), part);
        const double s = block_reduce_sum(part, red);
        const double d = L(j, j) - s;
        if (!(d > 0.0)) {
            if (threadIdx.x == 0) s_info = j + 1;
            __syncthreads();
            break;
        }
        const double ljj = sqrt(d);
        for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) {
            double t = L(i, j);
            for (int k = 0; k < j; k++) t = fma(-L(i, k), L(j, k), t);
            L(i, j) = t / ljj;
        }
        __syncthreads();
        if (threadIdx.x == 0) L(j, j) = ljj;
        __syncthreads();
    }
    if (threadIdx.x == 0 && info) *info = s_info;
}

// op(A) X = alpha B (side 0) or X op(A) = alpha B (side 1); X overwrites B (m x n, ld ldb).
// Reduced to S y = alpha b for every vector b: columns of B with S = op(A) (side 0), or rows of B
// with S = op(A)^T (side 1); S is lower or upper triangular and solved by substitution, one
// step per row of S with all vectors updated in parallel.
__global__ void __launch_bounds__(CT) trsm_kernel(int side, int uplo, int trans, int diag, int m, int n, double alpha,
                                                  const double *A, int lda, double *B, int ldb) {
    const int len = side == 0 ? m : n;      // order of S
    const int count = side == 0 ? n : m;    // number of vectors
    // S(i, k): side 0: op(A)(i, k); side 1: op(A)(k, i).
    const bool t_eff = (side == 0) ? (trans != 0) : (trans == 0);
    const bool lower_s = (uplo == 0) != t_eff;
    auto S = [&](int i, int k) -> double { return t_eff ? A[k + (size_t) i * lda] : A[i + (size_t) k * lda]; };
    auto Bref = [&](int i, int v) -> double & { return side == 0 ? B[i + (size_t) v * ldb] : B[v + (size_t) i * ldb]; };
    for (int e = threadIdx.x; e < len * count; e += blockDim.x) Bref(e % len, e / len) *= alpha;
    __syncthreads();
    for (int step = 0; step < len; step++) {
        const int i = lower_s ? step : len - 1 - step;
        if (diag == 0) {
            const double sii = S(i, i);
            for (int v = threadIdx.x; v < count; v += blockDim.x) Bref(i, v) /= sii;
        }
        __syncthreads();
        // eliminate x_i from the remaining rows
        const int rest = lower_s ? len - 1 - i : i;
        for (int e = threadIdx.x; e < rest * count; e += blockDim.x) {
            const int r = e % rest, v = e / rest;
            const int k = lower_s ? i + 1 + r : r;
            Bref(k, v) = fma(-S(k, i), Bref(i, v), Bref(k, v));
        }
        __syncthreads();
    }
}

// C = alpha op(A) op(A)^T + beta C on the uplo triangle of C (n x n); op(A) is n x k.
__global__ void syrk_kernel(int uplo, int trans, int n, int k, double alpha, const double *A, int lda, double beta,
                            double *C, int ldc) {
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || j >= n) return;
    if (uplo == 0 ? (i < j) : (i > j)) return;
    double s = 0.0;
    for (int l = 0; l < k; l++) {
        const double a = trans ? A[l + (size_t) i * lda] : A[i + (size_t) l * lda];
        const double b = trans ? A[l + (size_t) j * lda] : A[j + (size_t) l * lda];
        s = fma(a, b, s);
    }
    double *c = C + i + (size_t) j * ldc;
    *c = alpha * s + (beta != 0.0 ? beta * *c : 0.0);
}

// Sets the strict uplo triangle of A (n x n, ld lda) to value (HCoreKernels::FillMatrixTriangle,
// src/kernels/omp/kernels.cpp:246-264).
__global__ void fill_triangle_kernel(int uplo, int n, double *A, int lda, double value) {
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || j >= n) return;
    if (uplo == 0 ? (i > j) : (i < j)) A[i + (size_t) j * lda] = value;
}

// Panel solve of a tile Cholesky step: for every compressed_vt tile of the panel, W <- L^-1 W
// (Left, Lower, NoTrans, NonUnit, alpha 1 on the W region, rows x rank, ld rows): HCore<T>::Trsm
// as the tile Cholesky applies it (src/api/HCore.cpp:623-647), one CTA per tile, the rank read on
// the device.  Same operations in the same order as trsm_kernel, so the results are identical.
__global__ void __launch_bounds__(256) trsm_panel_kernel(const double *L, int nb, int ldl, const DevTile *tiles) {
    const DevTile t = tiles[blockIdx.x];
    const int r = *t.rank;
    if (r <= 0 || r > t.max_rank || t.rows != nb) return;
    double *W = t.v;
    const int ld = t.rows;
    for (int i = 0; i < nb; i++) {
        const double lii = L[i + (size_t) i * ldl];
        for (int c = threadIdx.x; c < r; c += blockDim.x) W[i + (size_t) c * ld] /= lii;
        __syncthreads();
        const int rest = nb - 1 - i;
        for (int e = threadIdx.x; e < rest * r; e += blockDim.x) {
            const int q = e % rest, c = e / rest;
            const int k = i + 1 + q;
            W[k + (size_t) c * ld] = fma(-L[k + (size_t) i * ldl], W[i + (size_t) c * ld], W[k + (size_t) c * ld]);
        }
        __syncthreads();
    }
}

}  // namespace

void launch_trsm_panel(const double *L, int nb, int ldl, const DevTile *tiles, int count, cudaStream_t st) {
    if (count > 0) { trsm_panel_kernel<<<count, 256, 0, st>>>(L, nb, ldl, tiles); note_launch(); }
}

void launch_fill_triangle(int uplo, int n, double *A, int lda, double value, cudaStream_t st) {
    dim3 blk(32, 8), grid((n + 31) / 32, (n + 7) / 8);
    { fill_triangle_kernel<<<grid, blk, 0, st>>>(uplo, n, A, lda, value); note_launch(); }
}

void launch_potrf(double *A, int n, int lda, int uplo, int *info_dev, cudaStream_t st) {
    { potrf_kernel<<<1, CT, 0, st>>>(A, n, lda, uplo, info_dev); note_launch(); }
}

void launch_trsm(int side, int uplo, int trans, int diag, int m, int n, double alpha, const double *A, int lda,
                 double *B, int ldb, cudaStream_t st) {
    { trsm_kernel<<<1, CT, 0, st>>>(side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb); note_launch(); }
}

void launch_syrk(int uplo, int trans, int n, int k, double alpha, const double *A, int lda, double beta, double *C,
                 int ldc, cudaStream_t st) {
    dim3 blk(16, 16), grid((n + 15) / 16, (n + 15) / 16);
    { syrk_kernel<<<grid, blk, 0, st>>>(uplo, trans, n, k, alpha, A, lda, beta, C, ldc); note_launch(); }
}

}  // namespace hcgb
