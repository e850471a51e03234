// Per-matrix dense building blocks behind the HCoreKernels<double> backend for GB300
// (hcorepp_gb300/backend): the operations HCore++'s CompressedTile<T>::Gemm and its tests call one
// matrix at a time (include/hcorepp/kernels/kernels.hpp:24-137), each on the context's stream:
// general products (the batched product kernels with one job), copies with transposition and
// scaling, lacpy / laset, row scaling, Householder QR (dgeqr2 form), forming and applying its Q
// (dorg2r / dorm2r), triangular multiply, symmetrisation and an FP64 one-sided Jacobi SVD.
//
// These serve the reference's own step-by-step recompression when it is built on this backend;
// the batched entry points (hcgb_gemm_batch, hcgb_tlr_gemm) are the fast path.  FP64 SIMT; one
// CTA per matrix for the factorisations.
#include <algorithm>
#include <string>

#include "internal.cuh"

namespace hcgb {

namespace {

__device__ __forceinline__ double block_reduce(double v, double *red) {
    v = warp_sum(v);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < nw; w++) t += red[w];
    return t;
}

// B (m x n) = alpha op(A), op = transpose when trans.
__global__ void copy_kernel(int trans, int m, int n, double alpha, const double *A, int lda, double *B, int ldb) {
    const long long total = (long long) m * n;
    for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x; e < total;
         e += (long long) gridDim.x * blockDim.x) {
        const int i = (int) (e % m), j = (int) (e / m);
        const double v = trans ? A[j + (size_t) i * lda] : A[i + (size_t) j * lda];
        B[i + (size_t) j * ldb] = alpha * v;
    }
}

// LAPACK dlacpy: uplo 0 general, 1 upper (i <= j), 2 lower (i >= j).
__global__ void lacpy_kernel(int uplo, int m, int n, const double *A, int lda, double *B, int ldb) {
    const long long total = (long long) m * n;
    for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x; e < total;
         e += (long long) gridDim.x * blockDim.x) {
        const int i = (int) (e % m), j = (int) (e / m);
        if ((uplo == 1 && i > j) || (uplo == 2 && i < j)) continue;
        B[i + (size_t) j * ldb] = A[i + (size_t) j * lda];
    }
}

// LAPACK dlaset: off-diagonal part (per uplo: 0 all, 1 strictly upper, 2 strictly lower) = offdiag,
// diagonal = diag; uplo 3 sets only the diagonal.
__global__ void laset_kernel(int uplo, int m, int n, double offdiag, double diag, double *A, int lda) {
    const long long total = (long long) m * n;
    for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x; e < total;
         e += (long long) gridDim.x * blockDim.x) {
        const int i = (int) (e % m), j = (int) (e / m);
        if (i == j) {
            A[i + (size_t) j * lda] = diag;
            continue;
        }
        if (uplo == 3 || (uplo == 1 && i > j) || (uplo == 2 && i < j)) continue;
        A[i + (size_t) j * lda] = offdiag;
    }
}

// Row i < rows of A (ld lda, cols columns) scaled by s[i] (device).
__global__ void scale_rows_kernel(int rows, int cols, const double *s, double *A, int lda) {
    const long long total = (long long) rows * cols;
    for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x; e < total;
         e += (long long) gridDim.x * blockDim.x) {
        const int i = (int) (e % rows), j = (int) (e / rows);
        A[i + (size_t) j * lda] *= s[i];
    }
}

// Copies the uplo triangle (1 upper, 2 lower) of the n x n matrix A onto the other one.
__global__ void symmetrize_kernel(int uplo, int n, double *A, int lda) {
    const long long total = (long long) n * n;
    for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x; e < total;
         e += (long long) gridDim.x * blockDim.x) {
        const int i = (int) (e % n), j = (int) (e / n);
        if (uplo == 1 && i > j) A[i + (size_t) j * lda] = A[j + (size_t) i * lda];
        if (uplo == 2 && i < j) A[i + (size_t) j * lda] = A[j + (size_t) i * lda];
    }
}

// Householder QR of A (m x n) in place, LAPACK dgeqr2 form: R on and above the diagonal, the
// reflectors v (v_i = 1 implicit) below it, tau[i].  One CTA; one warp per trailing column.
__global__ void __launch_bounds__(256) geqr2_kernel(int m, int n, double *A, int lda, double *tau) {
    __shared__ double red[8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int kmin = m < n ? m : n;
    for (int i = 0; i < kmin; i++) {
        double *ai = A + (size_t) i * lda;
        double a = 0.0;
        for (int r = i + 1 + threadIdx.x; r < m; r += blockDim.x) a = fma(ai[r], ai[r], a);
        const double sig2 = block_reduce(a, red);
        const double alpha = ai[i];
        double t = 0.0, beta = alpha;
        if (sig2 > 0.0) {
            beta = -copysign(sqrt(fma(alpha, alpha, sig2)), alpha);
            t = (beta - alpha) / beta;
            const double sc = 1.0 / (alpha - beta);
            for (int r = i + 1 + threadIdx.x; r < m; r += blockDim.x) ai[r] *= sc;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            ai[i] = beta;
            tau[i] = t;
        }
        __syncthreads();
        if (t != 0.0)
            for (int j = i + 1 + warp; j < n; j += nw) {
                double *aj = A + (size_t) j * lda;
                double w = lane == 0 ? aj[i] : 0.0;
                for (int r = i + 1 + lane; r < m; r += 32) w = fma(ai[r], aj[r], w);
                w = warp_sum(w) * t;
                if (lane == 0) aj[i] -= w;
                for (int r = i + 1 + lane; r < m; r += 32) aj[r] = fma(-w, ai[r], aj[r]);
            }
        __syncthreads();
    }
}

// LAPACK dorg2r: the first n columns of Q = H_0 ... H_{k-1} (reflectors in A's first k columns,
// m x n result in place).  One CTA.
__global__ void __launch_bounds__(256) org2r_kernel(int m, int n, int k, double *A, int lda, const double *tau) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    // columns k .. n-1 start as unit vectors
    for (int j = k; j < n; j++)
        for (int r = threadIdx.x; r < m; r += blockDim.x) A[r + (size_t) j * lda] = r == j ? 1.0 : 0.0;
    __syncthreads();
    for (int i = k - 1; i >= 0; i--) {
        const double *ai = A + (size_t) i * lda;
        const double t = tau[i];
        if (t != 0.0)
            for (int j = i + 1 + warp; j < n; j += nw) {
                double *aj = A + (size_t) j * lda;
                double w = lane == 0 ? aj[i] : 0.0;
                for (int r = i + 1 + lane; r < m; r += 32) w = fma(ai[r], aj[r], w);
                w = warp_sum(w) * t;
                if (lane == 0) aj[i] -= w;
                for (int r = i + 1 + lane; r < m; r += 32) aj[r] = fma(-w, ai[r], aj[r]);
            }
        __syncthreads();
        double *ci = A + (size_t) i * lda;
        for (int r = threadIdx.x; r < m; r += blockDim.x) {
            if (r < i) ci[r] = 0.0;
            else if (r == i) ci[r] = 1.0 - t;
            else ci[r] = -t * ci[r];
        }
        __syncthreads();
    }
}

// LAPACK dorm2r: C (m x n) <- op(Q) C (left) or C op(Q) (right), Q = H_0 ... H_{k-1} from geqr2
// (reflector i in column i of A, of length nq = m (left) or n (right)).  One CTA.
__global__ void __launch_bounds__(256) orm2r_kernel(int left, int trans, int m, int n, int k, const double *A,
                                                    int lda, const double *tau, double *C, int ldc) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    // Q^T C from the left applies H_0 first; Q C applies H_{k-1} first; on the right the reverse.
    const bool forward = (left && trans) || (!left && !trans);
    for (int s = 0; s < k; s++) {
        const int i = forward ? s : k - 1 - s;
        const double *v = A + (size_t) i * lda;
        const double t = tau[i];
        if (t != 0.0) {
            if (left) {  // rows i .. m-1 of every column j: c_j -= t v (v^T c_j)
                for (int j = warp; j < n; j += nw) {
                    double *cj = C + (size_t) j * ldc;
                    double w = lane == 0 ? cj[i] : 0.0;
                    for (int r = i + 1 + lane; r < m; r += 32) w = fma(v[r], cj[r], w);
                    w = warp_sum(w) * t;
                    if (lane == 0) cj[i] -= w;
                    for (int r = i + 1 + lane; r < m; r += 32) cj[r] = fma(-w, v[r], cj[r]);
                }
            } else {  // columns i .. n-1 of every row r: c_r -= t (c_r v) v^T
                for (int r = warp; r < m; r += nw) {
                    double w = lane == 0 ? C[r + (size_t) i * ldc] : 0.0;
                    for (int c = i + 1 + lane; c < n; c += 32) w = fma(C[r + (size_t) c * ldc], v[c], w);
                    w = warp_sum(w) * t;
                    if (lane == 0) C[r + (size_t) i * ldc] -= w;
                    for (int c = i + 1 + lane; c < n; c += 32) C[r + (size_t) c * ldc] = fma(-w, v[c], C[r + (size_t) c * ldc]);
                }
            }
        }
        __syncthreads();
    }
}

// B <- alpha op(A) T (left) or alpha T op(A) (right), A triangular, T = a copy of B (ld m).
__global__ void trmm_kernel(int left, int upper, int trans, int unit, int m, int n, double alpha, const double *A,
                            int lda, const double *T, double *B, int ldb) {
    const long long total = (long long) m * n;
    const int na = left ? m : n;
    for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x; e < total;
         e += (long long) gridDim.x * blockDim.x) {
        const int i = (int) (e % m), j = (int) (e / m);
        double s = 0.0;
        for (int q = 0; q < na; q++) {
            // left: sum_q op(A)[i, q] T[q, j]; right: sum_q T[i, q] op(A)[q, j]
            const int r = left ? i : q, c = left ? q : j;
            const int ar = trans ? c : r, ac = trans ? r : c;  // element of A itself
            double a;
            if (ar == ac) a = unit ? 1.0 : A[ar + (size_t) ac * lda];
            else if ((upper && ar < ac) || (!upper && ar > ac)) a = A[ar + (size_t) ac * lda];
            else continue;
            s = fma(a, left ? T[q + (size_t) j * m] : T[i + (size_t) q * m], s);
        }
        B[i + (size_t) j * ldb] = alpha * s;
    }
}

// One-sided Jacobi SVD (Hestenes) of X (rows x cols, rows >= cols, in place, ld ldx) with the
// rotations accumulated in V (cols x cols, ld ldv): X V = W with orthogonal columns; then
// sigma_j = ||w_j||.  Cyclic sweeps with a round-robin ordering of the pairs, one warp per pair,
// until no pair has |w_i . w_j| > tol ||w_i|| ||w_j|| (at most 60 sweeps).  *sweeps_out receives
// the sweep count (-1 if not converged).
__global__ void __launch_bounds__(256) jacobi_svd_kernel(int rows, int cols, double *X, int ldx, double *V, int ldv,
                                                        double tol, int *sweeps_out) {
    __shared__ int s_rot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int e = threadIdx.x; e < cols * cols; e += blockDim.x) {
        const int i = e % cols, j = e / cols;
        V[i + (size_t) j * ldv] = i == j ? 1.0 : 0.0;
    }
    const int n2 = cols + (cols & 1);
    int sweeps = 0;
    bool conv = cols < 2;
    while (!conv && sweeps < 60) {
        if (threadIdx.x == 0) s_rot = 0;
        __syncthreads();
        for (int t = 0; t < n2 - 1; t++) {
            for (int pp = warp; pp < n2 / 2; pp += nw) {
                int i, j;
                if (pp == 0) {
                    i = 0;
                    j = 1 + t % (n2 - 1);
                } else {
                    i = 1 + (pp + t) % (n2 - 1);
                    j = 1 + (n2 - 1 - pp + t) % (n2 - 1);
                }
                if (i >= cols || j >= cols) continue;
                double *xi = X + (size_t) i * ldx, *xj = X + (size_t) j * ldx;
                double a = 0.0, b = 0.0, c = 0.0;
                for (int r = lane; r < rows; r += 32) {
                    a = fma(xi[r], xi[r], a);
                    b = fma(xj[r], xj[r], b);
                    c = fma(xi[r], xj[r], c);
                }
                a = warp_sum(a);
                b = warp_sum(b);
                c = warp_sum(c);
                if (fabs(c) <= tol * sqrt(a * b) || c == 0.0) continue;
                const double zeta = (b - a) / (2.0 * c);
                const double tt = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double cs = 1.0 / sqrt(1.0 + tt * tt), sn = cs * tt;
                for (int r = lane; r < rows; r += 32) {
                    const double u = xi[r], w = xj[r];
                    xi[r] = cs * u - sn * w;
                    xj[r] = sn * u + cs * w;
                }
                double *vi = V + (size_t) i * ldv, *vj = V + (size_t) j * ldv;
                for (int r = lane; r < cols; r += 32) {
                    const double u = vi[r], w = vj[r];
                    vi[r] = cs * u - sn * w;
                    vj[r] = sn * u + cs * w;
                }
                if (lane == 0) atomicAdd(&s_rot, 1);
            }
            __syncthreads();
        }
        sweeps++;
        conv = s_rot == 0;
        __syncthreads();
    }
    if (threadIdx.x == 0) *sweeps_out = conv ? sweeps : -1;
}

// From X V = W: sigma (sorted descending), U = W_j / sigma_j and VT = V^T in the sorted order, for
// the first `kk` singular triples.  One CTA; perm in shared memory (cols <= 1024).
__global__ void __launch_bounds__(256) svd_finish_kernel(int rows, int cols, const double *X, int ldx,
                                                        const double *V, int ldv, double *S, double *U, int ldu,
                                                        double *VT, int ldvt, int kk, int want_u, int want_vt,
                                                        int transposed) {
    __shared__ double nrm[1024];
    __shared__ int perm[1024];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int j = warp; j < cols; j += nw) {
        const double *x = X + (size_t) j * ldx;
        double a = 0.0;
        for (int r = lane; r < rows; r += 32) a = fma(x[r], x[r], a);
        a = warp_sum(a);
        if (lane == 0) nrm[j] = sqrt(a);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < cols; j += blockDim.x) {
        int pos = 0;
        for (int l = 0; l < cols; l++) pos += nrm[l] > nrm[j] || (nrm[l] == nrm[j] && l < j);
        perm[pos] = j;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < kk; q += blockDim.x) S[q] = nrm[perm[q]];
    // A = X-side: U = W / sigma (rows x kk), VT = V^T (kk x cols).  When the SVD was taken of A^T the
    // roles swap: A^T = W S^-1 S V^T  =>  A = V S (W S^-1)^T, so U = V and VT = (W / sigma)^T.
    for (int e = threadIdx.x; e < rows * kk; e += blockDim.x) {
        const int r = e % rows, q = e / rows;
        const int j = perm[q];
        const double sj = nrm[j];
        const double w = sj > 0.0 ? X[r + (size_t) j * ldx] / sj : (r == q ? 1.0 : 0.0);
        if (!transposed && want_u) U[r + (size_t) q * ldu] = w;
        if (transposed && want_vt) VT[q + (size_t) r * ldvt] = w;
    }
    for (int e = threadIdx.x; e < cols * kk; e += blockDim.x) {
        const int r = e % cols, q = e / cols;
        const double v = V[r + (size_t) perm[q] * ldv];
        if (!transposed && want_vt) VT[q + (size_t) r * ldvt] = v;
        if (transposed && want_u) U[r + (size_t) q * ldu] = v;
    }
}

int grid_for(long long total) {
    const long long b = (total + 255) / 256;
    return (int) (b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

}  // namespace

void be_copy(cudaStream_t st, int trans, int m, int n, double alpha, const double *A, int lda, double *B, int ldb) {
    if (m > 0 && n > 0) { copy_kernel<<<grid_for((long long) m * n), 256, 0, st>>>(trans, m, n, alpha, A, lda, B, ldb); note_launch(); }
}
void be_lacpy(cudaStream_t st, int uplo, int m, int n, const double *A, int lda, double *B, int ldb) {
    if (m > 0 && n > 0) { lacpy_kernel<<<grid_for((long long) m * n), 256, 0, st>>>(uplo, m, n, A, lda, B, ldb); note_launch(); }
}
void be_laset(cudaStream_t st, int uplo, int m, int n, double offdiag, double diag, double *A, int lda) {
    if (m > 0 && n > 0) { laset_kernel<<<grid_for((long long) m * n), 256, 0, st>>>(uplo, m, n, offdiag, diag, A, lda); note_launch(); }
}
void be_scale_rows(cudaStream_t st, int rows, int cols, const double *s, double *A, int lda) {
    if (rows > 0 && cols > 0) { scale_rows_kernel<<<grid_for((long long) rows * cols), 256, 0, st>>>(rows, cols, s, A, lda); note_launch(); }
}
void be_symmetrize(cudaStream_t st, int uplo, int n, double *A, int lda) {
    if (n > 0) { symmetrize_kernel<<<grid_for((long long) n * n), 256, 0, st>>>(uplo, n, A, lda); note_launch(); }
}
void be_geqr2(cudaStream_t st, int m, int n, double *A, int lda, double *tau) {
    if (m > 0 && n > 0) { geqr2_kernel<<<1, 256, 0, st>>>(m, n, A, lda, tau); note_launch(); }
}
void be_org2r(cudaStream_t st, int m, int n, int k, double *A, int lda, const double *tau) {
    if (m > 0 && n > 0) { org2r_kernel<<<1, 256, 0, st>>>(m, n, k, A, lda, tau); note_launch(); }
}
void be_orm2r(cudaStream_t st, int left, int trans, int m, int n, int k, const double *A, int lda, const double *tau,
              double *C, int ldc) {
    if (m > 0 && n > 0 && k > 0) { orm2r_kernel<<<1, 256, 0, st>>>(left, trans, m, n, k, A, lda, tau, C, ldc); note_launch(); }
}
void be_trmm(cudaStream_t st, int left, int upper, int trans, int unit, int m, int n, double alpha, const double *A,
             int lda, const double *T, double *B, int ldb) {
    if (m > 0 && n > 0) { trmm_kernel<<<grid_for((long long) m * n), 256, 0, st>>>(left, upper, trans, unit, m, n, alpha, A, lda, T, B, ldb); note_launch(); }
}
void be_jacobi_svd(cudaStream_t st, int rows, int cols, double *X, int ldx, double *V, int ldv, double tol, int *sweeps) {
    { jacobi_svd_kernel<<<1, 256, 0, st>>>(rows, cols, X, ldx, V, ldv, tol, sweeps); note_launch(); }
}
void be_svd_finish(cudaStream_t st, int rows, int cols, const double *X, int ldx, const double *V, int ldv, double *S,
                   double *U, int ldu, double *VT, int ldvt, int kk, int want_u, int want_vt, int transposed) {
    { svd_finish_kernel<<<1, 256, 0, st>>>(rows, cols, X, ldx, V, ldv, S, U, ldu, VT, ldvt, kk, want_u, want_vt, transposed); note_launch(); }
}

}  // namespace hcgb
