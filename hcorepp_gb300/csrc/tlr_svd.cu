// Core of the recompression: M = R_U R_V^T, its SVD by one-sided Jacobi, the rank
// truncation, and the new left/right factors in the small basis.
//
// Replaces the R extraction + core GEMM + SVD + CalculateNewRank + CalculateVTnew of
// CompressedTile<T>::Gemm (src/operators/concrete/Compressed.cpp:441-527, :597-599) and the
// host-synchronising rank scan of the CUDA backend (src/kernels/cuda/CudaKernels.cu:656-697).
//
// One CTA per update.  One-sided Jacobi rotates pairs of columns of M (round-robin parallel
// ordering, one warp per pair, warp-shuffle dot products) until every pair is orthogonal to
// working precision: M J = W, sigma_j = ||w_j||, left vectors Ut = W Sigma^-1.  The right
// factor is formed as Z = M^T Ut_r (= V_r Sigma_r), so the rotations never need accumulating.
// The rank rule is the reference's (omp/kernels.cpp:82-104) applied to the sorted sigma.
#include <cfloat>

#include "internal.cuh"

namespace hcgb {

namespace {

constexpr int SVD_THREADS = 256;

__device__ __forceinline__ void jacobi_pair(int t, int pp, int n2, int &i, int &j) {
    const int nm1 = n2 - 1;
    if (pp == 0) {
        i = 0;
        j = 1 + t % nm1;
    } else {
        i = 1 + (pp + t) % nm1;
        j = 1 + (n2 - 1 - pp + t) % nm1;
    }
}

// Rotate columns x, y (length rows <= 32*RPL) so that x^T y = 0; true if a rotation was applied.
template <int RPL>
__device__ bool rotate_pair(double *x, double *y, int rows, double tol) {
    const int lane = threadIdx.x & 31;
    double xr[RPL], yr[RPL];
    double a = 0.0, b = 0.0, c = 0.0;
#pragma unroll
    for (int q = 0; q < RPL; q++) {
        const int r = lane + 32 * q;
        xr[q] = r < rows ? x[r] : 0.0;
        yr[q] = r < rows ? y[r] : 0.0;
        a = fma(xr[q], xr[q], a);
        b = fma(yr[q], yr[q], b);
        c = fma(xr[q], yr[q], c);
    }
    a = warp_sum(a);
    b = warp_sum(b);
    c = warp_sum(c);
    if (!(fabs(c) > tol * sqrt(a) * sqrt(b))) return false;
    const double zeta = (b - a) / (2.0 * c);
    const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.0)));
    const double cs = 1.0 / sqrt(fma(t, t, 1.0));
    const double sn = cs * t;
#pragma unroll
    for (int q = 0; q < RPL; q++) {
        const int r = lane + 32 * q;
        if (r < rows) {
            x[r] = fma(cs, xr[q], -sn * yr[q]);
            y[r] = fma(sn, xr[q], cs * yr[q]);
        }
    }
    return true;
}

template <int RPL>
__global__ void __launch_bounds__(SVD_THREADS) core_svd_kernel(const DevUpdate *ups, Workspace ws, Params p,
                                                               int smem_doubles) {
    extern __shared__ double sm[];
    __shared__ int s_rot, s_rank;
    const int slot = blockIdx.x;
    int *meta = ws.meta + (size_t) slot * META_INTS;
    if (meta[META_STATUS] != HCGB_OK || !meta[META_CKIND]) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int lr = lane >> 2, lc = lane & 3;
    const int k = meta[META_K], m = meta[META_M], n = meta[META_N];
    const int kU = m < k ? m : k, kV = n < k ? n : k;
    const int ld = ws.ld, ldm = ws.kmax;
    double *base = ws.slot(slot);
    const double *RU = base + ws.off_ustack;
    const double *RV = base + ws.off_vstack;
    double *Mc = base + ws.off_mcopy;
    // Aux arrays at the start of shared memory: sigma, 1/sigma (sorted), permutation.
    double *sig = sm;
    double *inv = sig + ws.kmax;
    int *perm = reinterpret_cast<int *>(inv + ws.kmax);
    double *pool = inv + ws.kmax + (ws.kmax + 1) / 2 + 1;
    const int pool_doubles = smem_doubles - (int) (pool - sm);
    // Working copy of M: shared memory when it fits, else the workspace.
    double *Mw;
    int ldw;
    if ((long) kU * kV <= (long) pool_doubles) {
        Mw = pool;
        ldw = kU;
    } else {
        Mw = base + ws.off_m;
        ldw = ldm;
    }

    // 1. M = R_U R_V^T on DMMA (R_U = triu of the U stack's top kU rows, likewise R_V).
    {
        const int ntr = (kU + 7) >> 3, ntc = (kV + 7) >> 3;
        for (int idx = warp; idx < ntr * ntc; idx += nw) {
            const int tr = idx % ntr, tc = idx / ntr;
            const int i = tr * 8 + lr, j = tc * 8 + lr;
            double d0 = 0.0, d1 = 0.0;
            const int l0 = ((tr > tc ? tr : tc) * 8) & ~3;
            for (int l4 = l0; l4 < k; l4 += 4) {
                const int l = l4 + lc;
                const double av = (i < kU && l < k && l >= i) ? RU[i + (size_t) l * ld] : 0.0;
                const double bv = (j < kV && l < k && l >= j) ? RV[j + (size_t) l * ld] : 0.0;
                dmma(d0, d1, av, bv);
            }
            const int col = tc * 8 + 2 * lc;
            if (i < kU && col < kV) {
                Mw[i + (size_t) col * ldw] = d0;
                Mc[i + (size_t) col * ldm] = d0;
            }
            if (i < kU && col + 1 < kV) {
                Mw[i + (size_t) (col + 1) * ldw] = d1;
                Mc[i + (size_t) (col + 1) * ldm] = d1;
            }
        }
    }
    __syncthreads();

    // 2. One-sided Jacobi on the kV columns of M.
    const double tol = DBL_EPSILON * sqrt((double) (kU > 1 ? kU : 1));
    const int n2 = kV + (kV & 1);
    int sweeps = 0;
    bool converged = (kV < 2);
    while (!converged && sweeps < MAX_JACOBI_SWEEPS) {
        if (threadIdx.x == 0) s_rot = 0;
        __syncthreads();
        for (int t = 0; t < n2 - 1; t++) {
            for (int pp = warp; pp < n2 / 2; pp += nw) {
                int i, j;
                jacobi_pair(t, pp, n2, i, j);
                if (i >= kV || j >= kV) continue;
                const bool rot = rotate_pair<RPL>(Mw + (size_t) i * ldw, Mw + (size_t) j * ldw, kU, tol);
                if (rot && lane == 0) atomicAdd(&s_rot, 1);
            }
            __syncthreads();
        }
        sweeps++;
        converged = (s_rot == 0);
        __syncthreads();
    }

    // 3. Singular values, descending order (stable), rank.
    for (int j = warp; j < kV; j += nw) {
        const double *col = Mw + (size_t) j * ldw;
        double s = 0.0;
        for (int r = lane; r < kU; r += 32) s = fma(col[r], col[r], s);
        s = warp_sum(s);
        if (lane == 0) inv[j] = sqrt(s);  // unsorted sigma, temporarily in inv[]
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kV; j += blockDim.x) {
        const double sj = inv[j];
        int pos = 0;
        for (int l = 0; l < kV; l++) {
            const double sl = inv[l];
            pos += (sl > sj) || (sl == sj && l < j);
        }
        perm[pos] = j;
        sig[pos] = sj;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int sizeS = kU < kV ? kU : kV;
        int r;
        if (p.fixed_rank > 0) {
            r = p.fixed_rank < k ? p.fixed_rank : k;
        } else {
            r = sizeS;
            const double thr = p.truncated ? p.accuracy * sig[0] : p.accuracy;
            for (int i = 1; i < sizeS; i++)
                if (sig[i] < thr) {
                    r = i;
                    break;
                }
        }
        if (r < 1) r = 1;
        const int maxr = ups[slot].c.max_rank;
        if (r > maxr) r = maxr;
        if (r > sizeS) r = sizeS;
        s_rank = r;
        meta[META_NEWRANK] = r;
        meta[META_SWEEPS] = sweeps;
        if (!converged) meta[META_STATUS] = HCGB_NOT_CONVERGED;
    }
    __syncthreads();
    const int r = s_rank;
    for (int i = threadIdx.x; i < r; i += blockDim.x) inv[i] = sig[i] > 0.0 ? 1.0 / sig[i] : 0.0;
    __syncthreads();

    // 4. New left factor in the small basis: C.U[:, i] = [w_perm(i) / sigma_i ; 0] (m rows).
    double *CU = ups[slot].c.data;
    const int ldcu = ups[slot].c.rows;
    for (int i = warp; i < r; i += nw) {
        const double *col = Mw + (size_t) perm[i] * ldw;
        const double s = inv[i];
        for (int l = lane; l < m; l += 32) CU[l + (size_t) i * ldcu] = l < kU ? col[l] * s : 0.0;
    }
    // 5. Right factor Z = M^T Ut_r (kV x r) into XV (n rows, zero below kV), on DMMA.
    double *XV = base + ws.off_xv;
    {
        const int ntr = (kV + 7) >> 3, ntc = (r + 7) >> 3;
        for (int idx = warp; idx < ntr * ntc; idx += nw) {
            const int tr = idx % ntr, tc = idx / ntr;
            const int jrow = tr * 8 + lr, icol = tc * 8 + lr;
            const double *ucol = Mw + (size_t) perm[icol < r ? icol : 0] * ldw;
            const double us = icol < r ? inv[icol] : 0.0;
            double d0 = 0.0, d1 = 0.0;
            for (int l4 = 0; l4 < kU; l4 += 4) {
                const int l = l4 + lc;
                const double av = (jrow < kV && l < kU) ? Mc[l + (size_t) jrow * ldm] : 0.0;
                const double bv = (l < kU) ? ucol[l] * us : 0.0;
                dmma(d0, d1, av, bv);
            }
            const int col = tc * 8 + 2 * lc;
            if (jrow < kV && col < r) XV[jrow + (size_t) col * ld] = d0;
            if (jrow < kV && col + 1 < r) XV[jrow + (size_t) (col + 1) * ld] = d1;
        }
        for (int i = warp; i < r; i += nw)
            for (int l = kV + lane; l < n; l += 32) XV[l + (size_t) i * ld] = 0.0;
    }
}

}  // namespace

size_t svd_smem_bytes(int kmax) {
    size_t aux = (size_t) 2 * kmax + (kmax + 1) / 2 + 1;
    size_t want = aux + (size_t) kmax * kmax;
    const size_t cap = 200 * 1024 / sizeof(double);
    if (want > cap) want = cap;
    return want * sizeof(double);
}

template <int RPL>
static void launch_core_svd_t(const DevUpdate *ups, int n, Workspace ws, Params p, cudaStream_t st) {
    const size_t smem = svd_smem_bytes(ws.kmax);
    cudaFuncSetAttribute(core_svd_kernel<RPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    core_svd_kernel<RPL><<<n, SVD_THREADS, smem, st>>>(ups, ws, p, (int) (smem / sizeof(double)));
}

// Rows of M are at most min(ld, kmax); the register tile of a rotation covers 32 * RPL rows.
void launch_core_svd(const DevUpdate *ups, int n, Workspace ws, Params p, cudaStream_t st) {
    const int rows = ws.ld < ws.kmax ? ws.ld : ws.kmax;
    if (rows <= 128) launch_core_svd_t<4>(ups, n, ws, p, st);
    else if (rows <= 256) launch_core_svd_t<8>(ups, n, ws, p, st);
    else if (rows <= 512) launch_core_svd_t<16>(ups, n, ws, p, st);
    else launch_core_svd_t<32>(ups, n, ws, p, st);
}

}  // namespace hcgb
