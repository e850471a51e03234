// Planning, stacking, factor products (FP64 DMMA GEMM; the larger ones go to oz_gemm.cu),
// the plain form's full-WY Q application, ordering and write-back of a batch of TLR tile
// updates.  Follows HCore<T>::Gemm's dispatch (src/api/HCore.cpp:23-344) and the
// stacking of CompressedTile<T>::Gemm (src/operators/concrete/Compressed.cpp:331-379).
#include "internal.cuh"

namespace hcgb {

namespace {

__device__ __forceinline__ GemmJob make_job(const double *A, int lda, int opA, const double *B, int ldb, int opB,
                                            double *C, int ldc, int M, int N, int K, double alpha, double beta) {
    GemmJob j;
    j.A = A;
    j.B = B;
    j.C = C;
    j.M = M;
    j.N = N;
    j.K = K;
    j.lda = lda < 1 ? 1 : lda;
    j.ldb = ldb < 1 ? 1 : ldb;
    j.ldc = ldc < 1 ? 1 : ldc;
    j.opA = opA;
    j.opB = opB;
    j.alpha = alpha;
    j.beta = beta;
    j.oz = 0;
    j.triA = j.triB = 0;
    j.prec = 0;
    return j;
}

// One thread per update: read ranks on the device, validate, choose the stacking side and
// emit up to three dependent GEMM jobs (phase 1, 2, 3).
__device__ void plan_update(const DevUpdate *ups, int n, double alpha, double beta, Workspace ws, Params p,
                            GemmJob *jobs, int s);

__global__ void plan_kernel(const DevUpdate *ups, int n, double alpha, double beta, Workspace ws, Params p,
                            GemmJob *jobs) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    plan_update(ups, n, alpha, beta, ws, p, jobs, s);
    // Low-precision forms: every product on tcgen05 in TF32 / BF16; otherwise the large products go
    // to the FP64-accurate tensor-core path.
    const int lp = lowp_prec(p.mode);
    for (int ph = 0; ph < 3; ph++) {
        GemmJob &j = jobs[(size_t) ph * n + s];
        j.prec = (lp && j.M > 0 && j.N > 0) ? lp : 0;
        j.oz = (!j.prec && p.oz && j.M > 0 && j.N > 0 && oz_shape(j.M, j.N, j.K, p.oz_min)) ? 1 : 0;
    }
}

__device__ void plan_update(const DevUpdate *ups, int n, double alpha, double beta, Workspace ws, Params p,
                            GemmJob *jobs, int s) {
    const DevUpdate u = ups[s];
    int *meta = ws.meta + (size_t) s * META_INTS;
    GemmJob none;
    none.M = 0;
    none.N = 0;
    none.K = 0;
    jobs[s] = none;
    jobs[n + s] = none;
    jobs[2 * n + s] = none;
    for (int f = 0; f < META_INTS; f++) meta[f] = 0;

    const int ak = u.a.kind, bk = u.b.kind, ck = u.c.kind;
    const int rA = ak ? *u.a.rank : 0;
    const int rB = bk ? *u.b.rank : 0;
    const int rC = ck ? *u.c.rank : 0;
    const int m = u.c.rows, nn = u.c.cols, kd = u.a.cols;
    int status = HCGB_OK;
    if (u.a.rows != m || u.b.cols != nn || u.b.rows != kd) status = HCGB_BAD_ARG;
    if ((ak && (rA < 0 || rA > u.a.max_rank)) || (bk && (rB < 0 || rB > u.b.max_rank)) ||
        (ck && (rC < 0 || rC > u.c.max_rank)))
        status = HCGB_RANK_OVERFLOW;
    if (!ak && !bk && ck) status = HCGB_UNSUPPORTED;  // DDC: hcgb_tile_gemm only
    if (m > ws.ld || nn > ws.ld || rA > ws.rmax || rB > ws.rmax) status = HCGB_POOL_TOO_SMALL;
    meta[META_CKIND] = ck;
    meta[META_RA] = rA;
    meta[META_RB] = rB;
    meta[META_RC] = rC;
    meta[META_M] = m;
    meta[META_N] = nn;
    if (status != HCGB_OK) {
        meta[META_STATUS] = status;
        return;
    }
    double *slot = ws.slot(s);
    double *Us = slot + ws.off_ustack;
    double *Vs = slot + ws.off_vstack;
    double *T1 = slot + ws.off_tmp1;  // rmax x rmax, ld rmax
    double *T2 = slot + ws.off_tmp2;  // ld x rmax (ld ld) or rmax x ld (ld rmax)
    const int ld = ws.ld, lr = ws.rmax;
    // Compressed views: U at data (ld rows), V region at v (ld rank, or ld cols when compressed_vt).
    const double *Au = u.a.data, *Av = u.a.v;
    const double *Bu = u.b.data, *Bv = u.b.v;
    const double *Ad = u.a.data, *Bd = u.b.data;
    // V factors as GEMM operands: V (rank x cols, ld rank), or for a compressed_vt tile the stored
    // W = V^T (cols x rank, ld cols) read with the opposite op.
    const int avt = ak == HCGB_COMPRESSED_VT, bvt = bk == HCGB_COMPRESSED_VT;
    const int lav = avt ? u.a.cols : rA, lbv = bvt ? u.b.cols : rB;

    if (ck) {
        int side = 0, k = 0;
        if (ak && bk) {
            side = (p.side_mode && rB < rA) ? 1 : 0;
            jobs[s] = make_job(Av, lav, avt, Bu, kd, 0, T1, lr, rA, rB, kd, 1.0, 0.0);  // T1 = Av Bu
            if (side == 0) {
                // V[:, rC:rC+rA] = (T1 Bv)^T = Bv^T T1^T   (ProcessVpointer's B part)
                jobs[n + s] = make_job(Bv, lbv, !bvt, T1, lr, 1, Vs + (size_t) rC * ld, ld, nn, rA, rB, 1.0, 0.0);
                k = rC + rA;
            } else {
                // U[:, rC:rC+rB] = alpha Au T1
                jobs[n + s] = make_job(Au, m, 0, T1, lr, 0, Us + (size_t) rC * ld, ld, m, rB, rA, alpha, 0.0);
                k = rC + rB;
            }
        } else if (!ak && bk) {
            side = 1;  // DCC: U[:, rC:] = alpha A Bu, V[:, rC:] = Bv^T (HCore.cpp:234-245)
            jobs[s] = make_job(Ad, m, 0, Bu, kd, 0, Us + (size_t) rC * ld, ld, m, rB, kd, alpha, 0.0);
            k = rC + rB;
        } else {
            side = 0;  // CDC: U[:, rC:] = alpha Au, V[:, rC:] = (Av B)^T = B^T Av^T (HCore.cpp:246-257)
            jobs[s] = make_job(Bd, kd, 1, Av, lav, !avt, Vs + (size_t) rC * ld, ld, nn, rA, kd, 1.0, 0.0);
            k = rC + rA;
        }
        if (k > ws.kmax) status = HCGB_POOL_TOO_SMALL;
        if (k == 0) status = HCGB_BAD_ARG;
        meta[META_SIDE] = side;
        meta[META_K] = k;
        if (status != HCGB_OK) {
            jobs[s] = none;
            jobs[n + s] = none;
            meta[META_STATUS] = status;
        }
        return;
    }
    // Dense C: plain GEMM chains, C <- alpha * left * right + beta * C.
    double *C = u.c.data;
    if (ak && bk) {
        jobs[s] = make_job(Av, lav, avt, Bu, kd, 0, T1, lr, rA, rB, kd, 1.0, 0.0);
        if (!p.side_mode || rA <= rB) {
            // HCore.cpp:178-264: T2 = T1 Bv, C = alpha Au T2 + beta C
            jobs[n + s] = make_job(T1, lr, 0, Bv, lbv, bvt, T2, lr, rA, nn, rB, 1.0, 0.0);
            jobs[2 * n + s] = make_job(Au, m, 0, T2, lr, 0, C, m, m, nn, rA, alpha, beta);
        } else {
            jobs[n + s] = make_job(Au, m, 0, T1, lr, 0, T2, ld, m, rB, rA, 1.0, 0.0);
            jobs[2 * n + s] = make_job(T2, ld, 0, Bv, lbv, bvt, C, m, m, nn, rB, alpha, beta);
        }
    } else if (!ak && bk) {
        jobs[s] = make_job(Ad, m, 0, Bu, kd, 0, T2, ld, m, rB, kd, 1.0, 0.0);  // DCD
        jobs[2 * n + s] = make_job(T2, ld, 0, Bv, lbv, bvt, C, m, m, nn, rB, alpha, beta);
    } else if (ak && !bk) {
        jobs[s] = make_job(Av, lav, avt, Bd, kd, 0, T2, lr, rA, nn, kd, 1.0, 0.0);  // CDD
        jobs[2 * n + s] = make_job(Au, m, 0, T2, lr, 0, C, m, m, nn, rA, alpha, beta);
    } else {
        jobs[2 * n + s] = make_job(Ad, m, 0, Bd, kd, 0, C, m, m, nn, kd, alpha, beta);  // DDD
    }
}

// dst[j + i*ldd] = scale * src[i + j*lds] for i < rows(src), j < cols(src): a transposed copy
// through a 32x33 shared tile so that both sides stay coalesced.
__device__ void transpose_scaled(const double *src, int lds, int rows, int cols, double *dst, int ldd,
                                 double scale, double (*tile)[33]) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, nty = blockDim.x >> 5;
    for (int i0 = 0; i0 < rows; i0 += 32)
        for (int j0 = 0; j0 < cols; j0 += 32) {
            for (int jj = ty; jj < 32; jj += nty) {
                int i = i0 + tx, j = j0 + jj;
                tile[jj][tx] = (i < rows && j < cols) ? src[i + (size_t) j * lds] : 0.0;
            }
            __syncthreads();
            for (int ii = ty; ii < 32; ii += nty) {
                int i = i0 + ii, j = j0 + tx;
                if (i < rows && j < cols) dst[j + (size_t) i * ldd] = scale * tile[tx][ii];
            }
            __syncthreads();
        }
}

__device__ void copy_scaled(const double *src, int lds, int rows, int cols, double *dst, int ldd, double scale) {
    for (int j = 0; j < cols; j++)
        for (int i = threadIdx.x; i < rows; i += blockDim.x)
            dst[i + (size_t) j * ldd] = scale * src[i + (size_t) j * lds];
}

// One CTA per update: the parts of the stacks that are copies of existing factors
// (LaCpy + MultiplyByAlpha + ProcessVpointer, Compressed.cpp:331-379).
__global__ void __launch_bounds__(256) stack_kernel(const DevUpdate *ups, double alpha, double beta, Workspace ws) {
    __shared__ double tile[32][33];
    const int s = blockIdx.x;
    const int *meta = ws.meta + (size_t) s * META_INTS;
    if (meta[META_STATUS] != HCGB_OK || !meta[META_CKIND]) return;
    const DevUpdate u = ups[s];
    const int m = meta[META_M], nn = meta[META_N], rA = meta[META_RA], rB = meta[META_RB], rC = meta[META_RC];
    const int side = meta[META_SIDE];
    double *slot = ws.slot(s);
    double *Us = slot + ws.off_ustack;
    double *Vs = slot + ws.off_vstack;
    const int ld = ws.ld;
    const double *Cu = u.c.data, *Cv = u.c.v;
    copy_scaled(Cu, m, m, rC, Us, ld, 1.0);                                      // U[:, :rC] = Cu
    if (side == 0 && u.a.kind) copy_scaled(u.a.data, m, m, rA, Us + (size_t) rC * ld, ld, alpha);  // alpha Au
    // V[:, :rC] = beta Cv^T; a compressed_vt C stores Cv^T itself (ProcessVpointer's Cholesky copy)
    if (u.c.kind == HCGB_COMPRESSED_VT) copy_scaled(Cv, nn, nn, rC, Vs, ld, beta);
    else transpose_scaled(Cv, rC, rC, nn, Vs, ld, beta, tile);
    if (side == 1 && u.b.kind) {
        const double *Bv = u.b.v;
        if (u.b.kind == HCGB_COMPRESSED_VT) copy_scaled(Bv, nn, nn, rB, Vs + (size_t) rC * ld, ld, 1.0);
        else transpose_scaled(Bv, rB, rB, nn, Vs + (size_t) rC * ld, ld, 1.0, tile);  // V[:, rC:] = Bv^T
    }
}

// ---------------------------------------------------------------------------------------
// Batched FP64 GEMM on DMMA: one 64x64 tile of C per CTA, 4 warps (2x2) of 32x32, k-chunks
// of 16 staged in shared memory.  Grid: x = tile index within the job, y = job.
// ---------------------------------------------------------------------------------------
constexpr int GT = 64, GK = 16, AS_LD = GK + 4, BS_LD = GT + 4;

// One 64 x 64 output tile of one job.
__device__ void gemm_tile(const GemmJob &jb, int tile, double (*As)[AS_LD], double (*Bs)[BS_LD]) {
    const int ntm = (jb.M + GT - 1) / GT;
    const int m0 = (tile % ntm) * GT, n0 = (tile / ntm) * GT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int lr = lane >> 2, lc = lane & 3;
    // Warp w owns 8-row blocks w and w + 4 of the tile and all eight 8-column blocks, so a small
    // job (say 30 x 30) still spreads over the four warps -- one per SM sub-partition and FP64
    // pipe -- instead of landing on one warp.
    const int rb0 = warp, rb1 = warp + 4;
    const int rem_m = jb.M - m0, rem_n = jb.N - n0;
    const bool r0ok = rb0 * 8 < rem_m, r1ok = rb1 * 8 < rem_m;
    const int nblk = rem_n <= 0 ? 0 : (rem_n >= 64 ? 8 : (rem_n + 7) >> 3);
    double acc[2][8][2];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j][0] = acc[i][j][1] = 0.0;

    for (int k0 = 0; k0 < jb.K; k0 += GK) {
        for (int e = threadIdx.x; e < GT * GK; e += blockDim.x) {
            int i, kk;
            if (jb.opA == 0) {
                i = e % GT;
                kk = e / GT;
            } else {
                kk = e % GK;
                i = e / GK;
            }
            const int gi = m0 + i, gk = k0 + kk;
            As[i][kk] = (gi < jb.M && gk < jb.K) ? job_a(jb, gi, gk) : 0.0;
        }
        for (int e = threadIdx.x; e < GT * GK; e += blockDim.x) {
            int j, kk;
            if (jb.opB == 0) {
                kk = e % GK;
                j = e / GK;
            } else {
                j = e % GT;
                kk = e / GT;
            }
            const int gj = n0 + j, gk = k0 + kk;
            Bs[kk][j] = (gj < jb.N && gk < jb.K) ? job_b(jb, gk, gj) : 0.0;
        }
        __syncthreads();
        // The FP64 pipe is the limit: no MMA is issued for 8x8 blocks or k-steps that lie wholly
        // outside the job (small factor products fill a fraction of the 64x64 tile).  All
        // conditions are warp-uniform.
        const int kend = jb.K - k0 < GK ? jb.K - k0 : GK;
#pragma unroll
        for (int kk = 0; kk < GK; kk += 4) {
            if (kk >= kend) break;
            const double af0 = As[rb0 * 8 + lr][kk + lc], af1 = As[rb1 * 8 + lr][kk + lc];
            double bf[8];
#pragma unroll
            for (int j = 0; j < 8; j++) bf[j] = Bs[kk + lc][j * 8 + lr];
#pragma unroll
            for (int j = 0; j < 8; j++)
                if (j < nblk) {
                    if (r0ok) dmma(acc[0][j][0], acc[0][j][1], af0, bf[j]);
                    if (r1ok) dmma(acc[1][j][0], acc[1][j][1], af1, bf[j]);
                }
        }
        __syncthreads();
    }
    const bool scale = jb.alpha != 1.0, accum = jb.beta != 0.0;
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 8; j++)
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int row = m0 + (i ? rb1 : rb0) * 8 + lr;
                const int col = n0 + j * 8 + 2 * lc + e;
                if (row < jb.M && col < jb.N) {
                    double *c = jb.C + row + (size_t) col * jb.ldc;
                    double v = scale ? jb.alpha * acc[i][j][e] : acc[i][j][e];
                    if (accum) v = fma(jb.beta, *c, v);
                    *c = v;
                }
            }
}

// Tiles of the FP64 jobs, compacted (sched: exclusive prefix of tiles per job, njobs + 1 entries);
// a grid sized to the GPU strides over them, so empty or small jobs cost no CTA launches.
__global__ void __launch_bounds__(128) gemm_jobs_kernel(const GemmJob *jobs, int njobs, const int *sched) {
    __shared__ double As[GT][AS_LD];
    __shared__ double Bs[GK][BS_LD];
    const int total = sched[njobs];
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        int lo = 0, hi = njobs;  // sched[lo] <= w < sched[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (sched[mid] <= w) lo = mid;
            else hi = mid;
        }
        const GemmJob jb = jobs[lo];
        gemm_tile(jb, w - sched[lo], As, Bs);
        __syncthreads();
    }
}

// Tile counts of every job for the three GEMM kernels and their exclusive prefix sums:
// sched[0 .. njobs] (FP64 DMMA, 64 x 64 tiles), sched[njobs + 1 .. 2 njobs + 1] (FP64-accurate
// tensor-core path, 128 x 64 tiles) and sched[2 njobs + 2 .. 3 njobs + 2] (TF32 / BF16 on tcgen05,
// 128 x 64 tiles).  One CTA; njobs up to 4 * 1024.
__global__ void __launch_bounds__(1024) schedule_kernel(const GemmJob *jobs, int njobs, int *sched) {
    constexpr int NL = 3;
    __shared__ int part[NL][1024];
    constexpr int PER = 4;
    int cnt[NL][PER], sum[NL] = {0, 0, 0};
    for (int q = 0; q < PER; q++) {
        const int j = threadIdx.x * PER + q;
        for (int l = 0; l < NL; l++) cnt[l][q] = 0;
        if (j < njobs) {
            const GemmJob &jb = jobs[j];
            if (jb.M > 0 && jb.N > 0 && jb.K >= 0) {
                if (jb.prec) cnt[2][q] = ((jb.M + 127) / 128) * ((jb.N + 63) / 64);
                else if (jb.oz) cnt[1][q] = ((jb.M + 127) / 128) * ((jb.N + 63) / 64);
                else cnt[0][q] = ((jb.M + GT - 1) / GT) * ((jb.N + GT - 1) / GT);
            }
        }
        for (int l = 0; l < NL; l++) sum[l] += cnt[l][q];
    }
    for (int l = 0; l < NL; l++) part[l][threadIdx.x] = sum[l];
    __syncthreads();
    // inclusive scan of the per-thread sums (Hillis-Steele over 1024 entries)
    for (int off = 1; off < 1024; off <<= 1) {
        int add[NL];
        for (int l = 0; l < NL; l++) add[l] = threadIdx.x >= off ? part[l][threadIdx.x - off] : 0;
        __syncthreads();
        for (int l = 0; l < NL; l++) part[l][threadIdx.x] += add[l];
        __syncthreads();
    }
    int run[NL];
    for (int l = 0; l < NL; l++) run[l] = part[l][threadIdx.x] - sum[l];  // exclusive starts
    for (int q = 0; q < PER; q++) {
        const int j = threadIdx.x * PER + q;
        if (j < njobs)
            for (int l = 0; l < NL; l++) sched[l * (njobs + 1) + j] = run[l];
        for (int l = 0; l < NL; l++) run[l] += cnt[l][q];
    }
    if (threadIdx.x == 1023)
        for (int l = 0; l < NL; l++) sched[l * (njobs + 1) + njobs] = part[l][1023];
}

// One CTA per update: V (r x n, ld r) = XV^T into the tile buffer, publish rank and record.
__global__ void __launch_bounds__(256) finalize_kernel(const DevUpdate *ups, Workspace ws, hcgb_update_info *info) {
    __shared__ double tile[32][33];
    const int s = blockIdx.x;
    const int *meta = ws.meta + (size_t) s * META_INTS;
    const int status = meta[META_STATUS];
    const bool ok = (status == HCGB_OK || status == HCGB_NOT_CONVERGED) && meta[META_CKIND];
    if (info && threadIdx.x == 0) {
        hcgb_update_info r;
        r.status = status;
        r.rank_a = meta[META_RA];
        r.rank_b = meta[META_RB];
        r.rank_c = meta[META_RC];
        r.k = meta[META_CKIND] ? meta[META_K] : 0;
        r.new_rank = ok ? meta[META_NEWRANK] : 0;
        r.sweeps = meta[META_SWEEPS];
        r.side = meta[META_SIDE];
        r.core_cols = meta[META_CORE_COLS];
        for (int q = 0; q < 4; q++) r.core_kcycles[q] = meta[META_KC_PRODUCT + q];
        r.sketch_cols = meta[META_LSK];
        r.sketch_accepted = meta[META_SK_ACC];
        info[ups[s].uid] = r;
    }
    if (!ok) return;
    const DevUpdate u = ups[s];
    const int r = meta[META_NEWRANK], nn = meta[META_N];
    const double *XV = ws.slot(s) + ws.off_xv;
    double *Cv = u.c.v;
    if (u.c.kind == HCGB_COMPRESSED_VT) copy_scaled(XV, ws.ld, nn, r, Cv, nn, 1.0);  // W = XV (n x r, ld n)
    else transpose_scaled(XV, ws.ld, nn, r, Cv, r, 1.0, tile);
    if (threadIdx.x == 0) *u.c.rank = r;
}

// DDC: W = alpha A B + beta Cu Cv sits in the tmp2 region (ld ws.ld); C <- [U = W | V = I].
__global__ void __launch_bounds__(256) ddc_finalize_kernel(const DevUpdate *ups, Workspace ws) {
    const int s = blockIdx.x;
    const DevUpdate u = ups[s];
    const int m = u.c.rows, nn = u.c.cols;
    const int r = m < nn ? m : nn;
    const double *W = ws.slot(s) + ws.off_tmp2;
    double *U = u.c.data;
    double *V = u.c.v;
    for (int j = 0; j < r; j++)
        for (int i = threadIdx.x; i < m; i += blockDim.x) U[i + (size_t) j * m] = W[i + (size_t) j * ws.ld];
    // V = I (r x n, ld r); a compressed_vt C stores W = V^T (n x r, ld n), the same identity pattern.
    const int vr = u.c.kind == HCGB_COMPRESSED_VT ? nn : r, vc = u.c.kind == HCGB_COMPRESSED_VT ? r : nn;
    for (int j = 0; j < vc; j++)
        for (int i = threadIdx.x; i < vr; i += blockDim.x) V[i + (size_t) j * vr] = (i == j) ? 1.0 : 0.0;
    if (threadIdx.x == 0) *u.c.rank = r;
}

__global__ void __launch_bounds__(1024) order_kernel(int n, Workspace ws) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int *mi = ws.meta + (size_t) i * META_INTS;
        const int ki = mi[META_CKIND] ? mi[META_K] : 0;
        int pos = 0;
        for (int j = 0; j < n; j++) {
            const int *mj = ws.meta + (size_t) j * META_INTS;
            const int kj = mj[META_CKIND] ? mj[META_K] : 0;
            pos += (kj > ki) || (kj == ki && j < i);
        }
        ws.order[pos] = i;
    }
}

__global__ void __launch_bounds__(256) transpose_kernel(const double *src, int lds, int rows, int cols, double *dst,
                                                      int ldd) {
    __shared__ double tile[32][33];
    transpose_scaled(src, lds, rows, cols, dst, ldd, 1.0, tile);
}

// One thread per update: the six jobs of the WY application of both Q factors (after the core).
//   0/1: G = V^T V of the U / V stack (unit lower Householder vectors), into off_m / off_mcopy
//   2/3: Y = V^T X, X = the new U (C's U buffer) / XV, into W (off_w); X is zero below row kk
//   4/5: X <- X - V W
__global__ void plan_wy_kernel(const DevUpdate *ups, int n, Workspace ws, Params p, GemmJob *jobs) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    GemmJob none;
    none.M = none.N = none.K = 0;
    none.oz = none.triA = none.triB = none.prec = 0;
    for (int q = 0; q < 6; q++) jobs[(size_t) q * n + s] = none;
    int *meta = ws.meta + (size_t) s * META_INTS;
    meta[META_WY] = 0;
    const int st = meta[META_STATUS];
    if ((st != HCGB_OK && st != HCGB_NOT_CONVERGED) || !meta[META_CKIND]) return;
    const int k = meta[META_K], m = meta[META_M], nn = meta[META_N], r = meta[META_NEWRANK];
    double *base = ws.slot(s);
    const int ld = ws.ld, lk = ws.kmax;
    for (int side = 0; side < 2; side++) {
        const int rows = side ? nn : m, kk = rows < k ? rows : k;
        const int lp = lowp_prec(p.mode);  // low-precision forms: every side in WY form
        if (!lp && (!p.oz || kk < p.wy_min)) continue;  // panel-wise apply_q_kernel
        if (kk < 1) continue;
        meta[META_WY] |= 1 << side;
        double *Vst = base + (side ? ws.off_vstack : ws.off_ustack);
        double *G = base + (side ? ws.off_mcopy : ws.off_m);
        double *W = base + ws.off_w + (size_t) side * lk * lk;
        double *X = side ? base + ws.off_xv : ups[s].c.data;
        const int ldx = side ? ld : ups[s].c.rows;
        GemmJob g = make_job(Vst, ld, 1, Vst, ld, 0, G, lk, kk, kk, rows, 1.0, 0.0);
        g.triA = g.triB = 1;
        GemmJob y = make_job(Vst, ld, 1, X, ldx, 0, W, lk, kk, r, kk, 1.0, 0.0);
        y.triA = 1;
        GemmJob u = make_job(Vst, ld, 0, W, lk, 0, X, ldx, rows, r, kk, -1.0, 1.0);
        u.triA = 1;
        // The Grams define the T factor of the QR and stay FP64-accurate; Y = V^T X and X - V W take
        // the form's product precision.
        y.prec = u.prec = lp;
        GemmJob *out[3] = {&g, &y, &u};
        for (int q = 0; q < 3; q++) {
            GemmJob &j = *out[q];
            j.oz = (!j.prec && p.oz && j.M > 0 && j.N > 0 && oz_shape(j.M, j.N, j.K, p.oz_min)) ? 1 : 0;
            jobs[(size_t) (2 * q + side) * n + s] = j;
        }
    }
}

// Two CTAs per update (U side, V side): solve T^-1 W = Y in place, T^-1 = striu(G) + diag(1/tau),
// by blocked back substitution over row blocks of 32 (bottom up): the block's rows first take the
// product of the already solved rows (every thread a few (row, column) dot products; G is
// symmetric, so row i of its upper part is read as column i, contiguous), then the 32 x 32
// triangle is solved with one thread per column from shared memory.  tau_i = 0 (an identity
// reflector) gives W_i = 0.
__global__ void __launch_bounds__(256) wy_solve_kernel(Workspace ws) {
    constexpr int BS = 32;
    __shared__ double Gb[BS][BS + 1];
    __shared__ double tb[BS];
    const int slot = ws.heavy(blockIdx.x >> 1), side = blockIdx.x & 1;
    const int *meta = ws.meta + (size_t) slot * META_INTS;
    const int st = meta[META_STATUS];
    if ((st != HCGB_OK && st != HCGB_NOT_CONVERGED) || !meta[META_CKIND] || !(meta[META_WY] & (1 << side))) return;
    const int k = meta[META_K], rows = side ? meta[META_N] : meta[META_M], r = meta[META_NEWRANK];
    const int kk = rows < k ? rows : k;
    double *base = ws.slot(slot);
    const double *G = base + (side ? ws.off_mcopy : ws.off_m);
    const double *tau = base + (side ? ws.off_tauv : ws.off_tauu);
    double *W = base + ws.off_w + (size_t) side * ws.kmax * ws.kmax;
    const int lk = ws.kmax;
    for (int bs = ((kk - 1) / BS) * BS; bs >= 0; bs -= BS) {
        const int be = bs + BS < kk ? bs + BS : kk, nbk = be - bs;
        // 1. rows bs..be-1 of W -= G[bs:be, be:kk] W[be:kk, :]
        if (be < kk) {
            for (int e = threadIdx.x; e < nbk * r; e += blockDim.x) {
                const int i = bs + e % nbk, c = e / nbk;
                const double *gi = G + (size_t) i * lk;
                const double *wc = W + (size_t) c * lk;
                double s0 = 0.0, s1 = 0.0;
                int j = be;
                for (; j + 1 < kk; j += 2) {
                    s0 = fma(gi[j], wc[j], s0);
                    s1 = fma(gi[j + 1], wc[j + 1], s1);
                }
                if (j < kk) s0 = fma(gi[j], wc[j], s0);
                W[i + (size_t) c * lk] -= s0 + s1;
            }
        }
        // 2. the diagonal block: G[bs:be, bs:be] (upper part) and tau into shared memory
        for (int e = threadIdx.x; e < nbk * nbk; e += blockDim.x) {
            const int a = e % nbk, b = e / nbk;
            Gb[a][b] = G[(size_t) (bs + b) * lk + bs + a];  // symmetric: G(a, b)
        }
        if (threadIdx.x < nbk) tb[threadIdx.x] = tau[bs + threadIdx.x];
        __syncthreads();
        for (int c = threadIdx.x; c < r; c += blockDim.x) {
            double *wc = W + (size_t) c * lk + bs;
            double x[BS];
#pragma unroll
            for (int a = 0; a < BS; a++) x[a] = a < nbk ? wc[a] : 0.0;
#pragma unroll
            for (int a = BS - 1; a >= 0; a--) {
                if (a < nbk) {
                    double sacc = x[a];
#pragma unroll
                    for (int b = a + 1; b < BS; b++)
                        if (b < nbk) sacc = fma(-Gb[a][b], x[b], sacc);
                    x[a] = tb[a] * sacc;
                }
            }
#pragma unroll
            for (int a = 0; a < BS; a++)
                if (a < nbk) wc[a] = x[a];
        }
        __syncthreads();
    }
}

}  // namespace

void launch_plan_wy(const DevUpdate *ups, int n, Workspace ws, Params p, GemmJob *jobs, cudaStream_t st) {
    { plan_wy_kernel<<<(n + 127) / 128, 128, 0, st>>>(ups, n, ws, p, jobs); note_launch(); }
}

void launch_wy_solve(int n, Workspace ws, cudaStream_t st) {
    { wy_solve_kernel<<<2 * n, 256, 0, st>>>(ws); note_launch(); }
}

void launch_transpose(const double *src, int lds, int rows, int cols, double *dst, int ldd, cudaStream_t st) {
    { transpose_kernel<<<1, 256, 0, st>>>(src, lds, rows, cols, dst, ldd); note_launch(); }
}

void launch_plan(const DevUpdate *ups, int n, double alpha, double beta, Workspace ws, Params p, GemmJob *jobs,
                 cudaStream_t st) {
    { plan_kernel<<<(n + 127) / 128, 128, 0, st>>>(ups, n, alpha, beta, ws, p, jobs); note_launch(); }
}

__global__ void __launch_bounds__(256) gather_ranks_kernel(const int *const *ptrs, int n, int *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = *ptrs[i];
}

void launch_gather_ranks(const int *const *ptrs, int n, int *out, cudaStream_t st) {
    if (n > 0) { gather_ranks_kernel<<<(n + 255) / 256, 256, 0, st>>>(ptrs, n, out); note_launch(); }
}

void launch_order(int n, Workspace ws, cudaStream_t st) {
    { order_kernel<<<1, 1024, 0, st>>>(n, ws); note_launch(); }
}

void launch_stack(const DevUpdate *ups, int n, double alpha, double beta, Workspace ws, cudaStream_t st) {
    { stack_kernel<<<n, 256, 0, st>>>(ups, alpha, beta, ws); note_launch(); }
}

static int device_sms() {
    static int sms[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152;
    if (!sms[dev]) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    return sms[dev] > 0 ? sms[dev] : 152;
}

void launch_gemm_jobs(const GemmJob *jobs, int njobs, int *sched, cudaStream_t st, bool has_lowp) {
    const int sms = device_sms();
    for (int off = 0; off < njobs; off += MAX_JOBS_PER_LAUNCH) {
        const int nj = njobs - off < MAX_JOBS_PER_LAUNCH ? njobs - off : MAX_JOBS_PER_LAUNCH;
        { schedule_kernel<<<1, 1024, 0, st>>>(jobs + off, nj, sched); note_launch(); }
        { gemm_jobs_kernel<<<4 * sms, 128, 0, st>>>(jobs + off, nj, sched); note_launch(); }
        launch_oz_gemm_jobs(jobs + off, nj, sched + nj + 1, sms, st);
        if (has_lowp) launch_tc_gemm_jobs(jobs + off, nj, sched + 2 * (nj + 1), sms, st);
    }
}

void launch_finalize(const DevUpdate *ups, int n, Workspace ws, hcgb_update_info *info, cudaStream_t st) {
    { finalize_kernel<<<n, 256, 0, st>>>(ups, ws, info); note_launch(); }
}

void launch_ddc_finalize(const DevUpdate *ups, int n, Workspace ws, cudaStream_t st) {
    { ddc_finalize_kernel<<<n, 256, 0, st>>>(ups, ws); note_launch(); }
}

Workspace make_workspace_layout(int ld, int kmax, int rmax, bool ddc_scratch, bool wy, bool learned) {
    Workspace w{};
    w.ld = ld;
    w.kmax = kmax;
    w.rmax = rmax;
    auto round = [](size_t x) { return (x + 31) & ~size_t(31); };  // 256-byte aligned sub-buffers
    size_t off = 0;
    const int npan = (kmax + QR_NB - 1) / QR_NB;
    w.off_ustack = off; off += round((size_t) ld * kmax);
    w.off_vstack = off; off += round((size_t) ld * kmax);
    w.off_tmp1 = off;   off += round((size_t) rmax * rmax);
    w.off_tmp2 = off;   off += round((size_t) ld * (size_t) (ddc_scratch ? (rmax > ld ? rmax : ld) : rmax));
    w.off_tauu = off;   off += round(kmax);
    w.off_tauv = off;   off += round(kmax);
    w.off_tu = off;     off += round((size_t) npan * QR_NB * QR_NB);
    w.off_tv = off;     off += round((size_t) npan * QR_NB * QR_NB);
    w.off_m = off;      off += round((size_t) kmax * kmax);
    w.off_mcopy = off;  off += round((size_t) kmax * kmax);
    w.off_xv = off;     off += round((size_t) ld * kmax);
    w.off_sigma = off;  off += round(kmax);
    w.off_mixed = off;  off += round(((size_t) kmax * (size_t) (kmax + ld) + 1) / 2);  // float X32 + J32
    w.off_w = wy ? off : 0;  // 0: absent (no region starts at 0 but the U stack)
    off += wy ? round(2 * (size_t) kmax * kmax) : 0;
    w.off_sk1 = learned ? off : 0;
    off += learned ? round((size_t) ld * kmax) : 0;
    w.off_sk2 = learned ? off : 0;
    off += learned ? round((size_t) ld * kmax) : 0;
    w.off_skaux = learned ? off : 0;
    off += learned ? round(8) : 0;
    w.feat = nullptr;
    w.pred = nullptr;
    w.slot_doubles = off;
    return w;
}

}  // namespace hcgb
