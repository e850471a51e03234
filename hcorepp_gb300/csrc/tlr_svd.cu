// Core of the recompression: M = R_U R_V^T, its SVD by one-sided Jacobi, the rank
// truncation, and the new left/right factors in the small basis.
//
// Replaces the R extraction + core GEMM + SVD + CalculateNewRank + CalculateVTnew of
// CompressedTile<T>::Gemm (src/operators/concrete/Compressed.cpp:441-527, :597-599) and the
// host-synchronising rank scan of the CUDA backend (src/kernels/cuda/CudaKernels.cu:656-697).
//
// One team per update (a whole 512-thread CTA for a core that does not fit half the shared
// memory, else half a CTA).  M = R_U R_V^T on DMMA; Householder QR with column pivoting of M,
// stopped once the remaining columns lie far below the truncation threshold; one-sided Jacobi on
// the rk columns of X = R^T (round-robin parallel ordering, 4-32 lanes per column pair, scaled
// rotations, tracked norms) until every pair is orthogonal to working precision: X J = W,
// sigma_j = ||w_j||.  The right factor is XV = P W_r (= V_r Sigma_r) and the left one
// U = M XV Sigma^-2 (= U_r), so the rotations never need accumulating.  The pivoted QR and the
// sweeps run in FP64 (plain form) or float-float (mixed form).  The rank rule is the reference's
// (omp/kernels.cpp:82-104) applied to the sorted sigma.
#include <cfloat>

#include "internal.cuh"
#include "df.cuh"

namespace hcgb {

namespace {

constexpr int SVD_THREADS = 512;
constexpr float PRECOND_TOL32 = 1e-6f;
constexpr int PRECOND_MAX_SWEEPS = 12;
constexpr int SVD_RED_DOUBLES = 64, SVD_REDI_INTS = 128;  // reduction area (up to 32 warps)
constexpr int SVD_AUX_FIXED = 1 + SVD_RED_DOUBLES + SVD_REDI_INTS / 2;  // aux = 6 kmax + this

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

template <typename T>
__device__ __forceinline__ T group_sum(T v, int G) {
    for (int o = G >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <>
__device__ __forceinline__ df group_sum<df>(df v, int G) {
    return df_group_sum(v, G);
}

// Tangent of the Jacobi angle that orthogonalises a pair with squared norms a, b and inner
// product c: zeta = (b - a) / (2 c), t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)) (Rutishauser).
// Evaluated in single precision after scaling both terms by the same power of two (read off the
// exponent of c with integer operations), so no double-precision divide or square root is spent
// on it; the rotation built from t is orthogonal to working precision whatever t's rounding.
__device__ __forceinline__ float jacobi_tangent(double a, double b, double c) {
    const int hi = __double2hiint(c);
    const int e = ((hi >> 20) & 0x7ff) - 1023;
    const int se = e < -1000 ? -1000 : (e > 1000 ? 1000 : e);
    const double scale = __hiloint2double((1023 - se) << 20, 0);  // 2^-se, exact
    const float num = (float) ((b - a) * scale);
    const float den = (float) (2.0 * c * scale);
    const float zf = num / den;
    if (fabsf(zf) > 1.0e18f) return 0.5f / zf;
    return copysignf(1.0f, zf) / (fabsf(zf) + sqrtf(fmaf(zf, zf, 1.0f)));
}

// A rotated pair's bookkeeping (tracked squared norms a - t cd, b + t cd; scales d cos; inverse scales
// (1/d) q cos) spread over the first four lanes of its group: every lane evaluates the same three FP64
// instructions on operands it selects, instead of one lane issuing six or seven (the FP64 pipe, one
// warp-wide instruction per ~19 cycles per SM on GB300, bounds the plain core).  Lanes 0 / 1 store
// column i's / j's norm and inverse scale, lanes 2 / 3 its scale.
__device__ __forceinline__ void pair_bookkeeping(int gl, int i, int j, double a, double b, double tt, double cd,
                                                 double cs, double q, double di, double dj, double dvi, double dvj,
                                                 double *nrm, double *dsc, int dstride) {
    const bool second = gl & 1, norm_lane = gl < 2;
    const int col = second ? j : i;
    const double m1 = norm_lane ? (second ? tt : -tt) : (second ? dj : di);
    const double v = fma(m1, norm_lane ? cd : cs, norm_lane ? (second ? b : a) : 0.0);
    const double w = (second ? dvj : dvi) * (q * cs);
    if (norm_lane) {
        nrm[col] = v;
        dsc[dstride + col] = w;
    } else if (gl < 4) {
        dsc[col] = v;
    }
}

// One sweep of one-sided Jacobi over the `ncols` columns (length `rows`) of X (ld ldx), with G
// lanes per column pair (32/G pairs per warp at a time) and up to RPL rows per lane in registers.
// Squared column norms are tracked in nrm[] (a' = a - t c, b' = b + t c), so each pair costs one
// inner product.  A pair is rotated when c^2 > tol2 a b and both columns are above the noise
// floor `tiny`; columns below it hold only rounding errors of the larger ones.
//
// The rotations are applied in scaled form (the idea of fast Givens rotations): column i is
// stored as x_i with the true column d_i x_i, so the rotation
//   X_i' = cos (X_i - t X_j),  X_j' = cos (X_j + t X_i)
// becomes x_i' = x_i - t (d_j / d_i) x_j, x_j' = x_j + t (d_i / d_j) x_i, d' = cos d: one FMA per
// element instead of a multiply and an FMA.  d and 1/d live in dsc[0..) and dsc[dstride..);
// the caller folds them back into the columns at the start of every sweep.
template <int G, int RPL, class TM>
__device__ int jacobi_sweep(const TM &tm, double *X, int ldx, int rows, int ncols, double *nrm, double tol2,
                            double tiny, int n2, double *dsc, int dstride) {
    static_assert(G >= 4, "pair_bookkeeping spreads a pair's bookkeeping over four lanes");
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    constexpr int PPW = 32 / G;
    const int gl = lane % G, grp = lane / G;
    const int npairs = n2 / 2;
    const int nchunks = (npairs + PPW - 1) / PPW;
    int rotations = 0;
    for (int t = 0; t < n2 - 1; t++) {
        for (int ch = warp; ch < nchunks; ch += nw) {
            const int pp = ch * PPW + grp;
            int i = 0, j = 0;
            bool act = pp < npairs;
            if (act) {
                jacobi_pair(t, pp, n2, i, j);
                act = i < ncols && j < ncols;
            }
            double *x = X + (size_t) (act ? i : 0) * ldx;
            double *y = X + (size_t) (act ? j : 0) * ldx;
            double xr[RPL], yr[RPL];
            double c = 0.0;
#pragma unroll
            for (int q = 0; q < RPL; q++) {
                xr[q] = yr[q] = 0.0;
                if (G * q < rows) {  // uniform across the warp: whole row slots beyond `rows` are skipped
                    const int r = gl + G * q;
                    if (act && r < rows) {
                        xr[q] = x[r];
                        yr[q] = y[r];
                    }
                    c = fma(xr[q], yr[q], c);
                }
            }
            c = group_sum(c, G);
            const double a = act ? nrm[i] : 0.0, b = act ? nrm[j] : 0.0;
            double di = 1.0, dj = 1.0;
            if (act) {
                di = dsc[i];
                dj = dsc[j];
            }
            const double cd = c * di * dj;  // true inner product
            const bool rot = act && a > tiny && b > tiny && cd * cd > tol2 * a * b;
            if (rot) {
                const double tt = (double) jacobi_tangent(a, b, cd);
                const double q = fma(tt, tt, 1.0);
                const double cs = rsqrt(q);
                const double dvi = dsc[dstride + i], dvj = dsc[dstride + j];
                const double t1 = tt * dj * dvi, t2 = tt * di * dvj;
#pragma unroll
                for (int q2 = 0; q2 < RPL; q2++) {
                    if (G * q2 < rows) {
                        const int r = gl + G * q2;
                        if (r < rows) {
                            x[r] = fma(-t1, yr[q2], xr[q2]);
                            y[r] = fma(t2, xr[q2], yr[q2]);
                        }
                    }
                }
                pair_bookkeeping(gl, i, j, a, b, tt, cd, cs, q, di, dj, dvi, dvj, nrm, dsc, dstride);
                if (gl == 0) rotations++;
            }
        }
        tm.sync();
    }
    return rotations;
}

// The same sweep with the column pairs read from memory by G-lane groups in a loop over the rows
// instead of register tiles (rows of any length, 32 / G pairs per warp): for long columns it packs
// more pairs into each warp instruction than the register tiles can, which shares the per-pair
// scalar FP64 work among more pairs at the price of reading the columns twice.
template <int G, class TM>
__device__ int jacobi_sweep_loop(const TM &tm, double *X, int ldx, int rows, int ncols, double *nrm, double tol2,
                                 double tiny, int n2, double *dsc, int dstride) {
    static_assert(G >= 4, "pair_bookkeeping spreads a pair's bookkeeping over four lanes");
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    constexpr int PPW = 32 / G;
    const int gl = lane % G, grp = lane / G;
    const int npairs = n2 / 2;
    const int nchunks = (npairs + PPW - 1) / PPW;
    int rotations = 0;
    for (int t = 0; t < n2 - 1; t++) {
        for (int ch = warp; ch < nchunks; ch += nw) {
            const int pp = ch * PPW + grp;
            int i = 0, j = 0;
            bool act = pp < npairs;
            if (act) {
                jacobi_pair(t, pp, n2, i, j);
                act = i < ncols && j < ncols;
            }
            double *x = X + (size_t) (act ? i : 0) * ldx;
            double *y = X + (size_t) (act ? j : 0) * ldx;
            double c0 = 0.0, c1 = 0.0;
            if (act) {
                int r = gl;
                for (; r + G < rows; r += 2 * G) {
                    c0 = fma(x[r], y[r], c0);
                    c1 = fma(x[r + G], y[r + G], c1);
                }
                if (r < rows) c0 = fma(x[r], y[r], c0);
            }
            const double c = group_sum(c0 + c1, G);
            const double a = act ? nrm[i] : 0.0, b = act ? nrm[j] : 0.0;
            double di = 1.0, dj = 1.0;
            if (act) {
                di = dsc[i];
                dj = dsc[j];
            }
            const double cd = c * di * dj;  // true inner product
            const bool rot = act && a > tiny && b > tiny && cd * cd > tol2 * a * b;
            if (rot) {
                const double tt = (double) jacobi_tangent(a, b, cd);
                const double q = fma(tt, tt, 1.0);
                const double cs = rsqrt(q);
                const double dvi = dsc[dstride + i], dvj = dsc[dstride + j];
                const double t1 = tt * dj * dvi, t2 = tt * di * dvj;
#pragma unroll 4
                for (int r = gl; r < rows; r += G) {
                    const double xv = x[r], yv = y[r];
                    x[r] = fma(-t1, yv, xv);
                    y[r] = fma(t2, xv, yv);
                }
                pair_bookkeeping(gl, i, j, a, b, tt, cd, cs, q, di, dj, dvi, dvj, nrm, dsc, dstride);
                if (gl == 0) rotations++;
            }
        }
        tm.sync();
    }
    return rotations;
}

// Jacobi iteration on X: exact squared column norms at the start of every sweep (the scales of
// the previous sweep folded into the columns), then sweeps until no pair rotates (or max_sweeps).
// RPL = 0 selects the looped sweep.
template <int G, int RPL, class TM>
__device__ void jacobi(const TM &tm, double *X, int ldx, int rows, int ncols, double *nrm, int *s_rot,
                       double *s_amax, int *sweeps_out, bool *converged_out, double tol, int max_sweeps, double *dsc,
                       int dstride) {
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    const double tol2 = tol * tol;
    const double noise = DBL_EPSILON * (double) (rows > 1 ? rows : 1);
    const int n2 = ncols + (ncols & 1);
    int sweeps = 0;
    bool converged = ncols < 2;
    for (int j = tm.tid; j < ncols; j += tm.nth) dsc[j] = dsc[dstride + j] = 1.0;
    tm.sync();
    auto fold_and_norms = [&](double &amax) {
        for (int j = warp; j < ncols; j += nw) {
            double *col = X + (size_t) j * ldx;
            const double dj = dsc[j];
            double sq = 0.0;
            for (int r = lane; r < rows; r += 32) {
                double v = col[r];
                if (dj != 1.0) {
                    v *= dj;
                    col[r] = v;
                }
                sq = fma(v, v, sq);
            }
            sq = warp_sum(sq);
            if (lane == 0) {
                nrm[j] = sq;
                dsc[j] = dsc[dstride + j] = 1.0;
            }
            amax = fmax(amax, sq);
        }
    };
    while (!converged && sweeps < max_sweeps) {
        if (tm.tid == 0) {
            *s_rot = 0;
            *s_amax = 0.0;
        }
        tm.sync();
        double amax = 0.0;
        fold_and_norms(amax);
        if (lane == 0) atomicMax(reinterpret_cast<unsigned long long *>(s_amax), __double_as_longlong(amax));
        tm.sync();
        const double tiny = *s_amax * noise * noise;
        int rot;
        if constexpr (RPL == 0)
            rot = jacobi_sweep_loop<G>(tm, X, ldx, rows, ncols, nrm, tol2, tiny, n2, dsc, dstride);
        else
            rot = jacobi_sweep<G, RPL>(tm, X, ldx, rows, ncols, nrm, tol2, tiny, n2, dsc, dstride);
        if (rot) atomicAdd(s_rot, rot);
        tm.sync();
        sweeps++;
        converged = (*s_rot == 0);
        tm.sync();
    }
    double amax = 0.0;
    fold_and_norms(amax);  // a sweep limit can leave scales unfolded
    tm.sync();
    *sweeps_out = sweeps;
    *converged_out = converged;
}

// Lane-group / register-tile choice for a column length: G lanes per pair, RPL rows per lane.
// ---------------------------------------------------------------------------------------------
// Float-float Jacobi (mixed form): the columns, the tracked squared norms and the scales d, 1/d are
// all float-float values, so neither the rows nor the per-pair bookkeeping touch the FP64 pipe.
// Same method as jacobi_sweep (round-robin ordering, scaled rotations, tracked norms); the rotation
// tangent is a float (any tangent gives an exact rotation once cos = 1/sqrt(1 + t^2) is formed to
// float-float accuracy, which one Newton step on the float reciprocal square root does).
// ---------------------------------------------------------------------------------------------
template <int G, int RPL, class TM>
__device__ int jacobi_sweep_df(const TM &tm, df *X, int ldx, int rows, int ncols, df *nrm, df *ds, df *dv, float tol, float tiny,
                               int n2) {
    static_assert(G >= 4, "a pair's bookkeeping is spread over four lanes of its group");
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    constexpr int PPW = 32 / G;
    const int gl = lane % G, grp = lane / G;
    const int npairs = n2 / 2;
    const int nchunks = (npairs + PPW - 1) / PPW;
    int rotations = 0;
    for (int t = 0; t < n2 - 1; t++) {
        for (int ch = warp; ch < nchunks; ch += nw) {
            const int pp = ch * PPW + grp;
            int i = 0, j = 0;
            bool act = pp < npairs;
            if (act) {
                jacobi_pair(t, pp, n2, i, j);
                act = i < ncols && j < ncols;
            }
            df *x = X + (size_t) (act ? i : 0) * ldx;
            df *y = X + (size_t) (act ? j : 0) * ldx;
            df xr[RPL], yr[RPL];
            df_acc ca{0.f, 0.f};
#pragma unroll
            for (int q = 0; q < RPL; q++) {
                xr[q] = yr[q] = df_f(0.f);
                if (G * q < rows) {
                    const int r = gl + G * q;
                    if (act && r < rows) {
                        xr[q] = x[r];
                        yr[q] = y[r];
                    }
                    df_acc_fma(ca, xr[q], yr[q]);
                }
            }
            const df c = group_sum(df_acc_value(ca), G);
            df a = df_f(0.f), b = df_f(0.f), di = df_f(1.f), dj = df_f(1.f);
            if (act) {
                a = nrm[i];
                b = nrm[j];
                di = ds[i];
                dj = ds[j];
            }
            const df cd = df_mul(df_mul(c, di), dj);  // true inner product
            // |c| / sqrt(a b) > tol, in float (all quantities well inside the float range)
            const bool rot = act && a.h > tiny && b.h > tiny && fabsf(cd.h) * rsqrtf(a.h) * rsqrtf(b.h) > tol;
            if (rot) {
                const float num = df_add(b, -a).h, den = 2.f * cd.h;
                const float zf = num / den;
                const float tt = fabsf(zf) > 1.0e18f ? 0.5f / zf
                                                     : copysignf(1.0f, zf) / (fabsf(zf) + sqrtf(fmaf(zf, zf, 1.0f)));
                const df q = df_add(df_f(1.f), df_mul(df_f(tt), df_f(tt)));
                const df cs = df_rsqrt(q);
                const df dvi = dv[i], dvj = dv[j];
                const df t1 = df_mul(df_mul(df_f(tt), dj), dvi), t2 = df_mul(df_mul(df_f(tt), di), dvj);
                const df mt1 = -t1;
#pragma unroll
                for (int q2 = 0; q2 < RPL; q2++) {
                    if (G * q2 < rows) {
                        const int r = gl + G * q2;
                        if (r < rows) {
                            x[r] = df_fma(mt1, yr[q2], xr[q2]);
                            y[r] = df_fma(t2, xr[q2], yr[q2]);
                        }
                    }
                }
                // the pair's bookkeeping spread over the first four lanes of its group (as the FP64
                // sweep's pair_bookkeeping): each evaluates the same float-float operations on
                // operands it selects, which shortens the dependent chain one lane would otherwise run
                {
                    const bool second = gl & 1, norm_lane = gl < 2;
                    const int col = second ? j : i;
                    // lanes 0 / 1: norm a - t cd, b + t cd; lanes 2 / 3: scale d cs
                    const df m1 = norm_lane ? (second ? df_f(tt) : df_f(-tt)) : (second ? dj : di);
                    const df prod = df_mul(m1, norm_lane ? cd : cs);
                    const df v = norm_lane ? df_add(second ? b : a, prod) : prod;
                    const df w = df_mul(second ? dvj : dvi, df_mul(q, cs));  // inverse scale, lanes 0 / 1
                    if (norm_lane) {
                        nrm[col] = v;
                        dv[col] = w;
                    } else if (gl < 4) {
                        ds[col] = v;
                    }
                }
                if (gl == 0) rotations++;
            }
        }
        tm.sync();
    }
    return rotations;
}

template <int G, int RPL, class TM>
__device__ void jacobi_df(const TM &tm, df *X, int ldx, int rows, int ncols, df *nrm, df *ds, df *dv, int *s_rot, float *s_amax,
                          int *sweeps_out, bool *converged_out, float tol, int max_sweeps) {
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    const float noise = 3.5527137e-15f * (float) (rows > 1 ? rows : 1);  // 2^-48 rows
    const int n2 = ncols + (ncols & 1);
    int sweeps = 0;
    bool converged = ncols < 2;
    for (int jj = tm.tid; jj < ncols; jj += tm.nth) ds[jj] = dv[jj] = df_f(1.f);
    tm.sync();
    // Exact squared norms; the scales of the previous sweep are folded into the columns.
    auto fold_and_norms = [&](float &amax) {
        for (int jj = warp; jj < ncols; jj += nw) {
            df *col = X + (size_t) jj * ldx;
            const df d = ds[jj];
            const bool scale = d.h != 1.f || d.l != 0.f;
            df sq = df_f(0.f);
            for (int r = lane; r < rows; r += 32) {
                df v = col[r];
                if (scale) {
                    v = df_mul(v, d);
                    col[r] = v;
                }
                sq = df_fma(v, v, sq);
            }
            sq = group_sum(sq, 32);
            __syncwarp();
            if (lane == 0) {
                nrm[jj] = sq;
                ds[jj] = dv[jj] = df_f(1.f);
            }
            amax = fmaxf(amax, sq.h);
        }
    };
    while (!converged && sweeps < max_sweeps) {
        if (tm.tid == 0) {
            *s_rot = 0;
            *s_amax = 0.f;
        }
        tm.sync();
        float amax = 0.f;
        fold_and_norms(amax);
        if (lane == 0) atomicMax(reinterpret_cast<int *>(s_amax), __float_as_int(amax));  // amax >= 0
        tm.sync();
        const float tiny = *s_amax * noise * noise;
        const int rot = jacobi_sweep_df<G, RPL>(tm, X, ldx, rows, ncols, nrm, ds, dv, tol, tiny, n2);
        if (rot) atomicAdd(s_rot, rot);
        tm.sync();
        sweeps++;
        converged = (*s_rot == 0);
        tm.sync();
    }
    float amax = 0.f;
    fold_and_norms(amax);  // a sweep limit can leave scales unfolded
    tm.sync();
    *sweeps_out = sweeps;
    *converged_out = converged;
}

template <int MAXRPL, class TM>
__device__ void jacobi_df_dispatch(const TM &tm, df *X, int ldx, int rows, int ncols, df *nrm, df *ds, df *dv, int *s_rot,
                                   float *s_amax, int *sweeps, bool *conv, float tol, int max_sweeps) {
    // (A looped sweep like the FP64 form's measured slower here, 296 vs 192 ms of core per multiply:
    // the float-float form is not bound by per-pair instructions on a scarce pipe, and reading each
    // pair twice costs more than it saves.)
    if (rows <= 32) jacobi_df<4, 8>(tm, X, ldx, rows, ncols, nrm, ds, dv, s_rot, s_amax, sweeps, conv, tol, max_sweeps);
    else if (rows <= 64) jacobi_df<8, 8>(tm, X, ldx, rows, ncols, nrm, ds, dv, s_rot, s_amax, sweeps, conv, tol, max_sweeps);
    else if (rows <= 128 && MAXRPL >= 16) jacobi_df<8, 16>(tm, X, ldx, rows, ncols, nrm, ds, dv, s_rot, s_amax, sweeps, conv, tol, max_sweeps);
    else if (rows <= 128) jacobi_df<16, 8>(tm, X, ldx, rows, ncols, nrm, ds, dv, s_rot, s_amax, sweeps, conv, tol, max_sweeps);
    else if (rows <= 256 && MAXRPL >= 16) jacobi_df<16, 16>(tm, X, ldx, rows, ncols, nrm, ds, dv, s_rot, s_amax, sweeps, conv, tol, max_sweeps);
    else if (rows <= 256 || MAXRPL <= 8) jacobi_df<32, 8>(tm, X, ldx, rows, ncols, nrm, ds, dv, s_rot, s_amax, sweeps, conv, tol, max_sweeps);
    else jacobi_df<32, MAXRPL>(tm, X, ldx, rows, ncols, nrm, ds, dv, s_rot, s_amax, sweeps, conv, tol, max_sweeps);
}

template <int MAXRPL, class TM>
__device__ void jacobi_dispatch(const TM &tm, double *X, int ldx, int rows, int ncols, double *nrm, int *s_rot,
                                double *s_amax, int *sweeps, bool *conv, double tol, int max_sweeps, double *dsc,
                                int dstride, bool x_in_smem) {
    // Fewer lanes per pair put more pairs in one warp instruction, so the per-pair scalar work
    // (tangent, tests, norm updates), which runs as full-width FP64 warp instructions on a pipe that
    // issues one of them per ~19 cycles per SM, is shared by 4-8 pairs; RPL rows per lane stay in
    // registers.  (Two lanes per pair for columns of up to 32 rows, one warp taking every pair of a
    // step, measured slower: 760 vs 673 kcycles per 17-32-column core.)
    // Longer columns held in shared memory: 4- or 8-lane groups in a loop over the rows (8 or 4 pairs
    // per warp instruction; each pair is read twice).  Columns in the workspace (cores too wide for
    // the team's shared memory) keep register tiles, which read them once: the loop measured 15-35 %
    // slower there (long-scoreboard stalls on the second read).
    if (rows <= 32) jacobi<4, 8>(tm, X, ldx, rows, ncols, nrm, s_rot, s_amax, sweeps, conv, tol, max_sweeps, dsc, dstride);
    else if (rows <= 64 && MAXRPL >= 16) jacobi<4, 16>(tm, X, ldx, rows, ncols, nrm, s_rot, s_amax, sweeps, conv, tol, max_sweeps, dsc, dstride);
    else if (rows <= 64) jacobi<8, 8>(tm, X, ldx, rows, ncols, nrm, s_rot, s_amax, sweeps, conv, tol, max_sweeps, dsc, dstride);
    else if (x_in_smem && rows <= 128) jacobi<4, 0>(tm, X, ldx, rows, ncols, nrm, s_rot, s_amax, sweeps, conv, tol, max_sweeps, dsc, dstride);
    else if (x_in_smem) jacobi<8, 0>(tm, X, ldx, rows, ncols, nrm, s_rot, s_amax, sweeps, conv, tol, max_sweeps, dsc, dstride);
    else if (rows <= 128 && MAXRPL >= 16) jacobi<8, 16>(tm, X, ldx, rows, ncols, nrm, s_rot, s_amax, sweeps, conv, tol, max_sweeps, dsc, dstride);
    else if (rows <= 128) jacobi<16, 8>(tm, X, ldx, rows, ncols, nrm, s_rot, s_amax, sweeps, conv, tol, max_sweeps, dsc, dstride);
    else if (rows <= 256 && MAXRPL >= 16) jacobi<16, 16>(tm, X, ldx, rows, ncols, nrm, s_rot, s_amax, sweeps, conv, tol, max_sweeps, dsc, dstride);
    else if (rows <= 256) jacobi<32, 8>(tm, X, ldx, rows, ncols, nrm, s_rot, s_amax, sweeps, conv, tol, max_sweeps, dsc, dstride);
    // Longer columns (nb = 1024 stacks): the register tile that would cover them spills, so the loop.
    else jacobi<8, 0>(tm, X, ldx, rows, ncols, nrm, s_rot, s_amax, sweeps, conv, tol, max_sweeps, dsc, dstride);
}

// ---------------------------------------------------------------------------------------------
// FP32 preconditioning of the plain form's Jacobi (the FP64 pipe is the plain core's bound): one-
// sided Jacobi in single precision on X32 = X * 2^-e (rows x ncols, ld rows) with the rotations
// accumulated in J (ncols x ncols, ld ncols, float-float), one warp per column pair, until every
// pair is orthogonal to tol32 or max_sweeps.  The caller then forms X J in FP64 and finishes with
// FP64 sweeps.  Each rotation is the rotation of a float tangent normalised to float-float accuracy,
// and J accumulates them in float-float, so J is orthogonal to ~1e-13: X -> X J moves singular values
// and subspaces only at that level (a truncation at a fixed rank inside a slowly decaying spectrum
// included), and the FP64 sweeps make the final columns orthogonal to working precision.
// ---------------------------------------------------------------------------------------------
template <class TM>
__device__ int jacobi_precond32(const TM &tm, float *X, int rows, int ncols, df *J, float tol32, int max_sweeps,
                                int *s_rot) {
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    for (int e = tm.tid; e < ncols * ncols; e += tm.nth) J[e] = df_f((e % ncols) == (e / ncols) ? 1.f : 0.f);
    const int n2 = ncols + (ncols & 1);
    const float tol2 = tol32 * tol32;
    int sweeps = 0;
    for (; sweeps < max_sweeps; sweeps++) {
        if (tm.tid == 0) *s_rot = 0;
        tm.sync();
        int rot = 0;
        for (int t = 0; t < n2 - 1; t++) {
            for (int pp = warp; pp < n2 / 2; pp += nw) {
                int i, j;
                jacobi_pair(t, pp, n2, i, j);
                if (i >= ncols || j >= ncols) continue;
                float *xi = X + (size_t) i * rows, *xj = X + (size_t) j * rows;
                float a = 0.f, b = 0.f, c = 0.f;
                for (int r = lane; r < rows; r += 32) {
                    const float u = xi[r], w = xj[r];
                    a = fmaf(u, u, a);
                    b = fmaf(w, w, b);
                    c = fmaf(u, w, c);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    a += __shfl_xor_sync(0xffffffffu, a, o);
                    b += __shfl_xor_sync(0xffffffffu, b, o);
                    c += __shfl_xor_sync(0xffffffffu, c, o);
                }
                if (c == 0.f || c * c <= tol2 * a * b) continue;
                const float zeta = (b - a) / (2.f * c);
                const float tt = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(fmaf(zeta, zeta, 1.f)));
                // The rotation of the float tangent, normalised to float-float accuracy
                // (cs = 1 / sqrt(1 + t^2), sn = cs t): orthogonal to ~2^-46, so the accumulated J is
                // orthogonal to working precision of the FP64 phase's purposes.
                const df tdf = df_f(tt);
                const df cs = df_rsqrt(df_fma(tdf, tdf, df_f(1.f))), sn = df_mul(cs, tdf);
                const float cs32 = cs.h, sn32 = sn.h;
                for (int r = lane; r < rows; r += 32) {
                    const float u = xi[r], w = xj[r];
                    xi[r] = cs32 * u - sn32 * w;
                    xj[r] = fmaf(sn32, u, cs32 * w);
                }
                df *ji = J + (size_t) i * ncols, *jj = J + (size_t) j * ncols;
                for (int r = lane; r < ncols; r += 32) {
                    const df u = ji[r], w = jj[r];
                    ji[r] = df_fma(-sn, w, df_mul(cs, u));
                    jj[r] = df_fma(sn, u, df_mul(cs, w));
                }
                rot++;
            }
            tm.sync();
        }
        if (lane == 0 && rot) atomicAdd(s_rot, rot);
        tm.sync();
        const bool done = *s_rot == 0;
        tm.sync();
        if (done) break;
    }
    return sweeps;
}

// One step of qrcp_truncated after the reflector of column s is formed (x = column s, v = [1; x[s+1:]],
// tau): H = I - tau v v^T applied to columns s+1 .. ncols-1 by groups of G lanes (32 / G columns per
// warp at a time), the squared norms below row s downdated and recomputed exactly when the downdate
// loses four or more digits (LAPACK dlaqp2's guard).
template <int G, class TM>
__device__ __forceinline__ void qrcp_apply(const TM &tm, double *A, int lda, int mrows, int ncols, int s,
                                           const double *x, double tau, double *nrm, double *nref) {
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    constexpr int CPW = 32 / G;
    const int gl = lane % G, grp = lane / G;
    for (int j0 = s + 1 + warp * CPW; j0 < ncols; j0 += nw * CPW) {
        const int j = j0 + grp;
        const bool act = j < ncols;
        double *y = A + (size_t) (act ? j : s) * lda;  // idle groups read column s and write nothing
        double w = 0.0;
        if (tau != 0.0) {
            w = gl == 0 ? y[s] : 0.0;
            for (int i = s + 1 + gl; i < mrows; i += G) w = fma(x[i], y[i], w);
            w = group_sum(w, G) * tau;
            if (act)
                for (int i = s + 1 + gl; i < mrows; i += G) y[i] = fma(-w, x[i], y[i]);
        }
        const double ys = y[s] - w;  // every lane of the group reads the old y[s] before lane 0 writes it
        __syncwarp();
        if (act && gl == 0) y[s] = ys;
        double nn = act ? nrm[j] - ys * ys : 0.0;
        const bool exact = act && !(nn > 1e-8 * nref[j]);
        if (__any_sync(0xffffffffu, exact)) {
            double e = 0.0;
            if (exact)
                for (int i = s + 1 + gl; i < mrows; i += G) e = fma(y[i], y[i], e);
            e = group_sum(e, G);
            if (exact) nn = e;
        }
        __syncwarp();
        if (act && gl == 0) {
            nrm[j] = nn;
            if (exact) nref[j] = nn;
        }
    }
}

// Householder QR with column pivoting of A (mrows x ncols, ld lda) in place, stopped early once
// every remaining column is below sqrt(stop2) in norm (LAPACK dgeqp3 semantics for the part that
// is computed: A P = Q R with R in the upper triangle, pvt[s] = original index of column s).
// stop2 < 0 disables the early stop; stop2 == 0 with rel > 0 sets stop2 = (rel * |r_00|)^2 after
// the first pivot.  Column norms are recomputed exactly while each column is updated, so no
// norm downdating is needed.  Returns the number of rows of R that were computed.
template <class TM>
__device__ int qrcp_truncated(const TM &tm, double *A, int lda, int mrows, int ncols, double stop2, double rel, double *nrm,
                              double *nref, int *pvt, double *red, int *redi) {
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    for (int j = warp; j < ncols; j += nw) {
        const double *col = A + (size_t) j * lda;
        double t = 0.0;
        for (int i = lane; i < mrows; i += 32) t = fma(col[i], col[i], t);
        t = warp_sum(t);
        if (lane == 0) nrm[j] = nref[j] = t;
    }
    for (int j = tm.tid; j < ncols; j += tm.nth) pvt[j] = j;
    tm.sync();
    const int kk = mrows < ncols ? mrows : ncols;
    int rkeep = kk;
    for (int s = 0; s < kk; s++) {
        // pivot = argmax of the remaining squared norms (ties to the lower index), by the first warp
        // alone: the scan is short, and one warp's reduction costs an eighth of the FP64 instructions
        // of a team-wide one, whose barrier it also saves
        double bv = -1.0;
        int bi = s;
        if (warp == 0) {
            for (int j = s + lane; j < ncols; j += 32)
                if (nrm[j] > bv) {
                    bv = nrm[j];
                    bi = j;
                }
            for (int o = 16; o > 0; o >>= 1) {
                const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov > bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (lane == 0) {
                red[32] = bv;
                redi[32] = bi;
                if (s == 0 && stop2 == 0.0 && rel > 0.0) red[33] = rel * rel * bv;
                else if (s == 0) red[33] = stop2;
            }
        }
        tm.sync();
        bv = red[32];
        bi = redi[32];
        const double lim = red[33];
        if (bv <= lim || bv <= 0.0) {
            rkeep = s;
            break;
        }
        if (bi != s) {
            double *cs = A + (size_t) s * lda, *cb = A + (size_t) bi * lda;
            for (int i = tm.tid; i < mrows; i += tm.nth) {
                const double t = cs[i];
                cs[i] = cb[i];
                cb[i] = t;
            }
            if (tm.tid == 0) {
                const double t = nrm[s];
                nrm[s] = nrm[bi];
                nrm[bi] = t;
                const double tr = nref[s];
                nref[s] = nref[bi];
                nref[bi] = tr;
                const int ti = pvt[s];
                pvt[s] = pvt[bi];
                pvt[bi] = ti;
            }
        }
        tm.sync();
        // Householder vector of column s (rows s..mrows-1), dlarfg convention, by the first warp.
        double *x = A + (size_t) s * lda;
        double t = 0.0;
        if (warp == 0) {
            for (int i = s + 1 + lane; i < mrows; i += 32) t = fma(x[i], x[i], t);
            t = warp_sum(t);
        }
        if (tm.tid == 0) {
            const double alpha = x[s];
            double tau = 0.0, scale = 0.0, beta = alpha;
            if (t != 0.0) {
                beta = -copysign(sqrt(fma(alpha, alpha, t)), alpha);
                tau = (beta - alpha) / beta;
                scale = 1.0 / (alpha - beta);
            }
            x[s] = beta;
            red[40] = tau;
            red[41] = scale;
        }
        tm.sync();
        const double tau = red[40], scale = red[41];
        for (int i = s + 1 + tm.tid; i < mrows; i += tm.nth) x[i] *= scale;
        tm.sync();
        // Apply H to the remaining columns; downdate their squared norms below row s
        // (nrm -= y_s^2) and recompute exactly when the downdate cancels (LAPACK dlaqp2's guard).
        // Columns of up to 64, 256 or more rows are handled by groups of 4, 8 or 16 lanes, several
        // columns per warp instruction, so the reductions and the per-column scalar work are shared.
        if (mrows <= 64) qrcp_apply<4>(tm, A, lda, mrows, ncols, s, x, tau, nrm, nref);
        else if (mrows <= 256) qrcp_apply<8>(tm, A, lda, mrows, ncols, s, x, tau, nrm, nref);
        else qrcp_apply<16>(tm, A, lda, mrows, ncols, s, x, tau, nrm, nref);
        tm.sync();
    }
    return rkeep;
}

// qrcp_apply in float-float arithmetic (mixed form): H applied to columns s+1 .. ncols-1 by groups of
// G lanes with Dot2 accumulation, squared norms downdated and recomputed when the downdate cancels.
template <int G, class TM>
__device__ __forceinline__ void qrcp_apply_df(const TM &tm, df *A, int lda, int mrows, int ncols, int s, const df *x,
                                              df tau, df *nrm, df *nref) {
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    constexpr int CPW = 32 / G;
    const int gl = lane % G, grp = lane / G;
    const bool has_tau = tau.h != 0.f;
    for (int j0 = s + 1 + warp * CPW; j0 < ncols; j0 += nw * CPW) {
        const int j = j0 + grp;
        const bool act = j < ncols;
        df *y = A + (size_t) (act ? j : s) * lda;  // idle groups read column s and write nothing
        df w = df_f(0.f);
        if (has_tau) {
            df_acc wa = df_acc_init(gl == 0 ? y[s] : df_f(0.f));
            for (int i = s + 1 + gl; i < mrows; i += G) df_acc_fma(wa, x[i], y[i]);
            w = df_mul(group_sum(df_acc_value(wa), G), tau);
            const df mw = -w;
            if (act)
                for (int i = s + 1 + gl; i < mrows; i += G) y[i] = df_fma(mw, x[i], y[i]);
        }
        const df ys = df_add(y[s], -w);  // every lane of the group reads the old y[s] before lane 0 writes it
        __syncwarp();
        if (act && gl == 0) y[s] = ys;
        df nn = act ? df_add(nrm[j], -df_mul(ys, ys)) : df_f(0.f);
        const bool exact = act && !(nn.h > 1e-8f * nref[j].h);  // lost 4+ digits since the last exact value
        if (__any_sync(0xffffffffu, exact)) {
            df e = df_f(0.f);
            if (exact)
                for (int i = s + 1 + gl; i < mrows; i += G) e = df_fma(y[i], y[i], e);
            e = group_sum(e, G);
            if (exact) nn = e;
        }
        __syncwarp();
        if (act && gl == 0) {
            nrm[j] = nn;
            if (exact) nref[j] = nn;
        }
    }
}

// Float-float version of qrcp_truncated (mixed form), on a matrix scaled so that its entries are
// near 1: same pivoting, early stop (stop2 on squared norms; stop2 == 0 with rel2 > 0 sets
// stop2 = rel2 * |r_00|^2 after the first pivot; stop2 < 0 disables it) and norm downdating with
// exact recomputation when a downdate cancels.  Pivot keys are the float norms' bit patterns
// (non-negative floats order like their bits).
template <class TM>
__device__ int qrcp_truncated_df(const TM &tm, df *A, int lda, int mrows, int ncols, float stop2, float rel2, df *nrm, df *nref,
                                 int *pvt, float *red, int *redi) {
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    for (int j = warp; j < ncols; j += nw) {
        const df *col = A + (size_t) j * lda;
        df t = df_f(0.f);
        for (int i = lane; i < mrows; i += 32) t = df_fma(col[i], col[i], t);
        t = group_sum(t, 32);
        if (lane == 0) nrm[j] = nref[j] = t;
    }
    for (int j = tm.tid; j < ncols; j += tm.nth) pvt[j] = j;
    tm.sync();
    const int kk = mrows < ncols ? mrows : ncols;
    int rkeep = kk;
    for (int s = 0; s < kk; s++) {
        int bv = -1, bi = s;  // float bits of the largest remaining squared norm (first warp only)
        if (warp == 0) {
            for (int j = s + lane; j < ncols; j += 32) {
                const int v = __float_as_int(nrm[j].h);
                if (v > bv) {
                    bv = v;
                    bi = j;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const int ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov > bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (lane == 0) {
                redi[64] = bv;
                redi[65] = bi;
                if (s == 0) red[33] = (stop2 == 0.f && rel2 > 0.f) ? rel2 * __int_as_float(bv) : stop2;
            }
        }
        tm.sync();
        const float bvf = __int_as_float(redi[64]);
        bi = redi[65];
        const float lim = red[33];
        if (bvf <= lim || bvf <= 0.f) {
            rkeep = s;
            break;
        }
        if (bi != s) {
            df *cs = A + (size_t) s * lda, *cb = A + (size_t) bi * lda;
            for (int i = tm.tid; i < mrows; i += tm.nth) {
                const df t = cs[i];
                cs[i] = cb[i];
                cb[i] = t;
            }
            if (tm.tid == 0) {
                const df t = nrm[s];
                nrm[s] = nrm[bi];
                nrm[bi] = t;
                const df tr = nref[s];
                nref[s] = nref[bi];
                nref[bi] = tr;
                const int ti = pvt[s];
                pvt[s] = pvt[bi];
                pvt[bi] = ti;
            }
        }
        tm.sync();
        // Householder vector of column s (rows s..mrows-1), dlarfg convention, by the first warp.
        df *x = A + (size_t) s * lda;
        df *rts = reinterpret_cast<df *>(red + 40);  // tau and scale
        df t = df_f(0.f);
        if (warp == 0) {
            for (int i = s + 1 + lane; i < mrows; i += 32) t = df_fma(x[i], x[i], t);
            t = group_sum(t, 32);
        }
        if (tm.tid == 0) {
            const df alpha = x[s];
            df tau = df_f(0.f), scale = df_f(0.f), beta = alpha;
            if (t.h != 0.f) {
                const df nrmx = df_sqrt(df_fma(alpha, alpha, t));
                beta = alpha.h >= 0.f ? -nrmx : nrmx;
                tau = df_div(df_add(beta, -alpha), beta);
                scale = df_div(df_f(1.f), df_add(alpha, -beta));
            }
            x[s] = beta;
            rts[0] = tau;
            rts[1] = scale;
        }
        tm.sync();
        const df tau = rts[0], scale = rts[1];
        for (int i = s + 1 + tm.tid; i < mrows; i += tm.nth) x[i] = df_mul(x[i], scale);
        tm.sync();
        if (mrows <= 64) qrcp_apply_df<4>(tm, A, lda, mrows, ncols, s, x, tau, nrm, nref);
        else if (mrows <= 256) qrcp_apply_df<8>(tm, A, lda, mrows, ncols, s, x, tau, nrm, nref);
        else qrcp_apply_df<16>(tm, A, lda, mrows, ncols, s, x, tau, nrm, nref);
        tm.sync();
    }
    return rkeep;
}

template <int RPL, class TM>
__device__ void core_update(const TM &tm, const DevUpdate *ups, const Workspace &ws, const Params &p, int slot,
                            double *sm, int smem_doubles, int &s_rot, int &s_rank, int &s_emax, double &s_amax);

// Stage key of an update in ws.order (sorted by decreasing key): its stack width k when C is
// compressed.  Both fields are written by the plan kernel only, so the key is stable while the
// heavy stages run.
__device__ __forceinline__ int order_key(const Workspace &ws, int slot) {
    const int *m = ws.meta + (size_t) slot * META_INTS;
    return m[META_CKIND] ? m[META_K] : 0;
}

// CTA of SVD_THREADS threads, in one of three team layouts chosen by the update's stack width k:
// heavy (k > kthr: the core does not fit half of the shared memory) — the whole CTA for one update;
// light (kthr4 < k <= kthr) — two half-CTA teams of SVD_THREADS / 2 threads, one update each, each
// with half of the shared memory and its own named barrier; small (k <= kthr4: the core fits a
// quarter) — four teams of SVD_THREADS / 4 threads.  Small cores are latency-bound (per-step
// barriers, dependent FP64 chains), so four of them per SM hide each other's latency.  With ws.order
// (sorted by decreasing k) the classes are contiguous: CTA b < H takes order[b]; the next ceil(L / 2)
// CTAs take the L light updates in pairs; the rest take the small ones in fours.  Without an order
// (one update per CTA) the team size follows the same class rule, so an update's arithmetic never
// depends on the launch it is part of.
template <int RPL>
__global__ void __launch_bounds__(SVD_THREADS, 1) core_svd_kernel(const DevUpdate *ups, int nup, Workspace ws,
                                                               Params p, int team_doubles, int kthr, int kthr4) {
    extern __shared__ double smem_all[];
    __shared__ int s_rot_a[4], s_rank_a[4], s_emax_a[4], s_nheavy, s_nlight;
    __shared__ double s_amax_a[4];
    if (threadIdx.x == 0) {
        int h = -1, h2 = -1;
        if (ws.order) {
            auto count_above = [&](int thr) {  // entries with key > thr (keys descending)
                int lo = 0, hi = nup;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (order_key(ws, ws.order[mid]) > thr) lo = mid + 1;
                    else hi = mid;
                }
                return lo;
            };
            h = count_above(kthr);
            h2 = count_above(kthr4);
        }
        s_nheavy = h;
        s_nlight = h2 - h;
    }
    __syncthreads();
    const int H = s_nheavy, NL = s_nlight;
    constexpr int HALF = SVD_THREADS / 2, QUART = SVD_THREADS / 4;
    const int quarter_doubles = team_doubles / 2;
    int idx, part = 0, cls;  // cls 0 heavy, 1 light, 2 small
    if (H < 0) {
        idx = blockIdx.x;
        if (idx >= nup) return;
        const int key = order_key(ws, idx);
        cls = key > kthr ? 0 : (key > kthr4 ? 1 : 2);
        if (cls == 1 && threadIdx.x >= HALF) return;
        if (cls == 2 && threadIdx.x >= QUART) return;
    } else {
        const int b = blockIdx.x, nlb = (NL + 1) / 2;
        if (b < H) {
            idx = b;
            cls = 0;
        } else if (b < H + nlb) {
            cls = 1;
            part = threadIdx.x / HALF;
            idx = H + 2 * (b - H) + part;
            if (idx >= H + NL) return;  // the odd light update's partner slot stays idle
        } else {
            cls = 2;
            part = threadIdx.x / QUART;
            idx = H + NL + 4 * (b - H - nlb) + part;
        }
    }
    if (idx >= nup) return;
    if (cls == 0)
        core_update<RPL>(Team<SVD_THREADS>{(int) threadIdx.x, 1}, ups, ws, p, ws.heavy(idx), smem_all,
                         2 * team_doubles, s_rot_a[0], s_rank_a[0], s_emax_a[0], s_amax_a[0]);
    else if (cls == 1)
        core_update<RPL>(Team<HALF>{(int) threadIdx.x % HALF, 1 + part}, ups, ws, p, ws.heavy(idx),
                         smem_all + (size_t) part * team_doubles, team_doubles, s_rot_a[part], s_rank_a[part],
                         s_emax_a[part], s_amax_a[part]);
    else
        core_update<RPL>(Team<QUART>{(int) threadIdx.x % QUART, 1 + part}, ups, ws, p, ws.heavy(idx),
                         smem_all + (size_t) part * quarter_doubles, quarter_doubles, s_rot_a[part], s_rank_a[part],
                         s_emax_a[part], s_amax_a[part]);
}

// The recompression core of one update (slot) by one team, with `smem_doubles` of shared memory at sm.
template <int RPL, class TM>
__device__ void core_update(const TM &tm, const DevUpdate *ups, const Workspace &ws, const Params &p, int slot,
                            double *sm, int smem_doubles, int &s_rot, int &s_rank, int &s_emax, double &s_amax) {
    int *meta = ws.meta + (size_t) slot * META_INTS;
    if (meta[META_STATUS] != HCGB_OK || !meta[META_CKIND]) return;
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    const int lr = lane >> 2, lc = lane & 3;
    const int k = meta[META_K], m = meta[META_M], n = meta[META_N];
    const int kU = m < k ? m : k, kV = n < k ? n : k;
    const int ld = ws.ld, ldm = ws.kmax;
    double *base = ws.slot(slot);
    const double *RU = base + ws.off_ustack;
    const double *RV = base + ws.off_vstack;
    double *Mc = base + ws.off_mcopy;
    // Aux arrays at the start of the team's shared memory, sized by this update's stack width ka
    // (every index below is < k): sorted sigma, scratch, column norms, the sort permutation, the QR
    // pivots, the Jacobi scales and a reduction area (64 doubles + 128 ints).
    const int ka = k > 0 ? k : 1;
    double *sig = sm;
    double *inv = sig + ka;
    double *nrm = inv + ka;
    int *perm = reinterpret_cast<int *>(nrm + ka);
    int *pvt = perm + ka;
    double *dsc = nrm + ka + ka + 1;  // Jacobi column scales d and 1/d (2 ka)
    double *red = dsc + 2 * ka;
    int *redi = reinterpret_cast<int *>(red + SVD_RED_DOUBLES);
    double *pool = red + SVD_RED_DOUBLES + SVD_REDI_INTS / 2;
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

    const long long t0 = clock64();
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
    tm.sync();

    // 2. Rank-revealing QR with column pivoting, M P = Q R, stopped once every remaining column
    //    is below QRCP_STOP (1e-2) of the truncation threshold.  The dropped block R22 lies far
    //    below the threshold: it cannot carry a kept singular value, it moves the kept ones by at
    //    most ||R22||_2 <= sqrt(kV) * 1e-2 * threshold (in practice ~1e-6 relative), and it only
    //    holds directions the truncation discards anyway.  The Jacobi stage then works on the
    //    rk rows above it.  (Fixed-rank mode keeps every row.)
    constexpr double QRCP_STOP = 1e-2;
    double stop2 = -1.0, rel = 0.0;
    if (p.fixed_rank <= 0) {
        if (p.truncated) {
            stop2 = 0.0;
            rel = QRCP_STOP * p.accuracy;  // |r_00| <= sigma_0, so this threshold is conservative
        } else {
            stop2 = (QRCP_STOP * p.accuracy) * (QRCP_STOP * p.accuracy);
        }
    }
    const long long t1 = clock64();
    int rk;
    int eshift = 0;  // mixed form: Mw holds float-float values of M * 2^-eshift from here to step 4
    if (p.mode == 1) {
        // Exact power-of-two scaling that brings the largest entry of M near 1 (float range), then
        // the pivoted QR and the Jacobi sweeps in float-float arithmetic on the FP32 pipe.
        if (tm.tid == 0) s_emax = 0;
        tm.sync();
        int em = 0;
        for (int e = tm.tid; e < kU * kV; e += tm.nth) {
            const int ef = (int) ((__double_as_longlong(Mw[(e % kU) + (size_t) (e / kU) * ldw]) >> 52) & 0x7ff);
            em = em > ef ? em : ef;
        }
        atomicMax(&s_emax, em);
        tm.sync();
        eshift = s_emax ? s_emax - 1023 : 0;
        const double down = __hiloint2double((1023 - eshift) << 20, 0);
        df *Md = reinterpret_cast<df *>(Mw);
        for (int e = tm.tid; e < kU * kV; e += tm.nth) {
            const size_t o = (e % kU) + (size_t) (e / kU) * ldw;
            Md[o] = df(Mw[o] * down);
        }
        tm.sync();
        const float stop2f = stop2 > 0.0 ? (float) (stop2 * down * down) : (float) stop2;
        rk = qrcp_truncated_df(tm, Md, ldw, kU, kV, stop2f, (float) (rel * rel), reinterpret_cast<df *>(nrm),
                               reinterpret_cast<df *>(inv), pvt, reinterpret_cast<float *>(red), redi);
    } else {
        rk = qrcp_truncated(tm, Mw, ldw, kU, kV, stop2, rel, nrm, inv, pvt, red, redi);
    }
    const long long t2 = clock64();
    if (rk < 1) rk = 1;
    double *XV = base + ws.off_xv;
    // 3. X = R(0:rk, :)^T (kV x rk), staged through XV, then into the working buffer (ld kV).
    for (int i = warp; i < rk; i += nw)
        for (int l = lane; l < kV; l += 32) XV[l + (size_t) i * ld] = l >= i ? Mw[i + (size_t) l * ldw] : 0.0;
    tm.sync();
    double *X = Mw;
    const int ldx = kV;
    for (int i = warp; i < rk; i += nw)
        for (int l = lane; l < kV; l += 32) X[l + (size_t) i * ldx] = XV[l + (size_t) i * ld];
    tm.sync();

    // 4. One-sided Jacobi on the rk columns of X (lane group sized to the column length kV).
    //    X J = W with orthogonal columns: sigma_i = ||w_i||, right singular vectors P W Sigma^-1.
    int sweeps = 0;
    bool converged = true;
    const double tol64 = 8.0 * DBL_EPSILON * (double) (kV > 1 ? kV : 1);
    if (p.mode == 1) {
        // Mixed form: X = R_rk^T is already float-float (scaled by 2^-eshift); the sweeps run in
        // float-float arithmetic, every per-pair quantity included (see jacobi_sweep_df).
        df *Xd = reinterpret_cast<df *>(X);
        const double up = __hiloint2double((1023 + eshift) << 20, 0);
        const float tol_df = 16.f * 3.5527137e-15f * (float) (kV > 1 ? kV : 1);
        // norms and scales as float-float values in the (double-sized) nrm and dsc arrays
        jacobi_df_dispatch<RPL>(tm, Xd, ldx, kV, rk, reinterpret_cast<df *>(nrm), reinterpret_cast<df *>(dsc),
                                reinterpret_cast<df *>(dsc + ka), &s_rot, reinterpret_cast<float *>(&s_amax),
                                &sweeps, &converged, tol_df, MAX_JACOBI_SWEEPS);
        for (int e = tm.tid; e < kV * rk; e += tm.nth) {
            const size_t o = (e % kV) + (size_t) (e / kV) * ldx;
            X[o] = (double) Xd[o] * up;
        }
        tm.sync();
    } else {
        // X32 (kV x rk floats) and J (rk x rk float-float): in shared memory behind X when they fit
        // the team's pool, else in the float region of the slot.
        const size_t x32_floats = ((size_t) kV * rk + 1) & ~size_t(1);
        const size_t pre_doubles = x32_floats / 2 + (size_t) rk * rk;
        const bool in_smem = Mw == pool && (size_t) kV * rk + pre_doubles <= (size_t) pool_doubles;
        const bool fits = in_smem || x32_floats + 2 * (size_t) rk * rk <= (size_t) ws.kmax * (ws.kmax + ws.ld);
        if (rk >= p.precond_min && fits) {
            // FP32 sweeps with accumulated rotations (FP32 pipe), then X <- X J in FP64: the FP64
            // sweeps below start from a nearly orthogonal X and need about half as many.
            float *X32 = reinterpret_cast<float *>(in_smem ? pool + (size_t) kV * rk : base + ws.off_mixed);
            df *J32 = reinterpret_cast<df *>(X32 + x32_floats);
            if (tm.tid == 0) s_emax = 0;
            tm.sync();
            int em = 0;
            for (int e = tm.tid; e < kV * rk; e += tm.nth) {
                const int ef = (int) ((__double_as_longlong(X[(e % kV) + (size_t) (e / kV) * ldx]) >> 52) & 0x7ff);
                em = em > ef ? em : ef;
            }
            atomicMax(&s_emax, em);
            tm.sync();
            const int esc = s_emax ? s_emax - 1023 : 0;
            const double down = __hiloint2double((1023 - esc) << 20, 0);
            for (int e = tm.tid; e < kV * rk; e += tm.nth)
                X32[e] = (float) (X[(e % kV) + (size_t) (e / kV) * ldx] * down);
            tm.sync();
            jacobi_precond32(tm, X32, kV, rk, J32, PRECOND_TOL32, PRECOND_MAX_SWEEPS, &s_rot);
            // XV (ld ws.ld) <- X J32 in FP64, then back into X
            for (int e = tm.tid; e < kV * rk; e += tm.nth) {
                const int r = e % kV, c = e / kV;
                const df *jc = J32 + (size_t) c * rk;
                double s0 = 0.0, s1 = 0.0;
                int l = 0;
                for (; l + 1 < rk; l += 2) {
                    s0 = fma(X[r + (size_t) l * ldx], (double) jc[l], s0);
                    s1 = fma(X[r + (size_t) (l + 1) * ldx], (double) jc[l + 1], s1);
                }
                if (l < rk) s0 = fma(X[r + (size_t) l * ldx], (double) jc[l], s0);
                XV[r + (size_t) c * ld] = s0 + s1;
            }
            tm.sync();
            for (int e = tm.tid; e < kV * rk; e += tm.nth) {
                const int r = e % kV, c = e / kV;
                X[r + (size_t) c * ldx] = XV[r + (size_t) c * ld];
            }
            tm.sync();
        }
        jacobi_dispatch<RPL>(tm, X, ldx, kV, rk, nrm, &s_rot, &s_amax, &sweeps, &converged, tol64, MAX_JACOBI_SWEEPS,
                             dsc, ka, Mw == pool);
    }

    const long long t3 = clock64();
    // 5. Singular values, descending order (stable), rank rule (omp/kernels.cpp:82-104).
    for (int j = warp; j < rk; j += nw) {
        const double *col = X + (size_t) j * ldx;
        double t = 0.0;
        for (int r = lane; r < kV; r += 32) t = fma(col[r], col[r], t);
        t = warp_sum(t);
        if (lane == 0) inv[j] = sqrt(t);  // unsorted sigma, temporarily in inv[]
    }
    tm.sync();
    for (int j = tm.tid; j < rk; j += tm.nth) {
        const double sj = inv[j];
        int pos = 0;
        for (int l = 0; l < rk; l++) {
            const double sl = inv[l];
            pos += (sl > sj) || (sl == sj && l < j);
        }
        perm[pos] = j;
        sig[pos] = sj;
    }
    tm.sync();
    if (tm.tid == 0) {
        const int sizeS = kU < kV ? kU : kV;
        int r;
        if (p.fixed_rank > 0) {
            r = p.fixed_rank < k ? p.fixed_rank : k;
        } else {
            // sigma_i for i >= rk are below the threshold by construction of the QR stop.
            r = rk < sizeS ? rk : sizeS;
            const double thr = p.truncated ? p.accuracy * sig[0] : p.accuracy;
            for (int i = 1; i < rk; i++)
                if (sig[i] < thr) {
                    r = i;
                    break;
                }
        }
        if (r < 1) r = 1;
        const int maxr = ups[slot].c.max_rank;
        if (r > maxr) r = maxr;
        if (r > rk) r = rk;
        s_rank = r;
        base[ws.off_sigma] = sig[0];  // the largest singular value (the learned form's residual test)
        meta[META_NEWRANK] = r;
        meta[META_SWEEPS] = sweeps;
        meta[META_CORE_COLS] = rk;
        if (!converged) meta[META_STATUS] = HCGB_NOT_CONVERGED;
    }
    tm.sync();
    const int r = s_rank;
    for (int i = tm.tid; i < r; i += tm.nth) inv[i] = sig[i] > 1e-150 ? 1.0 / (sig[i] * sig[i]) : 0.0;

    // 6. Right factor in the small basis: XV = P W_r (= V_r Sigma_r), n rows, zero below kV.
    for (int i = warp; i < r; i += nw) {
        const double *w = X + (size_t) perm[i] * ldx;
        for (int l = lane; l < kV; l += 32) XV[pvt[l] + (size_t) i * ld] = w[l];
        for (int l = kV + lane; l < n; l += 32) XV[l + (size_t) i * ld] = 0.0;
    }
    tm.sync();

    // 7. Left factor in the small basis: C.U[:, i] = [M XV[:, i] / sigma_i^2 ; 0] (= U_r), on DMMA.
    double *CU = ups[slot].c.data;
    const int ldcu = ups[slot].c.rows;
    {
        const int ntr = (kU + 7) >> 3, ntc = (r + 7) >> 3;
        for (int idx = warp; idx < ntr * ntc; idx += nw) {
            const int tr = idx % ntr, tc = idx / ntr;
            const int irow = tr * 8 + lr, icol = tc * 8 + lr;
            const double *vcol = XV + (size_t) (icol < r ? icol : 0) * ld;
            double d0 = 0.0, d1 = 0.0;
            for (int l4 = 0; l4 < kV; l4 += 4) {
                const int l = l4 + lc;
                const double av = (irow < kU && l < kV) ? Mc[irow + (size_t) l * ldm] : 0.0;
                const double bv = (icol < r && l < kV) ? vcol[l] : 0.0;
                dmma(d0, d1, av, bv);
            }
            const int col = tc * 8 + 2 * lc;
            if (irow < kU && col < r) CU[irow + (size_t) col * ldcu] = d0 * inv[col];
            if (irow < kU && col + 1 < r) CU[irow + (size_t) (col + 1) * ldcu] = d1 * inv[col + 1];
        }
        for (int i = warp; i < r; i += nw)
            for (int l = kU + lane; l < m; l += 32) CU[l + (size_t) i * ldcu] = 0.0;
    }
    if (tm.tid == 0) {
        const long long t4 = clock64();
        meta[META_KC_PRODUCT] = (int) ((t1 - t0) >> 10);
        meta[META_KC_QRCP] = (int) ((t2 - t1) >> 10);
        meta[META_KC_JACOBI] = (int) ((t3 - t2) >> 10);
        meta[META_KC_FACTORS] = (int) ((t4 - t3) >> 10);
    }
}

}  // namespace

namespace {

// Doubles of shared memory per half-CTA team: everything a core of kmax columns could use, capped at
// half of the per-block opt-in limit (less a reserve for the kernel's static shared variables), and
// never below the aux arrays.
int svd_team_doubles(int kmax) {
    static const int optin = [] {  // thread-safe one-time initialisation
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        return v > 0 ? v : 48 * 1024;
    }();
    const long aux = 6L * kmax + SVD_AUX_FIXED;
    const long want = aux + (long) kmax * kmax;
    const long cap = (optin - 256) / 2 / (long) sizeof(double);
    long t = want < cap ? want : cap;
    if (t < aux) t = aux;  // checked against the device limit by the caller
    return (int) t;
}

}  // namespace

size_t svd_smem_bytes(int kmax) { return 2 * sizeof(double) * (size_t) svd_team_doubles(kmax); }

template <int RPL>
static void launch_core_svd_t(const DevUpdate *ups, int n, Workspace ws, Params p, cudaStream_t st) {
    const int team = svd_team_doubles(ws.kmax);
    const size_t smem = 2 * sizeof(double) * (size_t) team;
    // Heavy: a core of k columns (its aux arrays, 6 k + SVD_AUX_FIXED doubles, and a k x k working
    // copy) does not fit the half-CTA team's shared memory; small: it fits a quarter-CTA team's.
    auto fits = [](long k, long doubles) { return k * k + 6 * k + SVD_AUX_FIXED <= doubles; };
    int kthr = 0, kthr4 = 0;
    while (fits(kthr + 1, team)) kthr++;
    while (fits(kthr4 + 1, team / 2)) kthr4++;
    cudaFuncSetAttribute(core_svd_kernel<RPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    { core_svd_kernel<RPL><<<n, SVD_THREADS, smem, st>>>(ups, n, ws, p, team, kthr, kthr4); note_launch(); }
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
