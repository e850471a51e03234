// Batched blocked Householder QR of the stacked factors and application of the resulting Q.
//
// Replaces HCoreKernels::Geqrf / ungqr / Unmqr on the TLR GEMM path
// (src/operators/concrete/Compressed.cpp:353, :384, :551, :611; LAPACK dgeqrf/dorgqr semantics:
// R on and above the diagonal, unit-lower reflectors below it, tau_j = 2 / (v_j^T v_j)).
//
// Plain form: one CTA per matrix.  The matrix stays in device memory (L2-resident working
// set); each panel of QR_NB columns is staged in shared memory and factored there with SIMT FP64
// and warp-shuffle norms; the compact-WY factor T (Q_panel = I - V T V^T, LAPACK dlarft) is kept
// for the later Q application; the trailing update A <- (I - V T^T V^T) A is two FP64
// tensor-core (DMMA) products with V and W = V^T A staged in shared memory.
// Mixed form (qr_kernel_df, apply_q_kernel_df): the same panels in float-float arithmetic on the
// FP32 pipe, one team per side (a whole 512-thread CTA for a wide stack, half a CTA otherwise).
#include "internal.cuh"
#include "df.cuh"

namespace hcgb {

namespace {

constexpr int NB = QR_NB;
constexpr int QR_THREADS = 256;
constexpr int QRD_THREADS = 512;  // mixed-form kernels: one heavy side, or both sides of a light update
constexpr int QR_HEAVY_K = 95;    // sides of updates with a wider stack get a whole CTA

__host__ __device__ __forceinline__ int round_up(int x, int m) { return (x + m - 1) / m * m; }

// Width of the W = V^T X buffer: the trailing columns are updated in chunks of at most this many.
__host__ __device__ __forceinline__ int qr_w_cols(int kmax) {
    const int w = round_up(kmax, 8);
    return w < 512 ? w : 512;
}

// Householder QR of the panel in shared memory: column c at Ps + c*ldp, rows 0..mr-1.
// LAPACK dlarfg convention: beta = -sign(alpha) * ||x||, tau = (beta - alpha) / beta,
// v = x / (alpha - beta) with v_0 = 1 implicit; tau = 0 when the tail is zero.
__device__ void factor_panel(double *Ps, int ldp, int mr, int nbp, double *tau_s, double *red) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int j = 0; j < nbp; j++) {
        double *x = Ps + (size_t) j * ldp;
        // the reflector's norm on the first warp alone: a block-wide sum would issue eight warps'
        // reductions on the FP64 pipe and cost two more barriers
        double ss = 0.0;
        if (warp == 0) {
            for (int r = j + 1 + lane; r < mr; r += 32) ss = fma(x[r], x[r], ss);
            ss = warp_sum(ss);
        }
        if (threadIdx.x == 0) {
            const double alpha = x[j];
            double tau = 0.0, scale = 0.0, beta = alpha;
            if (ss != 0.0) {
                beta = -copysign(sqrt(fma(alpha, alpha, ss)), alpha);
                tau = (beta - alpha) / beta;
                scale = 1.0 / (alpha - beta);
            }
            tau_s[j] = tau;
            red[40] = scale;
            x[j] = beta;
        }
        __syncthreads();
        const double scale = red[40], tau = tau_s[j];
        for (int r = j + 1 + threadIdx.x; r < mr; r += blockDim.x) x[r] *= scale;
        __syncthreads();
        if (tau != 0.0) {
            for (int c = j + 1 + warp; c < nbp; c += nw) {
                double *y = Ps + (size_t) c * ldp;
                double w = lane == 0 ? y[j] : 0.0;
                for (int r = j + 1 + lane; r < mr; r += 32) w = fma(x[r], y[r], w);
                w = warp_sum(w) * tau;
                if (lane == 0) y[j] -= w;
                for (int r = j + 1 + lane; r < mr; r += 32) y[r] = fma(-w, x[r], y[r]);
            }
        }
        __syncthreads();
    }
}

// Float-float version of factor_panel (mixed form), in place on the panel held as float-float
// values of (panel * 2^-eshift); same dlarfg convention.  red: >= 24 doubles of scratch.
template <class TM>
__device__ void factor_panel_df(const TM &tm, df *Ps, int ldp, int mr, int nbp, double *tau_s, double *red) {
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    df *redd = reinterpret_cast<df *>(red);
    for (int j = 0; j < nbp; j++) {
        df *x = Ps + (size_t) j * ldp;
        // the reflector's norm on the first warp alone (no team-wide reduction, two barriers fewer)
        df t = df_f(0.f);
        if (warp == 0) {
            for (int r = j + 1 + lane; r < mr; r += 32) t = df_fma(x[r], x[r], t);
            t = df_group_sum(t, 32);
        }
        if (tm.tid == 0) {
            const df alpha = x[j];
            df tau = df_f(0.f), scale = df_f(0.f), beta = alpha;
            if (t.h != 0.f) {
                const df nrmx = df_sqrt(df_fma(alpha, alpha, t));
                beta = alpha.h >= 0.f ? -nrmx : nrmx;
                tau = df_div(df_add(beta, -alpha), beta);
                scale = df_div(df_f(1.f), df_add(alpha, -beta));
            }
            tau_s[j] = (double) tau;
            redd[32] = scale;
            redd[33] = tau;
            x[j] = beta;
        }
        tm.sync();
        const df scale = redd[32], tau = redd[33];
        for (int r = j + 1 + tm.tid; r < mr; r += tm.nth) x[r] = df_mul(x[r], scale);
        tm.sync();
        if (tau.h != 0.f) {
            for (int c = j + 1 + warp; c < nbp; c += nw) {
                df *y = Ps + (size_t) c * ldp;
                df_acc wa = df_acc_init(lane == 0 ? y[j] : df_f(0.f));
                for (int r = j + 1 + lane; r < mr; r += 32) df_acc_fma(wa, x[r], y[r]);
                const df w = df_mul(df_group_sum(df_acc_value(wa), 32), tau);
                if (lane == 0) y[j] = df_add(y[j], -w);
                const df mw = -w;
                for (int r = j + 1 + lane; r < mr; r += 32) y[r] = df_fma(mw, x[r], y[r]);
            }
        }
        tm.sync();
    }
}

// Overwrite the panel with the explicit unit-lower V (zeros above the diagonal, zero padding).
__device__ void make_explicit_v(double *Ps, int ldp, int nbp) {
    for (int e = threadIdx.x; e < NB * ldp; e += blockDim.x) {
        const int c = e / ldp, r = e % ldp;
        if (c >= nbp) Ps[e] = 0.0;
        else if (r < c) Ps[e] = 0.0;
        else if (r == c) Ps[e] = 1.0;
    }
}

// Compact-WY T of the panel (LAPACK dlarft, forward / columnwise):
// T[i][i] = tau_i,  T[0:i, i] = -tau_i * T[0:i, 0:i] * (V[:, 0:i]^T v_i).  Ps holds explicit V.
__device__ void build_t(const double *Ps, int ldp, int mr, int nbp, const double *tau_s, double *Ts, double *Gs) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) Ts[e] = 0.0;
    const int npairs = nbp * (nbp - 1) / 2;
    for (int p = warp; p < npairs; p += nw) {
        int i = 1, base = 0;
        while (base + i <= p) {
            base += i;
            i++;
        }
        const int l = p - base;  // l < i
        const double *vl = Ps + (size_t) l * ldp, *vi = Ps + (size_t) i * ldp;
        double s = 0.0;
        for (int r = i + lane; r < mr; r += 32) s = fma(vl[r], vi[r], s);
        s = warp_sum(s);
        if (lane == 0) Gs[l * NB + i] = s;
    }
    __syncthreads();
    if (warp == 0) {
        const int j = lane;
        for (int i = 0; i < nbp; i++) {
            double v = 0.0;
            if (j < i) {
                for (int l = j; l < i; l++) v = fma(Ts[j * NB + l], Gs[l * NB + i], v);
                v *= -tau_s[i];
            }
            __syncwarp();
            if (j < i) Ts[j * NB + i] = v;
            if (j == i) Ts[i * NB + i] = tau_s[i];
            __syncwarp();
        }
    }
    __syncthreads();
}

// X (mr x nt, ld ldx) <- (I - V op(T) V^T) X with V = Ps (explicit, NB columns, ldp), T = Ts.
// trans_t: op(T) = T^T (applying Q^T, the QR trailing update); else op(T) = T (applying Q).
__device__ void apply_block_reflector_cols(const double *Ps, int ldp, const double *Ts, bool trans_t, double *X,
                                           int ldx, int mr, int nt, double *Ws, int ldw);

// Columns are processed in chunks of at most ldw (the width of the W buffer in shared memory).
__device__ void apply_block_reflector(const double *Ps, int ldp, const double *Ts, bool trans_t, double *X, int ldx,
                                      int mr, int nt, double *Ws, int ldw) {
    for (int c0 = 0; c0 < nt; c0 += ldw)
        apply_block_reflector_cols(Ps, ldp, Ts, trans_t, X + (size_t) c0 * ldx, ldx, mr,
                                   nt - c0 < ldw ? nt - c0 : ldw, Ws, ldw);
}

__device__ void apply_block_reflector_cols(const double *Ps, int ldp, const double *Ts, bool trans_t, double *X,
                                           int ldx, int mr, int nt, double *Ws, int ldw) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int lr = lane >> 2, lc = lane & 3;
    if (nt <= 0 || mr <= 0) return;
    const int nct = (nt + 7) >> 3;
    // Step A: W = V^T X  (NB x nt), K = rows.
    for (int ct = warp; ct < nct; ct += nw) {
        double a0 = 0.0, a1 = 0.0, b0 = 0.0, b1 = 0.0;
        const int col = ct * 8 + lr;
        const bool colok = col < nt;
        const double *xc = X + (size_t) (colok ? col : 0) * ldx;
        int r4 = 0;
        for (; r4 + 16 <= mr; r4 += 16) {
            double bv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) bv[q] = colok ? xc[r4 + 4 * q + lc] : 0.0;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int r = r4 + 4 * q + lc;
                dmma(a0, a1, Ps[(size_t) lr * ldp + r], bv[q]);
                dmma(b0, b1, Ps[(size_t) (8 + lr) * ldp + r], bv[q]);
            }
        }
        for (; r4 < mr; r4 += 4) {
            const int r = r4 + lc;
            const double bv = (colok && r < mr) ? xc[r] : 0.0;
            dmma(a0, a1, Ps[(size_t) lr * ldp + r], bv);
            dmma(b0, b1, Ps[(size_t) (8 + lr) * ldp + r], bv);
        }
        const int c0 = ct * 8 + 2 * lc;
        Ws[lr * ldw + c0] = a0;
        Ws[lr * ldw + c0 + 1] = a1;
        Ws[(8 + lr) * ldw + c0] = b0;
        Ws[(8 + lr) * ldw + c0 + 1] = b1;
    }
    __syncthreads();
    // Step B: W <- -op(T) W, one column per thread.
    for (int c = threadIdx.x; c < nct * 8; c += blockDim.x) {
        double w[NB], o[NB];
#pragma unroll
        for (int i = 0; i < NB; i++) w[i] = Ws[i * ldw + c];
#pragma unroll
        for (int i = 0; i < NB; i++) {
            double s = 0.0;
            if (trans_t) {
#pragma unroll
                for (int l = 0; l <= i; l++) s = fma(Ts[l * NB + i], w[l], s);
            } else {
#pragma unroll
                for (int l = i; l < NB; l++) s = fma(Ts[i * NB + l], w[l], s);
            }
            o[i] = -s;
        }
#pragma unroll
        for (int i = 0; i < NB; i++) Ws[i * ldw + c] = o[i];
    }
    __syncthreads();
    // Step C: X += V W  (mr x nt), K = NB.
    const int nrt = (mr + 7) >> 3;
    for (int idx = warp; idx < nrt * nct; idx += nw) {
        const int rt = idx % nrt, ct = idx / nrt;
        const int row = rt * 8 + lr, c0 = ct * 8 + 2 * lc;
        const bool rok = row < mr;
        double d0 = (rok && c0 < nt) ? X[row + (size_t) c0 * ldx] : 0.0;
        double d1 = (rok && c0 + 1 < nt) ? X[row + (size_t) (c0 + 1) * ldx] : 0.0;
#pragma unroll
        for (int ks = 0; ks < NB; ks += 4) {
            const double av = Ps[(size_t) (ks + lc) * ldp + rt * 8 + lr];
            const double bv = Ws[(ks + lc) * ldw + ct * 8 + lr];
            dmma(d0, d1, av, bv);
        }
        if (rok && c0 < nt) X[row + (size_t) c0 * ldx] = d0;
        if (rok && c0 + 1 < nt) X[row + (size_t) (c0 + 1) * ldx] = d1;
    }
    __syncthreads();
}

struct QrShared {
    double *Ps, *Ws, *Ts, *Gs, *red, *tau;
    int ldp, ldw;
};

__device__ QrShared carve(double *sm, int ld, int kmax) {
    QrShared s;
    s.ldp = round_up(ld, 8);
    s.ldw = qr_w_cols(kmax);
    s.Ps = sm;
    s.Ws = s.Ps + (size_t) NB * s.ldp;
    s.Ts = s.Ws + (size_t) NB * s.ldw;
    s.Gs = s.Ts + NB * NB;
    s.red = s.Gs + NB * NB;
    s.tau = s.red + 64;
    return s;
}

// grid = 2 * n: block 2s factors the U stack of update s, block 2s+1 its V stack.
__global__ void __launch_bounds__(QR_THREADS) qr_kernel(Workspace ws) {
    extern __shared__ double sm[];
    const int slot = ws.heavy(blockIdx.x >> 1), side = blockIdx.x & 1;
    const int *meta = ws.meta + (size_t) slot * META_INTS;
    if (meta[META_STATUS] != HCGB_OK || !meta[META_CKIND]) return;
    const int k = meta[META_K];
    const int m = side ? meta[META_N] : meta[META_M];
    double *base = ws.slot(slot);
    double *A = base + (side ? ws.off_vstack : ws.off_ustack);
    double *tau = base + (side ? ws.off_tauv : ws.off_tauu);
    double *Tg = base + (side ? ws.off_tv : ws.off_tu);
    const int lda = ws.ld;
    QrShared s = carve(sm, ws.ld, ws.kmax);
    const int kk = m < k ? m : k;
    for (int j0 = 0; j0 < kk; j0 += NB) {
        const int nbp = (kk - j0) < NB ? (kk - j0) : NB;
        const int mr = m - j0;
        for (int e = threadIdx.x; e < NB * s.ldp; e += blockDim.x) {
            const int c = e / s.ldp, r = e % s.ldp;
            s.Ps[e] = (c < nbp && r < mr) ? A[(j0 + r) + (size_t) (j0 + c) * lda] : 0.0;
        }
        __syncthreads();
        factor_panel(s.Ps, s.ldp, mr, nbp, s.tau, s.red);
        for (int e = threadIdx.x; e < nbp * mr; e += blockDim.x) {
            const int c = e / mr, r = e % mr;
            A[(j0 + r) + (size_t) (j0 + c) * lda] = s.Ps[(size_t) c * s.ldp + r];
        }
        if (threadIdx.x < nbp) tau[j0 + threadIdx.x] = s.tau[threadIdx.x];
        __syncthreads();
        make_explicit_v(s.Ps, s.ldp, nbp);
        __syncthreads();
        build_t(s.Ps, s.ldp, mr, nbp, s.tau, s.Ts, s.Gs);
        for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) Tg[(size_t) (j0 / NB) * NB * NB + e] = s.Ts[e];
        const int c0 = j0 + nbp;
        apply_block_reflector(s.Ps, s.ldp, s.Ts, true, A + j0 + (size_t) c0 * lda, lda, mr, k - c0, s.Ws, s.ldw);
    }
}

// ---------------------------------------------------------------------------------------------
// Mixed form of the stack QR: the whole stack is held as float-float values (scaled by a power of
// two) while it is factored, so the panels, the compact-WY T and the trailing updates run on the
// FP32 pipe; R and the reflectors are written back in double at the end (R scaled back, the
// reflectors and tau are scale-free).
// ---------------------------------------------------------------------------------------------
template <class TM>
__device__ void make_explicit_v_df(const TM &tm, df *Ps, int ldp, int nbp) {
    for (int e = tm.tid; e < NB * ldp; e += tm.nth) {
        const int c = e / ldp, r = e % ldp;
        if (c >= nbp || r < c) Ps[e] = df_f(0.f);
        else if (r == c) Ps[e] = df_f(1.f);
    }
}

template <class TM>
__device__ void build_t_df(const TM &tm, const df *Ps, int ldp, int mr, int nbp, const double *tau_s, df *Ts, df *Gs) {
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    for (int e = tm.tid; e < NB * NB; e += tm.nth) Ts[e] = df_f(0.f);
    const int npairs = nbp * (nbp - 1) / 2;
    for (int p = warp; p < npairs; p += nw) {
        int i = 1, base = 0;
        while (base + i <= p) {
            base += i;
            i++;
        }
        const int l = p - base;
        const df *vl = Ps + (size_t) l * ldp, *vi = Ps + (size_t) i * ldp;
        df sacc = df_f(0.f);
        for (int r = i + lane; r < mr; r += 32) sacc = df_fma(vl[r], vi[r], sacc);
        sacc = df_group_sum(sacc, 32);
        if (lane == 0) Gs[l * NB + i] = sacc;
    }
    tm.sync();
    if (warp == 0) {
        const int j = lane;
        for (int i = 0; i < nbp; i++) {
            const df ti = df(tau_s[i]);
            df v = df_f(0.f);
            if (j < i) {
                for (int l = j; l < i; l++) v = df_fma(Ts[j * NB + l], Gs[l * NB + i], v);
                v = -df_mul(v, ti);
            }
            __syncwarp();
            if (j < i) Ts[j * NB + i] = v;
            if (j == i) Ts[i * NB + i] = ti;
            __syncwarp();
        }
    }
    tm.sync();
}

// X (mr x nt, ld ldx, float-float) <- (I - V op(T) V^T) X, columns in chunks of ldw.
template <class TM>
__device__ void apply_block_reflector_df(const TM &tm, const df *Ps, int ldp, const df *Ts, bool trans_t, df *X, int ldx, int mr,
                                         int nt, df *Ws, int ldw) {
    const int warp = tm.warp(), lane = threadIdx.x & 31, nw = tm.nw();
    for (int c0 = 0; c0 < nt; c0 += ldw) {
        const int ntc = nt - c0 < ldw ? nt - c0 : ldw;
        df *Xc = X + (size_t) c0 * ldx;
        // A: W = V^T X, a warp per column, lanes over rows
        for (int c = warp; c < ntc; c += nw) {
            df_acc acc[NB];
#pragma unroll
            for (int i = 0; i < NB; i++) acc[i] = df_acc{0.f, 0.f};
            const df *xc = Xc + (size_t) c * ldx;
            for (int r = lane; r < mr; r += 32) {
                const df xv = xc[r];
#pragma unroll
                for (int i = 0; i < NB; i++) df_acc_fma(acc[i], Ps[(size_t) i * ldp + r], xv);
            }
#pragma unroll
            for (int i = 0; i < NB; i++) {
                const df v = df_group_sum(df_acc_value(acc[i]), 32);
                if (lane == 0) Ws[i * ldw + c] = v;
            }
        }
        tm.sync();
        // B: W <- -op(T) W, a thread per column
        for (int c = tm.tid; c < ntc; c += tm.nth) {
            df w[NB], o[NB];
#pragma unroll
            for (int i = 0; i < NB; i++) w[i] = Ws[i * ldw + c];
#pragma unroll
            for (int i = 0; i < NB; i++) {
                df sacc = df_f(0.f);
                if (trans_t) {
#pragma unroll
                    for (int l = 0; l <= i; l++) sacc = df_fma(Ts[l * NB + i], w[l], sacc);
                } else {
#pragma unroll
                    for (int l = i; l < NB; l++) sacc = df_fma(Ts[i * NB + l], w[l], sacc);
                }
                o[i] = -sacc;
            }
#pragma unroll
            for (int i = 0; i < NB; i++) Ws[i * ldw + c] = o[i];
        }
        tm.sync();
        // C: X += V W, a thread per element (rows fastest: coalesced)
        for (int e = tm.tid; e < mr * ntc; e += tm.nth) {
            const int r = e % mr, c = e / mr;
            df_acc x = df_acc_init(Xc[r + (size_t) c * ldx]);
#pragma unroll
            for (int i = 0; i < NB; i++) df_acc_fma(x, Ps[(size_t) i * ldp + r], Ws[i * ldw + c]);
            Xc[r + (size_t) c * ldx] = df_acc_value(x);
        }
        tm.sync();
    }
}

// One side (U: 0, V: 1) of one update's stack QR in the mixed form, by one team, with the team's
// shared memory at sm.
template <class TM>
__device__ void qr_side_df(const TM &tm, const Workspace &ws, int slot, int side, double *sm, int &s_emax) {
    const int *meta = ws.meta + (size_t) slot * META_INTS;
    if (meta[META_STATUS] != HCGB_OK || !meta[META_CKIND]) return;
    const int k = meta[META_K];
    const int m = side ? meta[META_N] : meta[META_M];
    double *base = ws.slot(slot);
    double *A = base + (side ? ws.off_vstack : ws.off_ustack);
    double *tau = base + (side ? ws.off_tauv : ws.off_tauu);
    double *Tg = base + (side ? ws.off_tv : ws.off_tu);
    const int lda = ws.ld;
    QrShared s = carve(sm, ws.ld, ws.kmax);
    df *Psd = reinterpret_cast<df *>(s.Ps), *Wsd = reinterpret_cast<df *>(s.Ws);
    df *Tsd = reinterpret_cast<df *>(s.Ts), *Gsd = reinterpret_cast<df *>(s.Gs);
    df *Ad = reinterpret_cast<df *>(A);
    // 1. the stack as float-float values of A * 2^-eshift (entries below 2)
    if (tm.tid == 0) s_emax = 0;
    tm.sync();
    int em = 0;
    for (int e = tm.tid; e < m * k; e += tm.nth) {
        const int ef = (int) ((__double_as_longlong(A[(e % m) + (size_t) (e / m) * lda]) >> 52) & 0x7ff);
        em = em > ef ? em : ef;
    }
    atomicMax(&s_emax, em);
    tm.sync();
    const int eshift = s_emax ? s_emax - 1023 : 0;
    const double down = __hiloint2double((1023 - eshift) << 20, 0), up = __hiloint2double((1023 + eshift) << 20, 0);
    for (int e = tm.tid; e < m * k; e += tm.nth) {
        const size_t o = (e % m) + (size_t) (e / m) * lda;
        Ad[o] = df(A[o] * down);
    }
    tm.sync();
    // 2. panels
    const int kk = m < k ? m : k;
    for (int j0 = 0; j0 < kk; j0 += NB) {
        const int nbp = (kk - j0) < NB ? (kk - j0) : NB;
        const int mr = m - j0;
        for (int e = tm.tid; e < NB * s.ldp; e += tm.nth) {
            const int c = e / s.ldp, r = e % s.ldp;
            Psd[e] = (c < nbp && r < mr) ? Ad[(j0 + r) + (size_t) (j0 + c) * lda] : df_f(0.f);
        }
        tm.sync();
        factor_panel_df(tm, Psd, s.ldp, mr, nbp, s.tau, s.red);
        for (int e = tm.tid; e < nbp * mr; e += tm.nth) {
            const int c = e / mr, r = e % mr;
            Ad[(j0 + r) + (size_t) (j0 + c) * lda] = Psd[(size_t) c * s.ldp + r];
        }
        if (tm.tid < nbp) tau[j0 + tm.tid] = s.tau[tm.tid];
        tm.sync();
        make_explicit_v_df(tm, Psd, s.ldp, nbp);
        tm.sync();
        build_t_df(tm, Psd, s.ldp, mr, nbp, s.tau, Tsd, Gsd);
        for (int e = tm.tid; e < NB * NB; e += tm.nth) Tg[(size_t) (j0 / NB) * NB * NB + e] = (double) Tsd[e];
        const int c0 = j0 + nbp;
        apply_block_reflector_df(tm, Psd, s.ldp, Tsd, true, Ad + j0 + (size_t) c0 * lda, lda, mr, k - c0, Wsd, s.ldw);
    }
    // 3. back to double: R (on and above the diagonal) scaled back, reflectors as they are
    for (int e = tm.tid; e < m * k; e += tm.nth) {
        const int r = e % m, c = e / m;
        const size_t o = r + (size_t) c * lda;
        const double v = (double) Ad[o];
        A[o] = r <= c ? v * up : v;
    }
}

// grid = 2 * n: X <- Q X for the U side (X = the C tile's U, m x r) and the V side (X = XV, n x r).
__global__ void __launch_bounds__(QR_THREADS) apply_q_kernel(const DevUpdate *ups, Workspace ws) {
    extern __shared__ double sm[];
    const int slot = ws.heavy(blockIdx.x >> 1), side = blockIdx.x & 1;
    const int *meta = ws.meta + (size_t) slot * META_INTS;
    const int st = meta[META_STATUS];
    if ((st != HCGB_OK && st != HCGB_NOT_CONVERGED) || !meta[META_CKIND]) return;
    if (meta[META_WY] & (1 << side)) return;  // applied in WY form
    const int k = meta[META_K];
    const int m = side ? meta[META_N] : meta[META_M];
    const int r = meta[META_NEWRANK];
    double *base = ws.slot(slot);
    const double *A = base + (side ? ws.off_vstack : ws.off_ustack);
    const double *Tg = base + (side ? ws.off_tv : ws.off_tu);
    double *X;
    int ldx;
    if (side == 0) {
        X = ups[slot].c.data;
        ldx = ups[slot].c.rows;
    } else {
        X = base + ws.off_xv;
        ldx = ws.ld;
    }
    const int lda = ws.ld;
    QrShared s = carve(sm, ws.ld, ws.kmax);
    const int kk = m < k ? m : k;
    const int npan = (kk + NB - 1) / NB;
    for (int p = npan - 1; p >= 0; p--) {
        const int j0 = p * NB;
        const int nbp = (kk - j0) < NB ? (kk - j0) : NB;
        const int mr = m - j0;
        for (int e = threadIdx.x; e < NB * s.ldp; e += blockDim.x) {
            const int c = e / s.ldp, rr = e % s.ldp;
            double v = 0.0;
            if (c < nbp && rr < mr) v = rr > c ? A[(j0 + rr) + (size_t) (j0 + c) * lda] : (rr == c ? 1.0 : 0.0);
            s.Ps[e] = v;
        }
        for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) s.Ts[e] = Tg[(size_t) p * NB * NB + e];
        __syncthreads();
        apply_block_reflector(s.Ps, s.ldp, s.Ts, false, X + j0, ldx, mr, r, s.Ws, s.ldw);
    }
}

// One side of one update's Q application in the mixed form (X <- Q X, X held as float-float values
// scaled by a power of two while the panels are applied, then written back in double), by one team.
template <class TM>
__device__ void apply_q_side_df(const TM &tm, const DevUpdate *ups, const Workspace &ws, int slot, int side,
                                double *sm, int &s_emax) {
    const int *meta = ws.meta + (size_t) slot * META_INTS;
    const int st = meta[META_STATUS];
    if ((st != HCGB_OK && st != HCGB_NOT_CONVERGED) || !meta[META_CKIND]) return;
    if (meta[META_WY] & (1 << side)) return;  // applied in WY form
    const int k = meta[META_K];
    const int m = side ? meta[META_N] : meta[META_M];
    const int r = meta[META_NEWRANK];
    double *base = ws.slot(slot);
    const double *A = base + (side ? ws.off_vstack : ws.off_ustack);
    const double *Tg = base + (side ? ws.off_tv : ws.off_tu);
    double *X;
    int ldx;
    if (side == 0) {
        X = ups[slot].c.data;
        ldx = ups[slot].c.rows;
    } else {
        X = base + ws.off_xv;
        ldx = ws.ld;
    }
    const int lda = ws.ld;
    QrShared s = carve(sm, ws.ld, ws.kmax);
    df *Psd = reinterpret_cast<df *>(s.Ps), *Wsd = reinterpret_cast<df *>(s.Ws), *Tsd = reinterpret_cast<df *>(s.Ts);
    df *Xd = reinterpret_cast<df *>(X);
    if (tm.tid == 0) s_emax = 0;
    tm.sync();
    int em = 0;
    for (int e = tm.tid; e < m * r; e += tm.nth) {
        const int ef = (int) ((__double_as_longlong(X[(e % m) + (size_t) (e / m) * ldx]) >> 52) & 0x7ff);
        em = em > ef ? em : ef;
    }
    atomicMax(&s_emax, em);
    tm.sync();
    const int eshift = s_emax ? s_emax - 1023 : 0;
    const double down = __hiloint2double((1023 - eshift) << 20, 0), up = __hiloint2double((1023 + eshift) << 20, 0);
    for (int e = tm.tid; e < m * r; e += tm.nth) {
        const size_t o = (e % m) + (size_t) (e / m) * ldx;
        Xd[o] = df(X[o] * down);
    }
    tm.sync();
    const int kk = m < k ? m : k;
    const int npan = (kk + NB - 1) / NB;
    for (int p = npan - 1; p >= 0; p--) {
        const int j0 = p * NB;
        const int nbp = (kk - j0) < NB ? (kk - j0) : NB;
        const int mr = m - j0;
        for (int e = tm.tid; e < NB * s.ldp; e += tm.nth) {
            const int c = e / s.ldp, rr = e % s.ldp;
            double v = 0.0;
            if (c < nbp && rr < mr) v = rr > c ? A[(j0 + rr) + (size_t) (j0 + c) * lda] : (rr == c ? 1.0 : 0.0);
            Psd[e] = df(v);
        }
        for (int e = tm.tid; e < NB * NB; e += tm.nth) Tsd[e] = df(Tg[(size_t) p * NB * NB + e]);
        tm.sync();
        apply_block_reflector_df(tm, Psd, s.ldp, Tsd, false, Xd + j0, ldx, mr, r, Wsd, s.ldw);
    }
    for (int e = tm.tid; e < m * r; e += tm.nth) {
        const size_t o = (e % m) + (size_t) (e / m) * ldx;
        X[o] = (double) Xd[o] * up;
    }
}

// Work split of the mixed-form QR and Q-application kernels (CTAs of QRD_THREADS threads): a side
// of an update with k > QR_HEAVY_K gets a whole CTA (CTA b < 2H: side b & 1 of order[b / 2]); the
// other updates take one CTA each, the U side in the first half-CTA team and the V side in the
// second (named barriers 1 and 2, half of the shared memory each); when two teams' shared memory
// does not fit one CTA (pair == 0), each such side takes a CTA of its own, served by the first
// team.  Without an order (one update): CTA b works on side b & 1 of update b / 2 with the team its
// class gets.  A side's team size depends only on its class, so its arithmetic never depends on
// the launch.  Returns false for threads without work.
__device__ bool qr_assign(const Workspace &ws, int nup, int pair, int &slot, int &side, int &half, bool &heavy) {
    __shared__ int s_nheavy;
    if (threadIdx.x == 0) {
        int h = -1;
        if (ws.order) {
            int lo = 0, hi = nup;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                const int *m = ws.meta + (size_t) ws.order[mid] * META_INTS;
                if ((m[META_CKIND] ? m[META_K] : 0) > QR_HEAVY_K) lo = mid + 1;
                else hi = mid;
            }
            h = lo;
        }
        s_nheavy = h;
    }
    __syncthreads();
    const int H = s_nheavy;
    constexpr int HALF = QRD_THREADS / 2;
    half = 0;
    int idx;
    if (H < 0) {
        idx = blockIdx.x >> 1;
        side = blockIdx.x & 1;
        if (idx >= nup) return false;
        const int *m = ws.meta + (size_t) idx * META_INTS;
        heavy = (m[META_CKIND] ? m[META_K] : 0) > QR_HEAVY_K;
        if (!heavy && threadIdx.x >= HALF) return false;
    } else if ((int) blockIdx.x < 2 * H) {
        idx = blockIdx.x >> 1;
        side = blockIdx.x & 1;
        heavy = true;
    } else if (pair) {
        idx = H + ((int) blockIdx.x - 2 * H);
        half = side = threadIdx.x / HALF;
        heavy = false;
        if (idx >= nup) return false;
    } else {
        idx = H + (((int) blockIdx.x - 2 * H) >> 1);
        side = ((int) blockIdx.x - 2 * H) & 1;
        heavy = false;
        if (idx >= nup || threadIdx.x >= HALF) return false;
    }
    slot = ws.heavy(idx);
    return true;
}

// grid = 2 * n (an upper bound on the CTAs the split needs).
__global__ void __launch_bounds__(QRD_THREADS, 1) qr_kernel_df(Workspace ws, int nup, int team_doubles, int pair) {
    extern __shared__ double smq[];
    __shared__ int s_emax[2];
    int slot, side, half;
    bool heavy;
    if (!qr_assign(ws, nup, pair, slot, side, half, heavy)) return;
    if (heavy) qr_side_df(Team<QRD_THREADS>{(int) threadIdx.x, 1}, ws, slot, side, smq, s_emax[0]);
    else
        qr_side_df(Team<QRD_THREADS / 2>{(int) threadIdx.x % (QRD_THREADS / 2), 1 + half}, ws, slot, side,
                   smq + (size_t) half * team_doubles, s_emax[half]);
}

__global__ void __launch_bounds__(QRD_THREADS, 1) apply_q_kernel_df(const DevUpdate *ups, Workspace ws, int nup,
                                                                   int team_doubles, int pair) {
    extern __shared__ double smq[];
    __shared__ int s_emax[2];
    int slot, side, half;
    bool heavy;
    if (!qr_assign(ws, nup, pair, slot, side, half, heavy)) return;
    if (heavy) apply_q_side_df(Team<QRD_THREADS>{(int) threadIdx.x, 1}, ups, ws, slot, side, smq, s_emax[0]);
    else
        apply_q_side_df(Team<QRD_THREADS / 2>{(int) threadIdx.x % (QRD_THREADS / 2), 1 + half}, ups, ws, slot, side,
                        smq + (size_t) half * team_doubles, s_emax[half]);
}

}  // namespace

size_t qr_smem_bytes(int ld, int kmax) {
    const int ldp = round_up(ld, 8), ldw = qr_w_cols(kmax);
    return sizeof(double) * ((size_t) NB * ldp + (size_t) NB * ldw + 2 * NB * NB + 64 + NB);
}

// Whether two teams' panel buffers fit one CTA of the mixed-form kernels.
static bool qr_pair_fits(size_t team_bytes) {
    static const int optin = [] {  // thread-safe one-time initialisation
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        return v > 0 ? v : 48 * 1024;
    }();
    return 2 * team_bytes + 256 <= (size_t) optin;
}

void launch_qr(Workspace ws, int n, bool mixed, cudaStream_t st) {
    const size_t smem = qr_smem_bytes(ws.ld, ws.kmax);
    if (mixed) {
        const int pair = qr_pair_fits(smem) ? 1 : 0;
        const size_t cta = pair ? 2 * smem : smem;
        cudaFuncSetAttribute(qr_kernel_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) cta);
        { qr_kernel_df<<<2 * n, QRD_THREADS, cta, st>>>(ws, n, (int) (smem / sizeof(double)), pair); note_launch(); }
    } else {
        cudaFuncSetAttribute(qr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
        { qr_kernel<<<2 * n, QR_THREADS, smem, st>>>(ws); note_launch(); }
    }
}

void launch_apply_q(const DevUpdate *ups, int n, Workspace ws, bool mixed, cudaStream_t st) {
    if (mixed) {
        const size_t smem = qr_smem_bytes(ws.ld, ws.kmax);
        const int pair = qr_pair_fits(smem) ? 1 : 0;
        const size_t cta = pair ? 2 * smem : smem;
        cudaFuncSetAttribute(apply_q_kernel_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) cta);
        { apply_q_kernel_df<<<2 * n, QRD_THREADS, cta, st>>>(ups, ws, n, (int) (smem / sizeof(double)), pair); note_launch(); }
        return;
    }
    const size_t smem = qr_smem_bytes(ws.ld, ws.kmax);
    cudaFuncSetAttribute(apply_q_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    { apply_q_kernel<<<2 * n, QR_THREADS, smem, st>>>(ups, ws); note_launch(); }
}

}  // namespace hcgb
