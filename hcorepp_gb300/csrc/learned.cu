// The learned recompression form: a rank predictor sizes a randomized sketch of each update's
// product P = U_s V_s^T (the stacked bases of the plain method), the sketch replaces the stacks,
// and the plain recompression runs as the fallback wherever an a-posteriori residual estimate
// says the sketch missed part of P above the truncation threshold.
//
// Per update (after the stacks are formed):
//   features   12 inputs of the predictor (ranks, leading singular-value ratios of the factors,
//              norms, tile distance, accuracy; below)
//   predict    y = MLP(features) ~ log2(1 + new rank)  (mlp.cu)
//   plan       l = ceil(2^y - 1) + 8 (oversampling), taken when l + 4 <= k * sk_pct / 100 (half the
//              stack width by default); Omega = [Omega_l | 4 probe
//              columns], seeded N(0, 1) entries
//   products   Z = V_s^T Omega, Y = P Omega = U_s Z
//   sketch QR  Householder QR of Y[:, :l], its reflectors applied to the probe columns, whose parts
//              below row l are (I - Q Q^T) P w_p; estimate e = 10 sqrt(2/pi) max_p ||.|| (the
//              probabilistic bound of Halko, Martinsson and Tropp, 2011, section 4.3; fails with
//              probability below 10^-4), then Q_Y formed explicitly
//   products   W = U_s^T Q_Y, V' = V_s W, so that Q_Y Q_Y^T P = Q_Y V'^T
//   pass A     the plain pipeline (stack QR, core SVD, truncation, Q application, write-back) on the
//              l-column stacks [Q_Y], [V']
//   test       accepted when e <= the truncation threshold (accuracy * sigma_0 of the sketch core, or
//              accuracy) and the new rank < l (the sketch was not saturated)
//   pass B     the plain pipeline on the original stacks for every update that was not sketched or
//              whose sketch failed: the fallback, which also defines the error bound
//
// No counterpart in the reference (HCore++ always recompresses by full QR + SVD,
// src/operators/concrete/Compressed.cpp:441-527); the truncation rule is the reference's
// (src/kernels/omp/kernels.cpp:82-104) in both passes.
#include <cfloat>

#include "internal.cuh"

namespace hcgb {

namespace {

constexpr int SK_PROBES = 4;
constexpr int SK_OVERSAMPLE = 8;

__device__ __forceinline__ double block_sum(double v, double *red) {
    v = warp_sum(v);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < nw; w++) t += red[w];
    return t;
}

// Squared Frobenius norm and the squared norms of the first three rows of the V factor
// (compressed), or the squared Frobenius norm (dense).
struct TileStats {
    double fro2, row2[3];
    int rank;
    bool dense;
};

__device__ TileStats tile_stats(const DevTile &t, int rank, double *red) {
    TileStats s{};
    s.rank = rank;
    s.dense = t.kind == 0;
    double acc = 0.0;
    if (s.dense) {
        const size_t cnt = (size_t) t.rows * t.cols;
        for (size_t e = threadIdx.x; e < cnt; e += blockDim.x) acc = fma(t.data[e], t.data[e], acc);
        s.fro2 = block_sum(acc, red);
        return s;
    }
    // V region: V (rank x cols, ld rank) or, for compressed_vt, W = V^T (cols x rank, ld cols).
    const double *V = t.v;
    const bool vt = t.kind == HCGB_COMPRESSED_VT;
    const size_t cnt = (size_t) rank * t.cols;
    for (size_t e = threadIdx.x; e < cnt; e += blockDim.x) acc = fma(V[e], V[e], acc);
    s.fro2 = block_sum(acc, red);
    for (int i = 0; i < 3; i++) {
        double a = 0.0;
        if (i < rank)
            for (int c = threadIdx.x; c < t.cols; c += blockDim.x) {
                const double v = vt ? V[c + (size_t) i * t.cols] : V[i + (size_t) c * rank];
                a = fma(v, v, a);
            }
        s.row2[i] = block_sum(a, red);
    }
    return s;
}

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

// log10(sigma_i / sigma_0) / 8 in [-2, 0]; the singular values of a compressed tile whose U has
// orthonormal columns and whose V has orthogonal rows (every tile this library writes, and the
// reference's compressed inputs) are the row norms of V.
__device__ float ratio_feature(const TileStats &s, int i) {
    if (s.dense) return 0.f;
    if (i >= s.rank || s.row2[0] <= 0.0) return -2.f;
    const double r = s.row2[i] / s.row2[0];
    return clampf((float) (0.5 * log10(r > 1e-300 ? r : 1e-300)) / 8.f, -2.f, 0.f);
}

// Features (MLP_IN = 12) of one update:
//   0-2  rank of A, B, C / rows of C (a dense operand counts as full rank)
//   3-4  log10(sigma_1 / sigma_0), log10(sigma_2 / sigma_0) of A, / 8;  5-6 of B;  7-8 of C
//   9    log10(||A||_F ||B||_F / ||C||_F) / 8, clamped to [-2, 2]
//   10   |i - j| / 32 (tile distance of C in a tile-matrix multiply)
//   11   log10(accuracy) / 8
__global__ void __launch_bounds__(128) features_kernel(const DevUpdate *ups, Workspace ws, double accuracy,
                                                      float *sink) {
    __shared__ double red[4];
    const int s = blockIdx.x;
    const int *meta = ws.meta + (size_t) s * META_INTS;
    const DevUpdate u = ups[s];
    float f[MLP_IN];
    for (int i = 0; i < MLP_IN; i++) f[i] = 0.f;
    if (meta[META_STATUS] == HCGB_OK && meta[META_CKIND]) {
        const int nb = u.c.rows > u.c.cols ? u.c.rows : u.c.cols;
        const TileStats a = tile_stats(u.a, meta[META_RA], red);
        const TileStats b = tile_stats(u.b, meta[META_RB], red);
        const TileStats c = tile_stats(u.c, meta[META_RC], red);
        f[0] = a.dense ? 1.f : (float) a.rank / nb;
        f[1] = b.dense ? 1.f : (float) b.rank / nb;
        f[2] = (float) c.rank / nb;
        f[3] = ratio_feature(a, 1);
        f[4] = ratio_feature(a, 2);
        f[5] = ratio_feature(b, 1);
        f[6] = ratio_feature(b, 2);
        f[7] = ratio_feature(c, 1);
        f[8] = ratio_feature(c, 2);
        const double num = a.fro2 * b.fro2, den = c.fro2;  // squared norms: q = (||A|| ||B|| / ||C||)^2
        const double q = (num > 0.0 ? num : 1e-300) / (den > 0.0 ? den : 1e-300);
        f[9] = clampf((float) (0.5 * log10(q)) / 8.f, -2.f, 2.f);
        f[10] = (float) u.dist / 32.f;
        f[11] = (float) log10(accuracy) / 8.f;
    }
    if (threadIdx.x < MLP_IN) {
        if (ws.feat) ws.feat[(size_t) s * MLP_IN + threadIdx.x] = f[threadIdx.x];
        if (sink) sink[(size_t) u.uid * MLP_IN + threadIdx.x] = f[threadIdx.x];
    }
}

__device__ __forceinline__ GemmJob sk_job(const double *A, int lda, int opA, const double *B, int ldb, double *C,
                                          int ldc, int M, int N, int K, const Params &p) {
    GemmJob j;
    j.A = A;
    j.B = B;
    j.C = C;
    j.M = M;
    j.N = N;
    j.K = K;
    j.lda = lda;
    j.ldb = ldb;
    j.ldc = ldc;
    j.opA = opA;
    j.opB = 0;
    j.alpha = 1.0;
    j.beta = 0.0;
    j.triA = j.triB = 0;
    j.prec = lowp_prec(p.mode);
    j.oz = (!j.prec && p.oz && oz_shape(M, N, K, p.oz_min)) ? 1 : 0;
    return j;
}

// One thread per update: the sketch width and the two jobs of Y = U_s (V_s^T Omega).
__global__ void sketch_plan_kernel(const DevUpdate *ups, int n, Workspace ws, Params p, int policy, GemmJob *jobs) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int *meta = ws.meta + (size_t) s * META_INTS;
    GemmJob none;
    none.M = none.N = none.K = 0;
    none.oz = none.triA = none.triB = none.prec = 0;
    jobs[s] = none;
    jobs[n + s] = none;
    meta[META_LSK] = 0;
    meta[META_SK_ACC] = 0;
    if (meta[META_STATUS] != HCGB_OK || !meta[META_CKIND] || p.fixed_rank > 0) return;
    const int k = meta[META_K], m = meta[META_M], nn = meta[META_N];
    float rhat;
    if (policy == 0) {
        const float y = ws.pred[s];
        rhat = exp2f(fminf(fmaxf(y, 0.f), 12.f)) - 1.f;
    } else {  // without the network: the larger of C's rank and the rank the product adds
        const int ra = meta[META_RA], rb = meta[META_RB], rc = meta[META_RC];
        const int add = (ra && rb) ? (ra < rb ? ra : rb) : (ra ? ra : rb);
        rhat = (float) (rc > add ? rc : add);
    }
    int l = (int) ceilf(rhat) + SK_OVERSAMPLE;
    if (l < 1 + SK_OVERSAMPLE) l = 1 + SK_OVERSAMPLE;
    const int mn = m < nn ? m : nn;
    // not narrow enough to pay for itself (or no smaller than the stacks): the plain recompression
    if (100 * (l + SK_PROBES) > p.sk_pct * k || l > mn) return;
    meta[META_LSK] = l;
    double *base = ws.slot(s);
    const int ld = ws.ld, lk = ws.kmax;
    // Z (k x (l + 4), ld kmax) = V_s^T Omega;  Y (m x (l + 4), ld ld) = U_s Z
    jobs[s] = sk_job(base + ws.off_vstack, ld, 1, base + ws.off_xv, ld, base + ws.off_m, lk, k, l + SK_PROBES, nn, p);
    jobs[n + s] = sk_job(base + ws.off_ustack, ld, 0, base + ws.off_m, lk, base + ws.off_sk1, ld, m, l + SK_PROBES, k,
                         p);
}

// Counter-based normal variates: a 64-bit mix (SplitMix64 finaliser) of (seed, update, index)
// gives two uniforms, Box-Muller gives N(0, 1).
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256) omega_kernel(const DevUpdate *ups, Workspace ws, unsigned long long seed) {
    const int s = blockIdx.x;
    const int *meta = ws.meta + (size_t) s * META_INTS;
    const int l = meta[META_LSK];
    if (!l) return;
    const int nn = meta[META_N], cols = l + SK_PROBES;
    double *O = ws.slot(s) + ws.off_xv;
    const unsigned long long key = mix64(seed ^ mix64((unsigned long long) ups[s].uid));
    for (int e = threadIdx.x; e < nn * cols; e += blockDim.x) {
        const int r = e % nn, c = e / nn;
        const unsigned long long h = mix64(key + (unsigned long long) e);
        const double u1 = ((h >> 11) + 1) * (1.0 / 9007199254740993.0);  // (0, 1]
        const double u2 = (double) (mix64(h) >> 11) * (1.0 / 9007199254740992.0);
        O[r + (size_t) c * ws.ld] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    }
}

// One CTA per sketched update: Householder QR of Y[:, :l] (m rows) in place with the reflectors
// applied to the probe columns too, the residual estimate, then Q_Y formed in place (as LAPACK's
// dorg2r does from the compact form).  FP64; column operations one warp per column.
__global__ void __launch_bounds__(256) sketch_qr_kernel(Workspace ws) {
    extern __shared__ double skq_smem[];
    double *tau = skq_smem;            // kmax
    double *red = tau + ws.kmax;       // 8 warps
    const int s = blockIdx.x;
    const int *meta = ws.meta + (size_t) s * META_INTS;
    const int l = meta[META_LSK];
    if (!l) return;
    const int m = meta[META_M], ld = ws.ld, ncol = l + SK_PROBES;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    double *Y = ws.slot(s) + ws.off_sk1;
    for (int i = 0; i < l; i++) {
        double *yi = Y + (size_t) i * ld;
        double a = 0.0;
        for (int r = i + 1 + threadIdx.x; r < m; r += blockDim.x) a = fma(yi[r], yi[r], a);
        const double sig2 = block_sum(a, red);
        const double alpha = yi[i];
        double t = 0.0, beta = alpha;
        if (sig2 > 0.0) {
            beta = -copysign(sqrt(fma(alpha, alpha, sig2)), alpha);
            t = (beta - alpha) / beta;
            const double sc = 1.0 / (alpha - beta);
            for (int r = i + 1 + threadIdx.x; r < m; r += blockDim.x) yi[r] *= sc;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            yi[i] = beta;
            tau[i] = t;
        }
        __syncthreads();
        if (t != 0.0)
            for (int j = i + 1 + warp; j < ncol; j += nw) {
                double *yj = Y + (size_t) j * ld;
                double w = lane == 0 ? yj[i] : 0.0;
                for (int r = i + 1 + lane; r < m; r += 32) w = fma(yi[r], yj[r], w);
                w = warp_sum(w) * t;
                if (lane == 0) yj[i] -= w;
                for (int r = i + 1 + lane; r < m; r += 32) yj[r] = fma(-w, yi[r], yj[r]);
            }
        __syncthreads();
    }
    // residual estimate from the probe columns (rows l .. m of Q^T P w_p)
    double mx = 0.0;
    for (int p = 0; p < SK_PROBES; p++) {
        const double *yp = Y + (size_t) (l + p) * ld;
        double a = 0.0;
        for (int r = l + threadIdx.x; r < m; r += blockDim.x) a = fma(yp[r], yp[r], a);
        mx = fmax(mx, block_sum(a, red));
    }
    if (threadIdx.x == 0) ws.slot(s)[ws.off_skaux] = 10.0 * sqrt(2.0 / 3.14159265358979323846) * sqrt(mx);
    // Q_Y in place: for i = l-1 .. 0, apply H_i to columns i+1 .. l-1, then column i = H_i e_i.
    for (int i = l - 1; i >= 0; i--) {
        const double *yi = Y + (size_t) i * ld;
        const double t = tau[i];
        if (t != 0.0)
            for (int j = i + 1 + warp; j < l; j += nw) {
                double *yj = Y + (size_t) j * ld;
                double w = 0.0;  // Y[i, j] is zero here
                for (int r = i + 1 + lane; r < m; r += 32) w = fma(yi[r], yj[r], w);
                w = warp_sum(w) * t;
                if (lane == 0) yj[i] = -w;
                for (int r = i + 1 + lane; r < m; r += 32) yj[r] = fma(-w, yi[r], yj[r]);
            }
        __syncthreads();
        double *ci = Y + (size_t) i * ld;
        for (int r = threadIdx.x; r < m; r += blockDim.x) {
            if (r < i) ci[r] = 0.0;
            else if (r == i) ci[r] = 1.0 - t;
            else ci[r] = -t * ci[r];
        }
        __syncthreads();
    }
}

// One thread per sketched update: W = U_s^T Q_Y (k x l, into off_m) and V' = V_s W (n x l, into
// the second sketch stack).
__global__ void sketch_plan2_kernel(int n, Workspace ws, Params p, GemmJob *jobs) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int *meta = ws.meta + (size_t) s * META_INTS;
    GemmJob none;
    none.M = none.N = none.K = 0;
    none.oz = none.triA = none.triB = none.prec = 0;
    jobs[s] = none;
    jobs[n + s] = none;
    const int l = meta[META_LSK];
    if (!l) return;
    const int k = meta[META_K], m = meta[META_M], nn = meta[META_N];
    double *base = ws.slot(s);
    const int ld = ws.ld, lk = ws.kmax;
    jobs[s] = sk_job(base + ws.off_ustack, ld, 1, base + ws.off_sk1, ld, base + ws.off_m, lk, k, l, m, p);
    jobs[n + s] = sk_job(base + ws.off_vstack, ld, 0, base + ws.off_m, lk, base + ws.off_sk2, ld, nn, l, k, p);
}

__global__ void sketch_pass_kernel(int n, Workspace ws, Params p, int stage) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int *meta = ws.meta + (size_t) s * META_INTS;
    const int l = meta[META_LSK];
    if (stage == 0) {
        meta[META_SK_CK] = meta[META_CKIND];
        meta[META_SK_K] = meta[META_K];
        meta[META_SK_ST] = meta[META_STATUS];
        meta[META_SK_ACC] = 0;
        if (l) meta[META_K] = l;
        else meta[META_CKIND] = 0;  // not part of the sketch pass
    } else if (stage == 1) {
        bool acc = false;
        if (l) {
            const double *base = ws.slot(s);
            const double est = base[ws.off_skaux], sig0 = base[ws.off_sigma];
            const double thr = p.truncated ? p.accuracy * sig0 : p.accuracy;
            const int st = meta[META_STATUS];
            acc = (st == HCGB_OK || st == HCGB_NOT_CONVERGED) && est <= thr && meta[META_NEWRANK] < l;
        }
        meta[META_SK_ACC] = acc ? 1 : 0;
        if (acc) {
            meta[META_CKIND] = 0;  // done: the fallback pass skips it
        } else {
            meta[META_CKIND] = meta[META_SK_CK];
            meta[META_K] = meta[META_SK_K];
            meta[META_STATUS] = meta[META_SK_ST];
        }
    } else {
        meta[META_CKIND] = meta[META_SK_CK];
        meta[META_K] = meta[META_SK_K];
    }
}

__global__ void learned_records_kernel(const DevUpdate *ups, int n, Workspace ws, hcgb_update_info *info) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int *meta = ws.meta + (size_t) s * META_INTS;
    const int status = meta[META_STATUS];
    const bool ok = (status == HCGB_OK || status == HCGB_NOT_CONVERGED) && meta[META_CKIND];
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

}  // namespace

void launch_features(const DevUpdate *ups, int n, Workspace ws, double accuracy, float *sink, cudaStream_t st) {
    if (n > 0) { features_kernel<<<n, 128, 0, st>>>(ups, ws, accuracy, sink); note_launch(); }
}

void launch_sketch_plan(const DevUpdate *ups, int n, Workspace ws, Params p, int policy, unsigned long long seed,
                        GemmJob *jobs, cudaStream_t st) {
    if (n <= 0) return;
    { sketch_plan_kernel<<<(n + 127) / 128, 128, 0, st>>>(ups, n, ws, p, policy, jobs); note_launch(); }
    { omega_kernel<<<n, 256, 0, st>>>(ups, ws, seed); note_launch(); }
}

void launch_sketch_qr(int n, Workspace ws, cudaStream_t st) {
    if (n <= 0) return;
    const size_t smem = sizeof(double) * (ws.kmax + 8);
    { sketch_qr_kernel<<<n, 256, smem, st>>>(ws); note_launch(); }
}

void launch_sketch_plan2(int n, Workspace ws, Params p, GemmJob *jobs, cudaStream_t st) {
    if (n > 0) { sketch_plan2_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, ws, p, jobs); note_launch(); }
}

void launch_sketch_pass(int n, Workspace ws, Params p, int stage, cudaStream_t st) {
    if (n > 0) { sketch_pass_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, ws, p, stage); note_launch(); }
}

void launch_learned_records(const DevUpdate *ups, int n, Workspace ws, hcgb_update_info *info, cudaStream_t st) {
    if (n > 0 && info) { learned_records_kernel<<<(n + 127) / 128, 128, 0, st>>>(ups, n, ws, info); note_launch(); }
}

}  // namespace hcgb
