// Internal declarations shared by the CUDA translation units of libhcgb.
//
// Execution model of one batched call (a "wave" of independent tile updates, one
// update per C tile):
//   plan      : read the device-side ranks, choose the stacking side, and resolve
//               every factor product into a GemmJob (no host round trip)
//   stack     : copy/scale/transpose the C factors into the stacked bases
//               U = [Cu | alpha*Ua'] (m x k), V = [beta*Cv^T | Vb'] (n x k)
//   gemm x3   : the factor products, written straight into the stacks (or into a dense C):
//               a schedule kernel compacts the wave's output tiles, then persistent FP64 DMMA
//               (small) and FP64-accurate 16-bit tensor-core (large) product kernels
//   order     : updates sorted by stack width (the heavy stages' CTA order)
//   qr        : blocked Householder QR of both stacks (plain: panel SIMT + trailing DMMA;
//               mixed: float-float on the FP32 pipe)
//   core_svd  : M = R_U R_V^T, pivoted QR, one-sided Jacobi, rank truncation, new factors in
//               the small basis
//   apply_q   : new U = Q_U [U_r; 0], new V = Q_V [XV; 0] (panels, or full WY for wide sides
//               in the plain form)
//   finalize  : transpose V into the tile buffer, publish the new rank
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "hcgb.h"

namespace hcgb {

constexpr int QR_NB = 16;          // Householder panel width (columns)
constexpr int MAX_JACOBI_SWEEPS = 40;

// FP64 tensor-core MMA (the only FP64 tensor path on sm_103a): {d0,d1} += a * b for an
// 8x8x4 tile.  Fragment layout (PTX ISA, mma.m8n8k4 .f64):
//   a : A[lane/4][lane%4]        (8 x 4, row)
//   b : B[lane%4][lane/4]        (4 x 8, col)
//   d : D[lane/4][2*(lane%4)+e]  (8 x 8), e = 0, 1
__device__ __forceinline__ void dmma(double &d0, double &d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

// A set of NTH threads (whole warps) of one CTA that works on one update together: the thread's
// index in the team and the named barrier its members synchronise on (bar.sync id, NTH), so that
// two teams of one CTA never wait for each other.
template <int NTH>
struct Team {
    static constexpr int nth = NTH;
    int tid, bar;
    __device__ __forceinline__ int warp() const { return tid >> 5; }
    __device__ __forceinline__ static constexpr int nw() { return NTH >> 5; }
    __device__ __forceinline__ void sync() const { asm volatile("bar.sync %0, %1;" ::"r"(bar), "n"(NTH) : "memory"); }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// C = alpha * op(A) * op(B) + beta * C  (column-major; op 0 = N, 1 = T).  M <= 0: no job.
struct GemmJob {
    const double *A;
    const double *B;
    double *C;
    int M, N, K;
    int lda, ldb, ldc;
    int opA, opB;
    double alpha, beta;
    int oz;          // 1: computed on the 16-bit tensor cores by error-free splitting (oz_gemm.cu)
    int triA, triB;  // 1: the stored operand is read as unit lower trapezoidal (Householder vectors)
    int prec;        // 0: FP64-accurate (DMMA or oz); 1: TF32, 2: BF16 on tcgen05 (tc_gemm.cu)
};

constexpr int JOBS_PER_UPDATE = 6;  // job slots per update: 3 factor-product phases, 6 for the WY application

// Element (i, k) of op(A) with the job's op / unit-lower view (both GEMM kernels).
__device__ __forceinline__ double job_a(const GemmJob &jb, int i, int k) {
    const int r = jb.opA == 0 ? i : k, c = jb.opA == 0 ? k : i;
    if (jb.triA && r <= c) return r == c ? 1.0 : 0.0;
    return jb.A[r + (size_t) c * jb.lda];
}
__device__ __forceinline__ double job_b(const GemmJob &jb, int k, int j) {
    const int r = jb.opB == 0 ? k : j, c = jb.opB == 0 ? j : k;
    if (jb.triB && r <= c) return r == c ? 1.0 : 0.0;
    return jb.B[r + (size_t) c * jb.ldb];
}

// Precision of the factor products and of the WY Q-application products in arithmetic form `mode`.
__host__ __device__ inline int lowp_prec(int mode) { return mode == HCGB_TF32 ? 1 : (mode == HCGB_BF16 ? 2 : 0); }

// Products worth the split (enough k to amortise the 4 FP64 instructions per output, enough outputs
// for a tile).
constexpr int OZ_MIN_OUTPUTS = 2048;
__host__ __device__ inline bool oz_shape(int M, int N, int K, int min_outputs = OZ_MIN_OUTPUTS) {
    return K >= 16 && M >= 16 && N >= 8 && (long long) M * N >= min_outputs;
}

struct DevTile {
    double *data;  // U (rows x rank, ld rows), or the dense tile
    double *v;     // V region: data + rows * max_rank for a stored tile; the U buffer of the stored tile
                   // when this descriptor is the transpose of a compressed_vt tile (factors swapped)
    int *rank;
    int rows, cols, max_rank, kind;
};

struct DevUpdate {
    DevTile a, b, c;
    int uid;   // index of this update's record in the caller's hcgb_update_info array
    int dist;  // |i - j| of the C tile in a tile-matrix multiply (a feature of the rank predictor)
};

// Per-update bookkeeping written by the plan kernel and read by the later stages.
enum MetaField {
    META_STATUS = 0,
    META_CKIND,      // 1 when C is compressed (recompression needed)
    META_RA,
    META_RB,
    META_RC,
    META_SIDE,       // 0: stack [Cu | alpha Au], 1: stack [Cu | alpha Au (Av Bu)]
    META_K,          // columns of both stacks
    META_M,          // rows of C / of the U stack
    META_N,          // cols of C / rows of the V stack
    META_NEWRANK,
    META_SWEEPS,
    META_CORE_COLS,  // rows of R kept by the rank-revealing QR of the core
    META_KC_PRODUCT,  // core-kernel phase durations in units of 1024 SM cycles (diagnostics)
    META_KC_QRCP,
    META_KC_JACOBI,
    META_KC_FACTORS,
    META_WY,         // bit 0 / bit 1: the U / V factor's Q is applied in WY form (else apply_q_kernel)
    META_LSK,        // learned form: sketch width l (0: this update takes the plain recompression)
    META_SK_CK,      // learned form: CKIND, K and STATUS saved while the sketch / fallback passes run
    META_SK_K,
    META_SK_ST,
    META_SK_ACC,     // learned form: 1 when the sketch result passed the residual test
    META_INTS = 22
};

// Device workspace: n slots of `slot_doubles` doubles plus an int meta block.
struct Workspace {
    double *base;
    int *meta;            // n * META_INTS
    int *order;           // optional (n ints): heavy-stage CTA b works on update order[b]
    size_t slot_doubles;
    int ld;               // leading dimension of every stack / temporary (>= rows, cols)
    int kmax;             // max columns of a stack
    int rmax;             // max rank of an A/B factor
    size_t off_ustack, off_vstack, off_tmp1, off_tmp2, off_tauu, off_tauv, off_tu, off_tv;
    size_t off_m, off_mcopy, off_xv, off_sigma, off_mixed;
    size_t off_w;  // WY application: W_U, W_V (kmax x kmax each), present when built with wy
    size_t off_sk1, off_sk2, off_skaux;  // learned form: sketch stacks (ld x kmax each), residual estimate
    float *feat;   // learned form / feature sink: MLP_IN features per update (n x MLP_IN), or null
    float *pred;   // learned form: predicted log2(1 + rank) per update (n), or null

    __host__ __device__ double *slot(int s) const { return base + slot_doubles * (size_t) s; }
    // Update processed by CTA `b` of the QR / core / Q-application launches: largest first, so the
    // long updates of a launch start at once instead of after the short ones.
    __device__ int heavy(int b) const { return order ? order[b] : b; }
};

// Layout of one workspace slot for stacks of up to `ld` rows and `kmax` columns; factor ranks
// up to `rmax`.  ddc_scratch reserves an ld x ld product for the DDC combination.
Workspace make_workspace_layout(int ld, int kmax, int rmax, bool ddc_scratch, bool wy = false, bool learned = false);

struct Params {
    double accuracy;
    int truncated;
    int fixed_rank;
    int side_mode;   // 0: always the reference's [Cu | alpha Au]; 1: pick the smaller stack
    int mode;        // hcgb_mode: 0 plain FP64; 1 float-float QR / core / Q application; 2 / 3 TF32 / BF16
                     // factor products and Q-application products (QR, core, truncation in FP64)
    int oz;          // 1: large factor products on the 16-bit tensor cores (FP64-accurate splitting)
    int oz_min;      // outputs a product needs to go to the tensor cores (OZ_MIN_OUTPUTS by default)
    int wy_min;      // reflectors a side needs for the WY Q application (WY_MIN_REFLECTORS by default)
    int precond_min; // plain form: Jacobi columns a core needs for the FP32 preconditioning sweeps
    int sk_pct;      // learned form: sketch an update only when its sketch (with probes) is at most
                     // this percentage of its stack width
};

// Default of Params::sk_pct: a sketch of half the stack width halves the QR and Q-application work,
// which pays for the sketch products and its own QR; wider sketches cost more than they save.
constexpr int SKETCH_MAX_PCT = 50;

// Default of Params::precond_min: off.  Measured on the 32 x 32-tile nb = 512 multiply, the FP32
// preconditioning sweeps cut the FP64 sweeps from ~4.7 to ~3 but cost more than they save
// (918-925 ms per multiply from 16, 32 or 64 core columns on, 844 ms off).
constexpr int PRECOND_MIN_COLS = 1 << 30;

// ---- launchers (stream-ordered, asynchronous) ----
void launch_plan(const DevUpdate *ups, int n, double alpha, double beta, Workspace ws, Params p, GemmJob *jobs,
                 cudaStream_t st);
void launch_stack(const DevUpdate *ups, int n, double alpha, double beta, Workspace ws, cudaStream_t st);
// ws.order <- updates sorted by decreasing stack width k (0 for a dense C; ties by index); needs
// ws.order != nullptr.  The key ignores the status, so it cannot change while the heavy stages run.
void launch_order(int n, Workspace ws, cudaStream_t st);
// out[i] = *ptrs[i] (device rank ints gathered for one host read).
void launch_gather_ranks(const int *const *ptrs, int n, int *out, cudaStream_t st);
// Batched products: sched = device scratch of 2 * njobs + 2 ints (tile prefix sums), njobs <= 4096.
// has_lowp: the list may hold TF32 / BF16 jobs (launches the tcgen05 kernel too).
void launch_gemm_jobs(const GemmJob *jobs, int njobs, int *sched, cudaStream_t st, bool has_lowp = false);
void launch_oz_gemm_jobs(const GemmJob *jobs, int njobs, const int *sched, int sms, cudaStream_t st);
void launch_tc_gemm_jobs(const GemmJob *jobs, int njobs, const int *sched, int sms, cudaStream_t st);
// Bounded mbarrier waits of the tcgen05 kernels that gave up (0 unless something else failed).
unsigned int tc_wait_timeouts();
unsigned int oz_wait_timeouts();
constexpr int MAX_JOBS_PER_LAUNCH = 4096;
constexpr int SCHED_INTS_PER_UPDATE = 16;  // >= (3 * 4n + 3) / n: one WY launch schedules 4n jobs, 3 tile lists
// Q application in full WY form (Q = I - V T V^T, T^-1 = striu(V^T V) + diag(1/tau)): jobs for
// the Grams, Y = V^T X and X -= V W, then the triangular solve T^-1 W = Y.  Used for the sides
// with at least WY_MIN_REFLECTORS reflectors (their products run on the tensor cores); the
// others keep the panel-wise apply_q_kernel, which skips the WY sides.  Plain form only: the mixed
// form's float-float panels are faster than either.
constexpr int WY_MIN_REFLECTORS = 48;
void launch_plan_wy(const DevUpdate *ups, int n, Workspace ws, Params p, GemmJob *jobs, cudaStream_t st);
void launch_wy_solve(int n, Workspace ws, cudaStream_t st);
void launch_qr(Workspace ws, int n, bool mixed, cudaStream_t st);
void launch_core_svd(const DevUpdate *ups, int n, Workspace ws, Params p, cudaStream_t st);
void launch_apply_q(const DevUpdate *ups, int n, Workspace ws, bool mixed, cudaStream_t st);
void launch_finalize(const DevUpdate *ups, int n, Workspace ws, hcgb_update_info *info, cudaStream_t st);
// FP64 throughput probes (TFLOP/s): tensor-core DMMA and SIMT DFMA.
int measure_fp64_peak(cudaStream_t st, double *dmma_tflops, double *dfma_tflops);
// DDC (dense A, dense B, compressed C): C <- full rank, U = alpha A B + beta Cu Cv, V = I.
void launch_ddc_finalize(const DevUpdate *ups, int n, Workspace ws, cudaStream_t st);
// dst (cols x rows, ld ldd) = src^T (src rows x cols, ld lds); one CTA.
void launch_transpose(const double *src, int lds, int rows, int cols, double *dst, int ldd, cudaStream_t st);

// Dense tile building blocks of a tile Cholesky (chol.cu).
void launch_trsm_panel(const double *L, int nb, int ldl, const DevTile *tiles, int count, cudaStream_t st);
void launch_fill_triangle(int uplo, int n, double *A, int lda, double value, cudaStream_t st);
void launch_potrf(double *A, int n, int lda, int uplo, int *info_dev, cudaStream_t st);
void launch_trsm(int side, int uplo, int trans, int diag, int m, int n, double alpha, const double *A, int lda,
                 double *B, int ldb, cudaStream_t st);
void launch_syrk(int uplo, int trans, int n, int k, double alpha, const double *A, int lda, double beta, double *C,
                 int ldc, cudaStream_t st);

// Rank-trimmed packing of a tile list (pack.cu): offsets (n + 1) and the packed copy, or back.
void launch_pack(const DevTile *tiles, int n, long long *offsets, double *packed, bool unpack, cudaStream_t st);

// Every kernel launch of the library is counted (hcgb_kernel_launches reads the total).
void note_launch();

// ---- learned form (learned.cu): features, sketch recompression and its fallback ----
// Per-update features (ws.feat, and sink[uid * MLP_IN ..] when sink != null); needs ws.feat.
void launch_features(const DevUpdate *ups, int n, Workspace ws, double accuracy, float *sink, cudaStream_t st);
// Sketch width per update from ws.pred (policy 0) or from the input ranks (policy 1), the jobs
// Z = V_s^T Omega (jobs[0 .. n)) and Y = U_s Z (jobs[n .. 2n)), and Omega itself.
void launch_sketch_plan(const DevUpdate *ups, int n, Workspace ws, Params p, int policy, unsigned long long seed,
                        GemmJob *jobs, cudaStream_t st);
// Householder QR of Y's first l columns, residual probe, explicit Q_Y; then the jobs W = U_s^T Q_Y
// (jobs[0 .. n)) and V' = V_s W (jobs[n .. 2n)).
void launch_sketch_qr(int n, Workspace ws, cudaStream_t st);
void launch_sketch_plan2(int n, Workspace ws, Params p, GemmJob *jobs, cudaStream_t st);
// stage 0: before the sketch pass; 1: residual test, before the fallback pass; 2: restore.
void launch_sketch_pass(int n, Workspace ws, Params p, int stage, cudaStream_t st);
void launch_learned_records(const DevUpdate *ups, int n, Workspace ws, hcgb_update_info *info, cudaStream_t st);

// ---- per-matrix operations of the HCoreKernels backend (backend.cu); asynchronous on st ----
void be_copy(cudaStream_t st, int trans, int m, int n, double alpha, const double *A, int lda, double *B, int ldb);
void be_lacpy(cudaStream_t st, int uplo, int m, int n, const double *A, int lda, double *B, int ldb);
void be_laset(cudaStream_t st, int uplo, int m, int n, double offdiag, double diag, double *A, int lda);
void be_scale_rows(cudaStream_t st, int rows, int cols, const double *s, double *A, int lda);
void be_symmetrize(cudaStream_t st, int uplo, int n, double *A, int lda);
void be_geqr2(cudaStream_t st, int m, int n, double *A, int lda, double *tau);
void be_org2r(cudaStream_t st, int m, int n, int k, double *A, int lda, const double *tau);
void be_orm2r(cudaStream_t st, int left, int trans, int m, int n, int k, const double *A, int lda, const double *tau,
              double *C, int ldc);
void be_trmm(cudaStream_t st, int left, int upper, int trans, int unit, int m, int n, double alpha, const double *A,
             int lda, const double *T, double *B, int ldb);
void be_jacobi_svd(cudaStream_t st, int rows, int cols, double *X, int ldx, double *V, int ldv, double tol, int *sweeps);
void be_svd_finish(cudaStream_t st, int rows, int cols, const double *X, int ldx, const double *V, int ldv, double *S,
                   double *U, int ldu, double *VT, int ldvt, int kk, int want_u, int want_vt, int transposed);

// ---- rank predictor of the learned form (mlp.cu) ----
constexpr int MLP_IN = 12, MLP_HIDDEN = 64;
constexpr int MLP_PARAMS = MLP_HIDDEN * MLP_IN + MLP_HIDDEN + MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN + MLP_HIDDEN + 1;
struct RankModel {
    float *master = nullptr;  // FP32 master parameters, then grad, Adam m1, m2 (4 x MLP_PARAMS floats)
    float *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
    __nv_bfloat16 *w = nullptr;  // BF16 weights read by the forward / backward kernels
    int adam_t = 0;
    int device = 0;
    int init(unsigned long long seed);
    int set_params(const float *host);
    int get_params(float *host) const;
    void release();
};
void launch_mlp_forward(const RankModel &m, const float *X, int n, float *Y, cudaStream_t st);
// grad += dL/dparams of L = inv_total * sum over samples (y - t)^2, *loss += sum (y - t)^2, for the
// samples idx[off .. off + n) (or rows off .. off + n when idx is null).
void launch_mlp_grad(const RankModel &m, const float *X, const float *T, const int *idx, int off, int n,
                     float inv_total, double *loss, cudaStream_t st);
void launch_adam(RankModel &m, float lr, cudaStream_t st);
void launch_targets_from_records(const hcgb_update_info *info, int n, float *T, int *keep, cudaStream_t st);

size_t qr_smem_bytes(int ld, int kmax);
size_t svd_smem_bytes(int kmax);

}  // namespace hcgb
