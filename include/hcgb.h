/*
 * hcgb.h -- C ABI of the GB300-native TLR GEMM (HCore++'s tile GEMM with recompression).
 *
 * The entry points replace, for the TLR GEMM path, what HCore++'s CUDA backend does behind
 * its C++ API.  Every pointer inside a tile is DEVICE memory; descriptor arrays passed to
 * the entry points are HOST memory.  No exception crosses this boundary: every entry
 * point returns an hcgb_status.
 *
 * Tile buffers use HCore++'s own DataHolder layout so that a reference tile buffer can be
 * handed over unchanged:
 *   dense      : rows x cols, column-major, leading dimension = rows
 *                (DenseTile, include/hcorepp/operators/concrete/Dense.hpp:90-91)
 *   compressed : [U: rows x max_rank (ld rows) | V: max_rank x cols (ld = rank)]
 *                (CompressedTile, src/operators/concrete/Compressed.cpp:50-73, :176-185)
 *   compressed_vt (HCore++'s Cholesky-flow reading of the same buffer):
 *                [U: rows x max_rank (ld rows) | W: cols x rank (ld cols)], tile = U W^T.
 *                HCore<T>::Trsm solves on W (src/api/HCore.cpp:636-640), HCore<T>::Syrk forms
 *                U (W^T W) U^T (:512-545), and Gemm's aCholesky branch reads and writes W
 *                (src/api/HCore.cpp:160-174, src/operators/concrete/Compressed.cpp:273-276,
 *                :529-595, :669-673, ProcessVpointer's Cholesky copies omp/kernels.cpp:35-56).
 * A compressed tile's rank lives in a device int so that batched calls never need the host.
 */
#ifndef HCGB_H
#define HCGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    HCGB_OK = 0,
    HCGB_CUDA_ERROR = 1,      /* a CUDA runtime call failed (reference: GPU_ERROR_CHECK -> exit,
                                 include/hcorepp/kernels/cuda/error_checking.h:38-45) */
    HCGB_BAD_ARG = 2,         /* invalid argument (reference: std::invalid_argument / runtime_error) */
    HCGB_POOL_TOO_SMALL = 3,  /* scratch does not fit (reference: pool/MemoryHandler.hpp:52-54) */
    HCGB_RANK_OVERFLOW = 4,   /* a rank exceeds the tile's capacity */
    HCGB_NOT_CONVERGED = 5,   /* the Jacobi SVD hit its sweep limit */
    HCGB_UNSUPPORTED = 6      /* combination not available on this entry point */
} hcgb_status;

typedef enum { HCGB_DENSE = 0, HCGB_COMPRESSED = 1, HCGB_COMPRESSED_VT = 2 } hcgb_tile_kind;
typedef enum { HCGB_NOTRANS = 0, HCGB_TRANS = 1 } hcgb_op;
typedef enum { HCGB_GESVD = 0, HCGB_GESDD = 1 } hcgb_svd_type;

/* One tile in device memory. */
typedef struct {
    double *data;   /* device buffer, layout above */
    int *rank;      /* compressed: device int with the current rank; dense: NULL */
    int rows;
    int cols;
    int max_rank;   /* compressed: capacity of the buffer in columns of U / rows of V */
    int kind;       /* hcgb_tile_kind */
} hcgb_tile;

/* Recompression settings.  Mirrors operators::CompressionParameters
 * (include/hcorepp/operators/helpers/CompressionParameters.hpp:44-46, :116-127).
 * use_trmm / use_ungqr / op_type are accepted for interface parity; the GPU path always
 * forms the same truncated product (QR of both stacks, SVD of the small core, Q applied). */
typedef struct {
    double accuracy;
    int truncated_svd;  /* 1: relative threshold sigma_i < accuracy * sigma_0; 0: absolute */
    int fixed_rank;     /* > 0: fixed-rank truncation */
    int use_trmm;
    int use_ungqr;
    int op_type;        /* hcgb_svd_type */
    int mode;           /* hcgb_mode: arithmetic of the recompression core */
} hcgb_params;

/* HCGB_PLAIN_FP64: the recompression (stack QR, core SVD, Q application) in double precision.
 * HCGB_MIXED: the stack QR, the core SVD's pivoted QR and Jacobi sweeps and the panel-wise Q
 * application in float-float arithmetic (a value is the unevaluated sum of two floats, 48-bit
 * significand) on the FP32 pipe, each block scaled by an exact power of two first; the core
 * product, the new factors, the truncation test and all factor products stay in double precision.
 * Backward error of the float-float stages ~2^-48 relative: same ranks and product accuracy as the
 * plain form at the accuracies this path is used at (>= 1e-12 relative), about 1.6x as fast.
 * In both forms the larger factor products run on the 16-bit tensor cores by FP64-accurate
 * error-free splitting unless hcgb_set_tensor_products(ctx, 0). */
typedef enum { HCGB_PLAIN_FP64 = 0, HCGB_MIXED = 1, HCGB_TF32 = 2, HCGB_BF16 = 3 } hcgb_mode;
/* HCGB_TF32 / HCGB_BF16: the low-precision forms.  Every factor product and the two large products of
 * the Q application (Y = V^T X and X - V W of the compact-WY form, used on every side) run on the
 * fifth-generation tensor cores (tcgen05.mma kind::tf32 / kind::f16 with BF16 operands, FP32
 * accumulation in tensor memory) after per-row / per-column power-of-two scaling of the operands.
 * The Householder QR of the stacks (and its T factor), the core SVD and the truncation test stay in
 * FP64.  The product error is that of TF32 (2^-11) / BF16 (2^-8) operand rounding: these forms do
 * not reach accuracies below ~1e-3 relative; callers read the error and the rank growth off the
 * result. */

/* One tile update C <- alpha * A * B + beta * C (NoTrans operands). */
typedef struct {
    hcgb_tile a;
    hcgb_tile b;
    hcgb_tile c;
} hcgb_update;

/* Per-update record a batched call can return (device array, one entry per update). */
typedef struct {
    int status;     /* hcgb_status of the update */
    int rank_a;     /* input ranks (0 for dense operands) */
    int rank_b;
    int rank_c;
    int k;          /* columns of the stacked bases that were recompressed (0 for a dense C) */
    int new_rank;   /* rank of C after the update (0 for a dense C) */
    int sweeps;     /* Jacobi sweeps the core SVD took */
    int side;       /* 0: stacked [Cu | alpha Au]; 1: stacked [Cu | alpha Au (Av Bu)] */
    int core_cols;  /* rows of R the rank-revealing QR of the core kept (columns Jacobi rotated) */
    int core_kcycles[4]; /* core SVD phases in units of 1024 SM cycles: core product, pivoted QR,
                            Jacobi, new factors (diagnostics) */
    int sketch_cols;     /* learned form: columns of the randomized sketch (0: plain recompression) */
    int sketch_accepted; /* learned form: 1 if the sketch passed its residual test, 0 if the plain
                            recompression ran as the fallback */
} hcgb_update_info;

/* Pipeline stages, for hcgb_profile_read. */
typedef enum {
    HCGB_STAGE_PLAN = 0, HCGB_STAGE_STACK, HCGB_STAGE_GEMM, HCGB_STAGE_QR, HCGB_STAGE_CORE_SVD,
    HCGB_STAGE_APPLY_Q, HCGB_STAGE_FINALIZE, HCGB_STAGE_SKETCH, HCGB_NUM_STAGES
} hcgb_stage;

typedef struct hcgb_context hcgb_context;

/* Context = one device + one stream + a grow-only device workspace.
 * Replaces kernels::RunContext for CUDA (include/hcorepp/kernels/cuda/RunContext.hpp:15-53:
 * GetStream / Sync / RequestWorkBuffer).  stream may be NULL for the legacy default stream. */
int hcgb_context_create(int device, void *stream, hcgb_context **out);
int hcgb_context_destroy(hcgb_context *ctx);
int hcgb_context_set_stream(hcgb_context *ctx, void *stream);
/* kernels::RunContext::Sync (src/kernels/cuda/RunContext.cpp:52-54) */
int hcgb_sync(hcgb_context *ctx);
/* Text of the last error recorded on this context ("" if none). */
const char *hcgb_last_error(hcgb_context *ctx);

/* Device scratch (bytes) one batched call of n updates needs.  Replaces
 * HCore<T>::CalculateMemoryPoolSize / CalculateGemmPoolSize (src/api/HCore.cpp:346-480)
 * and HCoreKernels::CalculateGemmWorkspaceSize (src/kernels/cuda/kernels.cpp:138-265). */
size_t hcgb_workspace_bytes(int n, int max_rows, int max_cols, int max_rank_c, int max_rank_ab);

/* Batched tile updates: every entry updates a DIFFERENT C tile (the updates are independent).
 * Replaces n calls of HCore<T>::Gemm (src/api/HCore.cpp:23-344) with NoTrans operands.
 * Ranks are read and written on the device; nothing is synchronised with the host.
 * info_dev (optional, device, n records) receives a per-update hcgb_update_info.
 * Supported combinations: CCC, DCC, CDC, CCD, DCD, CDD, DDD (DDC: hcgb_tile_gemm).  Any compressed
 * operand may be HCGB_COMPRESSED_VT; a compressed_vt C is written back in that layout. */
int hcgb_gemm_batch(hcgb_context *ctx, double alpha, double beta, int n, const hcgb_update *updates,
                    const hcgb_params *params, hcgb_update_info *info_dev);

/* Tile-matrix multiply C <- alpha * A * B + beta * C over tile grids (all tiles rows x cols equal
 * to nb), following examples/matrix_multiplication/omp_main.cpp:112-124: for every C tile the
 * k-updates run in ascending k, C tiles are independent.  Grids are column-major host arrays of
 * tile descriptors: A is mt x kt, B is kt x nt, C is mt x nt.  beta is applied on every k step,
 * as in the reference driver.  Asynchronous on the context stream.  info_dev (optional, device,
 * mt*nt*kt records) receives the record of update (i, j, k) at index k*mt*nt + i + j*mt. */
int hcgb_tlr_gemm(hcgb_context *ctx, int mt, int nt, int kt, double alpha, const hcgb_tile *a_grid,
                  const hcgb_tile *b_grid, double beta, const hcgb_tile *c_grid, const hcgb_params *params,
                  hcgb_update_info *info_dev);

/* Number of independent C-tile groups hcgb_tlr_gemm runs concurrently (one stream each; default 8;
 * 1 = every k-wave of the whole grid in one stream, the order the reference's driver uses).
 * The results do not depend on it. */
int hcgb_set_concurrency(hcgb_context *ctx, int groups);

/* Order of the k-updates of each C tile in hcgb_tlr_gemm.  0 (default): ascending k, the order of
 * the reference's driver.  1: each C tile's updates sorted by estimated recompression cost, largest
 * first (the sum C + sum_k A_ik B_kj is the same; rounding and truncation happen in another order,
 * within the accuracy bound).  The expensive updates of all tiles then share a few k-waves. */
int hcgb_set_k_order(hcgb_context *ctx, int policy);

/* enable = 1: hcgb_tlr_gemm records every launch of a multiply (all C-tile groups and k-waves) into
 * one CUDA graph and launches the graph; a later call with the same arguments (grids, alpha, beta,
 * params, info_dev) and the same context settings replays it without any per-kernel launch from
 * the host.  The descriptors and the k order are those of the capturing call: with the cost-first
 * k order (hcgb_set_k_order 1) a replay keeps the order computed from the ranks at capture time
 * (the sum is the same in any order).  The workspace must not be reallocated in between (another
 * call needing a larger one forces a new capture).  enable = 0 drops the graph.  Default 0. */
int hcgb_set_graph(hcgb_context *ctx, int enable);

/* Tuning knobs of the batched pipeline (chosen by hcorepp_gb300/autotune.py per tile size and
 * stack-width class; results do not depend on them beyond rounding): a factor product goes to the
 * FP64-accurate tensor-core path when it has at least oz_min_outputs outputs (default 2048, with
 * K >= 16, M >= 16, N >= 8), and in the plain form a side's Q is applied in WY form when it has at
 * least wy_min_reflectors reflectors (default 48). */
int hcgb_set_tuning(hcgb_context *ctx, int oz_min_outputs, int wy_min_reflectors);

/* Plain form: a core SVD with at least min_cols Jacobi columns first runs one-sided Jacobi sweeps in
 * FP32 with the rotations accumulated in float-float (J orthogonal to ~1e-13), then X <- X J in FP64
 * and FP64 sweeps to working precision; smaller cores run FP64 sweeps only.  min_cols = 0 restores
 * the default (off: a value above every core width); same results up to rounding. */
int hcgb_set_precond(hcgb_context *ctx, int min_cols);

/* Learned form: an update is sketched only when its sketch (predicted rank + 8 oversampling + 4
 * probe columns) is at most `percent` of its stack width (1..100; 0 restores the default, 50).  A
 * narrower limit keeps the sketch to the updates where it halves the QR and Q-application work; 100
 * sketches every update whose sketch is narrower than its stacks. */
int hcgb_set_sketch_limit(hcgb_context *ctx, int percent);

/* Factor products of k >= 16 with at least 2048 outputs run on the 16-bit tensor cores by
 * error-free splitting (each FP64 operand cut into eight 7-bit integer digit planes relative to its
 * row / column maximum, plane products accumulated exactly in FP32 and combined in FP64; result
 * error below 2^-44 max|A_i| max|B_j|, the order of an FP64 product's worst-case bound).
 * enable = 0 keeps every product on the FP64 DMMA path.  Default 1.  Schedule-independent. */
int hcgb_set_tensor_products(hcgb_context *ctx, int enable);

/* Single tile update, the drop-in for HCore<T>::Gemm (src/api/HCore.cpp:23-344).  op_a/op_b
 * accept HCGB_NOTRANS and HCGB_TRANS.  Synchronous: on return *c's rank on the device has been
 * updated; *new_rank (if not NULL) receives it on the host, like CompressedTile::Gemm updating
 * mRank (src/operators/concrete/Compressed.cpp:656-662).  The DDC combination rewrites C at full
 * rank with an identity V (HCore.cpp:272-299) and needs max_rank >= min(rows, cols).
 * HCore<T>::Gemm(..., aCholesky = true) is this call with A, B and C given as HCGB_COMPRESSED_VT
 * and op_b = HCGB_TRANS (the one combination the reference's Cholesky branch handles).
 * flops (if not NULL) is incremented by the reference's count for the update. */
int hcgb_tile_gemm(hcgb_context *ctx, double alpha, const hcgb_tile *a, int op_a, const hcgb_tile *b, int op_b,
                   double beta, hcgb_tile *c, const hcgb_params *params, int *new_rank,
                   unsigned long long *flops);

/* Dense -> compressed tile construction, the GPU form of CompressedTile(rows, cols, data, ld, params,
 * ...) (src/operators/concrete/Compressed.cpp:75-146): truncated SVD of the dense tile `dense`
 * (device, rows x cols, ld rows) by the same QR + core-SVD route as a tile update, rank by the
 * params' rule clamped to [1, out->max_rank].  `out` is a compressed tile of the same shape whose
 * buffer and device rank the call fills (the reference clamps at max(min(rows, cols)/3, 1)).
 * Synchronous; *rank (if not NULL) receives the rank. */
int hcgb_compress_tile(hcgb_context *ctx, const double *dense, int rows, int cols, hcgb_tile *out,
                       const hcgb_params *params, int *rank);

/* Batched form of hcgb_compress_tile: `count` dense tiles dense[i] (host array of device pointers,
 * each rows x cols, ld rows) compressed into out[i] (host array of compressed tile descriptors of
 * that shape) by one batched pipeline launch per chunk of tiles instead of one call per tile (the
 * reference constructs its input tiles one by one, Compressed.cpp:75-146, TileMatrix.cpp:17-185).
 * Same arithmetic and rank rule per tile as hcgb_compress_tile.  The chunk is sized so that the
 * workspace stays within half of the device's free memory.  Synchronous; ranks (host array of
 * `count`, or NULL) receives the ranks.  Returns HCGB_NOT_CONVERGED if any tile's core did not
 * converge (the tiles are still written). */
int hcgb_compress_tiles(hcgb_context *ctx, int count, const double *const *dense, int rows, int cols,
                        hcgb_tile *out, const hcgb_params *params, int *ranks);

/* ---- Dense per-tile building blocks of a tile Cholesky (device pointers, column-major) ---- */
typedef enum { HCGB_LOWER = 0, HCGB_UPPER = 1 } hcgb_uplo;
typedef enum { HCGB_LEFT = 0, HCGB_RIGHT = 1 } hcgb_side;
typedef enum { HCGB_NONUNIT = 0, HCGB_UNIT = 1 } hcgb_diag;

/* Cholesky factorisation of the uplo triangle of A (n x n, ld lda), LAPACK dpotrf semantics;
 * replaces HCoreKernels::potrf (src/kernels/cuda/CudaKernels.cu:1019-1049, omp/kernels.cpp:234-243).
 * Synchronous; *info (if not NULL) receives 0 or the order of the first non-positive minor. */
int hcgb_potrf(hcgb_context *ctx, int uplo, int n, double *A, int lda, int *info);
/* op(A) X = alpha B (HCGB_LEFT) or X op(A) = alpha B (HCGB_RIGHT), X overwriting B (m x n);
 * BLAS dtrsm semantics; replaces HCoreKernels::trsm (src/kernels/cuda/kernels.cpp:290-298).
 * trans: HCGB_NOTRANS / HCGB_TRANS.  Asynchronous. */
int hcgb_trsm(hcgb_context *ctx, int side, int uplo, int trans, int diag, int m, int n, double alpha,
              const double *A, int lda, double *B, int ldb);
/* C = alpha op(A) op(A)^T + beta C on the uplo triangle (C n x n, op(A) n x k); BLAS dsyrk
 * semantics; replaces HCoreKernels::syrk (src/kernels/cuda/kernels.cpp:299-306).  Asynchronous. */
int hcgb_syrk(hcgb_context *ctx, int uplo, int trans, int n, int k, double alpha, const double *A, int lda,
              double beta, double *C, int ldc);
/* Tile Cholesky A = L L^T of an nt x nt tile matrix (grid: nt*nt descriptors, column-major; only
 * i >= j is read): nb x nb tiles, dense on the diagonal, HCGB_COMPRESSED_VT below it (tile = U W^T).
 * The reference provides the per-tile operations but no driver; this composes them right-looking:
 * for each k, Potrf(A_kk) (src/api/HCore.cpp:585-621), the panel Trsm W_ik <- L_kk^-1 W_ik
 * (:623-647) in one launch, and every trailing update A_ij -= A_ik A_jk^T, j <= i -- Syrk on the
 * diagonal (:482-583), Gemm(aCholesky) below (:23-344) -- batched into pipeline launches of up to
 * 1024 updates.  Synchronous (one host wait per step, on the potrf info).  *info (if not NULL)
 * receives 0 or k * nb + the potrf info of the first failing diagonal tile.  info_dev (optional)
 * receives one hcgb_update_info per trailing update, in step order (k ascending; within a step
 * i ascending, then j = k+1 .. i). */
int hcgb_tile_cholesky(hcgb_context *ctx, int nt, const hcgb_tile *grid, const hcgb_params *params, int *info,
                       hcgb_update_info *info_dev);

/* Sets the strict uplo triangle of A (n x n, ld lda) to value; replaces
 * HCoreKernels::FillMatrixTriangle (src/kernels/omp/kernels.cpp:246-264), which HCore<T>::Syrk
 * applies after a compressed-A update (src/api/HCore.cpp:555-563).  Asynchronous. */
int hcgb_fill_triangle(hcgb_context *ctx, int uplo, int n, double *A, int lda, double value);

/* Rank-trimmed transfer packing of `count` tiles (the batched device side of TilePacker,
 * include/hcorepp/operators/interface/TilePacker.hpp:18-62, whose PackTile / UnPackTile move one
 * tile at its full capacity): each tile's used part -- dense: rows x cols; compressed: U (rows x
 * rank) then V (rank x cols); compressed_vt: U then W = V^T (cols x rank) -- concatenated in list
 * order into the device buffer `packed_dev`.  offsets_dev (device, count + 1 long long) receives
 * each tile's start (in doubles) and, last, the total, computed on the device from the tiles'
 * device ranks, so a caller reads the total (8 bytes) before copying the packed data out.
 * packed_dev must hold the total; the sum of the tiles' capacities always suffices.
 * hcgb_unpack_tiles is the inverse: the ranks must already be in the tiles' rank ints.
 * Asynchronous on the context stream. */
int hcgb_pack_tiles(hcgb_context *ctx, int count, const hcgb_tile *tiles, double *packed_dev,
                    long long *offsets_dev);
int hcgb_unpack_tiles(hcgb_context *ctx, int count, const hcgb_tile *tiles, const double *packed_dev,
                      long long *offsets_dev);

/* Stage timing with CUDA events on the context stream (the GB300 replacement of the reference's
 * DebuggingTimer snapshots, src/helpers/debugging-timer/ActiveTimer.cpp:47-60).  While enabled,
 * every pipeline stage is bracketed by events; hcgb_profile_read synchronises the stream and
 * returns the accumulated milliseconds and kernel launches per stage since the last reset. */
int hcgb_profile_enable(hcgb_context *ctx, int enable);
int hcgb_profile_reset(hcgb_context *ctx);
int hcgb_profile_read(hcgb_context *ctx, double *ms_per_stage, long long *launches_per_stage, int nstages);

/* Number of kernels this library has launched in this process so far (all devices, all
 * contexts).  The difference across a region counts the library's launches in it. */
long long hcgb_kernel_launches(void);

/* Measures this device's FP64 throughput with two probe kernels (~0.1 s): the FP64 tensor-core
 * MMA (DMMA) rate and the FP64 FMA rate of the SIMT pipes, in TFLOP/s.  These are the roofline
 * denominators of the FP64 path. */
int hcgb_fp64_peak(hcgb_context *ctx, double *dmma_tflops, double *dfma_tflops);

/* ---- The learned form (no counterpart in the reference) ----
 * A rank predictor sizes a randomized sketch of each update's product P = U_s V_s^T (the stacked
 * bases of the plain recompression): l = predicted rank + 8 columns of seeded Gaussian test vectors,
 * Y = P Omega, Q_Y from a Householder QR of Y, and the plain recompression (stack QR, core SVD,
 * truncation by the reference's rule, Q application) run on the l-column stacks [Q_Y], [V_s U_s^T Q_Y].
 * Four more Gaussian probe vectors w_p give the a-posteriori estimate
 * e = 10 sqrt(2/pi) max_p ||(I - Q_Y Q_Y^T) P w_p|| of ||(I - Q_Y Q_Y^T) P||_2 (Halko, Martinsson and
 * Tropp 2011, 4.3; wrong with probability below 1e-4).  The sketch result is kept when e is below the
 * truncation threshold (accuracy * sigma_0, or accuracy) and the new rank is below l; otherwise the
 * plain recompression runs on the original stacks (the fallback), in the same call.  Updates whose
 * stacks are not wider than l + 4 columns, and fixed-rank truncations, take the plain recompression.
 * Every batched entry point of the context (hcgb_gemm_batch, hcgb_tlr_gemm, hcgb_tile_cholesky) uses
 * the form while it is set; the per-update records report sketch_cols and sketch_accepted.
 *
 * The predictor: an MLP with 12 inputs, two hidden layers of 64 (GELU) and one output, BF16 weights,
 * FP32 accumulation; y = predicted log2(1 + rank).  Inputs per update (HCGB_RANK_FEATURES floats):
 * ranks of A, B, C / rows of C (dense operands count as full rank); log10(sigma_1 / sigma_0) and
 * log10(sigma_2 / sigma_0) of A, B and C, each / 8 (a compressed tile's singular values taken as the
 * row norms of its V factor); log10(||A||_F ||B||_F / ||C||_F) / 8; |i - j| / 32 of the C tile;
 * log10(accuracy) / 8.  Trained by the library's own kernels (forward, backward, Adam on an FP32
 * master copy) with mean squared error on log2(1 + rank). */
#define HCGB_RANK_FEATURES 12
#define HCGB_RANK_MODEL_PARAMS 5057
typedef struct hcgb_rank_model hcgb_rank_model;

/* Device-resident predictor, Glorot-initialised from `seed`, on the context's device. */
int hcgb_rank_model_create(hcgb_context *ctx, unsigned long long seed, hcgb_rank_model **out);
int hcgb_rank_model_destroy(hcgb_rank_model *m);
/* Parameters as HCGB_RANK_MODEL_PARAMS floats (W1 64x12 row-major, b1, W2 64x64 row-major, b2, w3,
 * b3): host_in (if not NULL) replaces them (the BF16 weights are rounded from it), then host_out (if not
 * NULL) receives the FP32 master copy.  Synchronous. */
int hcgb_rank_model_params(hcgb_rank_model *m, float *host_out, const float *host_in);
/* out_dev[i] = predicted log2(1 + rank) for the features of row i (device, n x HCGB_RANK_FEATURES). */
int hcgb_rank_model_predict(hcgb_context *ctx, hcgb_rank_model *m, int n, const float *features_dev, float *out_dev);
/* Gradient of (1/n) sum_i (y_i - t_i)^2 with respect to the parameters (host, HCGB_RANK_MODEL_PARAMS
 * floats) and that loss.  Synchronous. */
int hcgb_rank_model_gradient(hcgb_context *ctx, hcgb_rank_model *m, int n, const float *features_dev,
                             const float *targets_dev, float *grad_host, double *loss);
/* Trains on the (features, records) pairs of n updates -- features as recorded by
 * hcgb_set_feature_sink, records the hcgb_update_info of the same updates -- with targets
 * log2(1 + new_rank) of every recompressed update (k > 0, status OK or NOT_CONVERGED): `epochs`
 * passes over a seeded shuffle, minibatches of `batch`, Adam with step `lr`.  *final_loss receives
 * the last epoch's mean squared error, *samples the number of pairs used.  Synchronous. */
int hcgb_rank_model_train(hcgb_context *ctx, hcgb_rank_model *m, int n, const float *features_dev,
                          const hcgb_update_info *records_dev, int epochs, int batch, float lr,
                          unsigned long long seed, double *final_loss, int *samples);
/* Turns the learned form on for this context: policy 0 sizes the sketch by the predictor m; policy 1
 * (m may be NULL) sizes it without a network, from the input ranks (max(rank C, the rank the product
 * adds)).  m = NULL with policy 0 turns the form off. */
int hcgb_set_rank_model(hcgb_context *ctx, hcgb_rank_model *m, int policy);
/* While set, every batched call records each recompressed update's predictor features at
 * features_dev[record index * HCGB_RANK_FEATURES] (the record index of info_dev); NULL stops it. */
int hcgb_set_feature_sink(hcgb_context *ctx, float *features_dev);

/* ---- Per-matrix operations (the HCoreKernels<double> backend, hcorepp_gb300/backend) ----
 * The operations HCore++'s CompressedTile<T>::Gemm and its tests call one matrix at a time through
 * HCoreKernels<T> (include/hcorepp/kernels/kernels.hpp:24-137), for a build of the reference on this
 * library.  Column-major device matrices; asynchronous on the context stream unless stated. */
typedef enum { HCGB_PART_GENERAL = 0, HCGB_PART_UPPER = 1, HCGB_PART_LOWER = 2, HCGB_PART_DIAGONAL = 3 } hcgb_part;
typedef enum { HCGB_SVD_NONE = 0, HCGB_SVD_SOME = 1, HCGB_SVD_ALL = 2 } hcgb_svd_job;
/* C = alpha op(A) op(B) + beta C (trans 0 / 1); HCoreKernels::Gemm (src/kernels/cuda/kernels.cpp:18-24). */
int hcgb_dgemm(hcgb_context *ctx, int transa, int transb, int m, int n, int k, double alpha, const double *A, int lda,
               const double *B, int ldb, double beta, double *C, int ldc);
/* B (m x n) = alpha op(A): the copies and transpositions of MultiplyByAlpha, ProcessVpointer,
 * CalculateUVptr and transpose (src/kernels/omp/kernels.cpp:22-79, :106-114). */
int hcgb_dcopy2d(hcgb_context *ctx, int trans, int m, int n, double alpha, const double *A, int lda, double *B,
                 int ldb);
/* LAPACK dlacpy / dlaset (part: general, upper, lower; dlaset also HCGB_PART_DIAGONAL = only the
 * diagonal, FillIdentityMatrix); HCoreKernels::LaCpy / Laset (omp/kernels.cpp:152-177). */
int hcgb_dlacpy(hcgb_context *ctx, int part, int m, int n, const double *A, int lda, double *B, int ldb);
int hcgb_dlaset(hcgb_context *ctx, int part, int m, int n, double offdiag, double diag, double *A, int lda);
/* Row i < rows of A scaled by s[i] (device): CalculateVTnew (omp/kernels.cpp:116-130). */
int hcgb_dscale_rows(hcgb_context *ctx, int rows, int cols, const double *s, double *A, int lda);
/* The uplo triangle of A copied onto the other one: HCoreKernels::Symmetrize. */
int hcgb_dsymmetrize(hcgb_context *ctx, int uplo, int n, double *A, int lda);
/* Householder QR in LAPACK's compact form (dgeqrf semantics), its Q (dorgqr) and applying it (dormqr,
 * side HCGB_LEFT / HCGB_RIGHT, trans HCGB_NOTRANS / HCGB_TRANS): HCoreKernels::Geqrf, ungqr, Unmqr. */
int hcgb_dgeqrf(hcgb_context *ctx, int m, int n, double *A, int lda, double *tau);
int hcgb_dorgqr(hcgb_context *ctx, int m, int n, int k, double *A, int lda, const double *tau);
int hcgb_dormqr(hcgb_context *ctx, int side, int trans, int m, int n, int k, const double *A, int lda,
                const double *tau, double *C, int ldc);
/* B = alpha op(A) B (left) or alpha B op(A) (right), A triangular (BLAS dtrmm): HCoreKernels::Trmm. */
int hcgb_dtrmm(hcgb_context *ctx, int side, int uplo, int trans, int diag, int m, int n, double alpha,
               const double *A, int lda, double *B, int ldb);
/* SVD of A (m x n, destroyed) by one-sided Jacobi in FP64: S (min(m, n), descending), U (m x min,
 * jobu SOME; ALL only when m <= n), VT (min x n, jobvt SOME; ALL only when n <= m); min(m, n) <=
 * 1024.  HCoreKernels::SVD (gesvd / gesdd, omp/kernels.cpp:182-192).  Synchronous; *info = 1 and
 * HCGB_NOT_CONVERGED if the sweep limit was reached. */
int hcgb_dgesvd(hcgb_context *ctx, int jobu, int jobvt, int m, int n, double *A, int lda, double *S, double *U,
                int ldu, double *VT, int ldvt, int *info);

/* One tile update that allocates nothing (no counterpart in the reference; an addition of this
 * library).  For callers that may not allocate device memory themselves: task-runtime workers whose
 * runtime owns the device memory and places the tile buffers, and real-time or embedded callers
 * that forbid allocation after start-up.  Same arithmetic as hcgb_tile_gemm with NoTrans
 * operands (combinations CCC, DCC, CDC, CCD, DCD, CDD, DDD), but asynchronous on `stream` (NULL =
 * legacy default stream of the current device), no context, no host synchronisation: the new
 * rank is written to c->rank on the device, and info_dev (optional, one device record) receives
 * the update's hcgb_update_info.
 * Scratch: a fixed 8 MiB array inside the library, one per GPU that loads it, held until the
 * process exits.  Updates whose scratch layout does not fit are rejected with
 * HCGB_POOL_TOO_SMALL (tiles up to 512 x 512 with capacities max_rank <= 170 fit).  All calls on a
 * device share the array: calls that overlap on the GPU race, so order them.  The first call on
 * each device looks up the array's device address (with that device current); make it before any
 * stream capture begins.  The address is kept for the life of the process: a device reset
 * (cudaDeviceReset) after that first call is not supported. */
int hcgb_tile_gemm_noalloc(double alpha, const hcgb_tile *a, const hcgb_tile *b, double beta, hcgb_tile *c,
                           const hcgb_params *params, void *stream, hcgb_update_info *info_dev);

#ifdef __cplusplus
}
#endif

#endif /* HCGB_H */
