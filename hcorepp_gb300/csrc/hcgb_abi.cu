// C ABI of libhcgb (declared in include/hcgb.h): contexts, workspace sizing, the batched /
// tile-matrix / single-tile GEMM entry points, dense->compressed construction, the tile Cholesky
// building blocks and driver, and rank-trimmed tile packing.  Host code only; the kernels live in
// tlr_plan.cu, oz_gemm.cu, tlr_qr.cu, tlr_svd.cu, chol.cu, pack.cu and noalloc.cu.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.cuh"

using namespace hcgb;

namespace hcgb {
static std::atomic<long long> g_kernel_launches{0};
void note_launch() { g_kernel_launches.fetch_add(1, std::memory_order_relaxed); }
static void note_launches(long long n) { g_kernel_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace hcgb

extern "C" long long hcgb_kernel_launches(void) { return g_kernel_launches.load(std::memory_order_relaxed); }

struct hcgb_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    void *ws = nullptr;          // workspace slots + meta
    size_t ws_bytes = 0;
    void *desc = nullptr;        // DevUpdate[] followed by GemmJob[3 * n]
    size_t desc_bytes = 0;
    void *stage = nullptr;       // pinned host staging for descriptors
    size_t stage_bytes = 0;
    cudaEvent_t stage_done = nullptr;
    std::string last_error;
    // stage profiling
    bool prof = false;
    std::vector<cudaEvent_t> ev_free;
    // one list of (stage, event) marks per pipeline; the time to the next mark belongs to the stage
    std::vector<std::vector<std::pair<int, cudaEvent_t>>> ev_pending;
    double stage_ms[HCGB_NUM_STAGES] = {0};
    long long stage_launches[HCGB_NUM_STAGES] = {0};
    // independent C-tile groups of hcgb_tlr_gemm, one stream each
    int groups = 8;
    int k_order = 0;  // 0: ascending k per C tile (reference order); 1: estimated cost, largest first
    int oz = 1;       // large factor products on the 16-bit tensor cores (FP64-accurate splitting)
    int oz_min = OZ_MIN_OUTPUTS;     // tuning: outputs a product needs for the tensor cores
    int wy_min = WY_MIN_REFLECTORS;  // tuning: reflectors a side needs for the WY Q application
    int precond_min = PRECOND_MIN_COLS;  // tuning: core columns for the plain form's FP32 preconditioning
    int sk_pct = SKETCH_MAX_PCT;         // learned form: widest sketch, in percent of the stack width
    std::vector<cudaStream_t> group_streams;
    std::vector<cudaEvent_t> group_events;  // [0] fork, [1..] joins
    void *pack_desc = nullptr;  // DevTile[] of hcgb_pack_tiles / hcgb_unpack_tiles
    size_t pack_desc_bytes = 0;
    hcgb_update_info *tile_info = nullptr;  // the one record hcgb_tile_gemm reads back (allocated once)
    // learned form
    bool learned = false;                     // the learned form is on
    struct hcgb_rank_model *model = nullptr;  // rank predictor (policy 0)
    int sk_policy = 0;                        // 0: sketch width from the predictor; 1: from the input ranks
    unsigned long long sk_seed = 0x5eedULL;   // seed of the Gaussian test matrices
    float *feature_sink = nullptr;            // device: per-update predictor features, indexed like info
    // per-matrix operations (hcgb_d*)
    void *be_scratch = nullptr;
    size_t be_scratch_bytes = 0;
    // CUDA graph of the last hcgb_tlr_gemm (hcgb_set_graph)
    bool graph_mode = false;
    cudaGraphExec_t graph_exec = nullptr;
    std::string graph_key;      // the call's arguments and the context settings it was captured with
    void *graph_desc = nullptr;  // descriptors the graph reads (its own buffer: other calls reuse desc)
    size_t graph_desc_bytes = 0;
    void *graph_ws = nullptr;    // workspace the graph was captured on
    long long graph_launches = 0;
    cudaStream_t capture_stream = nullptr;  // captures run here when the context stream is the legacy one
};

struct hcgb_rank_model {
    hcgb::RankModel m;
};

namespace {

int fail(hcgb_context *ctx, int code, const std::string &msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

#define HCGB_CUDA(ctx, call)                                                                       \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail((ctx), HCGB_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int ensure_device(hcgb_context *ctx, void **buf, size_t *have, size_t want) {
    if (*have >= want) return HCGB_OK;
    if (*buf) {
        HCGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        HCGB_CUDA(ctx, cudaFree(*buf));
        *buf = nullptr;
        *have = 0;
    }
    size_t sz = want + want / 8;
    HCGB_CUDA(ctx, cudaMalloc(buf, sz));
    *have = sz;
    return HCGB_OK;
}

int ensure_stage(hcgb_context *ctx, size_t want) {
    // The previous descriptor upload must have left the staging buffer before it is reused.
    HCGB_CUDA(ctx, cudaEventSynchronize(ctx->stage_done));
    if (ctx->stage_bytes >= want) return HCGB_OK;
    if (ctx->stage) HCGB_CUDA(ctx, cudaFreeHost(ctx->stage));
    ctx->stage = nullptr;
    size_t sz = want + want / 8;
    HCGB_CUDA(ctx, cudaMallocHost(&ctx->stage, sz));
    ctx->stage_bytes = sz;
    return HCGB_OK;
}

bool compressed(int kind) { return kind == HCGB_COMPRESSED || kind == HCGB_COMPRESSED_VT; }

DevTile to_dev(const hcgb_tile &t) {
    DevTile d;
    d.data = t.data;
    d.rank = t.rank;
    d.rows = t.rows;
    d.cols = t.cols;
    d.max_rank = compressed(t.kind) ? t.max_rank : 0;
    d.kind = compressed(t.kind) ? t.kind : 0;
    d.v = compressed(t.kind) ? t.data + (size_t) t.rows * t.max_rank : nullptr;
    return d;
}

int check_tile(hcgb_context *ctx, const hcgb_tile &t, const char *name) {
    if (!t.data || t.rows <= 0 || t.cols <= 0)
        return fail(ctx, HCGB_BAD_ARG, std::string(name) + ": null buffer or empty shape");
    if (compressed(t.kind) && (!t.rank || t.max_rank <= 0))
        return fail(ctx, HCGB_BAD_ARG, std::string(name) + ": compressed tile without rank or capacity");
    if (t.kind != HCGB_DENSE && !compressed(t.kind))
        return fail(ctx, HCGB_BAD_ARG, std::string(name) + ": unknown tile kind");
    return HCGB_OK;
}

// Shapes that size the workspace and the GEMM grids of a batch (host-side maxima from the
// tile kinds and capacities; the actual ranks are only known on the device).
struct BatchShape {
    int ld = 8, kmax = 8, rmax = 8;
    int p_m[3] = {0, 0, 0}, p_n[3] = {0, 0, 0};
    bool any_compressed_c = false;
};

BatchShape shape_of(const hcgb_update *ups, int n) {
    BatchShape s;
    for (int i = 0; i < n; i++) {
        const hcgb_update &u = ups[i];
        const bool ak = compressed(u.a.kind), bk = compressed(u.b.kind),
                   ck = compressed(u.c.kind);
        const int m = u.c.rows, nn = u.c.cols;
        const int ra = ak ? u.a.max_rank : 0, rb = bk ? u.b.max_rank : 0, rc = ck ? u.c.max_rank : 0;
        s.ld = std::max({s.ld, m, nn, u.a.cols});
        s.rmax = std::max({s.rmax, ra, rb});
        auto grow = [&](int ph, int M, int N) {
            s.p_m[ph] = std::max(s.p_m[ph], M);
            s.p_n[ph] = std::max(s.p_n[ph], N);
        };
        if (ck) {
            s.any_compressed_c = true;
            if (ak && bk) {
                s.kmax = std::max(s.kmax, rc + std::max(ra, rb));
                grow(0, ra, rb);
                grow(1, std::max(m, nn), std::max(ra, rb));
            } else if (!ak && bk) {
                s.kmax = std::max(s.kmax, rc + rb);
                grow(0, m, rb);
            } else if (ak && !bk) {
                s.kmax = std::max(s.kmax, rc + ra);
                grow(0, nn, ra);
            }
        } else {
            if (ak && bk) {
                grow(0, ra, rb);
                grow(1, std::max(ra, m), std::max(nn, rb));
            } else if (!ak && bk) {
                grow(0, m, rb);
            } else if (ak && !bk) {
                grow(0, ra, nn);
            }
            grow(2, m, nn);
        }
    }
    s.ld = (s.ld + 7) / 8 * 8;
    return s;
}

size_t workspace_bytes_for(const Workspace &w, int n, bool features = false) {
    size_t b = sizeof(double) * w.slot_doubles * (size_t) n + sizeof(int) * (META_INTS + 1) * (size_t) n + 256;
    if (features) b += sizeof(float) * (MLP_IN + 1) * (size_t) n + 256;
    return b;
}

Params to_params(const hcgb_params *p, const hcgb_context *ctx) {
    Params q;
    q.oz = ctx ? ctx->oz : 1;
    q.oz_min = ctx ? ctx->oz_min : OZ_MIN_OUTPUTS;
    q.wy_min = ctx ? ctx->wy_min : WY_MIN_REFLECTORS;
    q.precond_min = ctx ? ctx->precond_min : PRECOND_MIN_COLS;
    q.sk_pct = ctx ? ctx->sk_pct : SKETCH_MAX_PCT;
    q.accuracy = p ? p->accuracy : 1e-9;
    q.truncated = p ? p->truncated_svd : 0;
    q.fixed_rank = p ? p->fixed_rank : 0;
    q.side_mode = 1;
    q.mode = p ? p->mode : 0;
    return q;
}

cudaEvent_t take_event(hcgb_context *ctx) {
    cudaEvent_t e;
    if (!ctx->ev_free.empty()) {
        e = ctx->ev_free.back();
        ctx->ev_free.pop_back();
    } else {
        cudaEventCreate(&e);
    }
    return e;
}

// Launch the full pipeline for n updates whose descriptors are already on the device.
void launch_pipeline(hcgb_context *ctx, cudaStream_t st, const DevUpdate *dups, GemmJob *djobs, int *sched, int n,
                     double alpha,
                     double beta, const Workspace &ws, const BatchShape &sh, const Params &p,
                     hcgb_update_info *info) {
    std::vector<std::pair<int, cudaEvent_t>> ev;
    auto mark = [&](int stage) {
        if (!ctx->prof) return;
        cudaEvent_t e = take_event(ctx);
        cudaEventRecord(e, st);
        ev.push_back({stage, e});
    };
    long long *cnt = ctx->stage_launches;
    const bool lowp = lowp_prec(p.mode) != 0;
    mark(HCGB_STAGE_PLAN);
    launch_plan(dups, n, alpha, beta, ws, p, djobs, st);
    cnt[HCGB_STAGE_PLAN]++;
    mark(HCGB_STAGE_STACK);
    if (sh.any_compressed_c) {
        launch_stack(dups, n, alpha, beta, ws, st);
        cnt[HCGB_STAGE_STACK]++;
    }
    mark(HCGB_STAGE_GEMM);
    for (int ph = 0; ph < 3; ph++)
        if (sh.p_m[ph] > 0 && sh.p_n[ph] > 0) {
            launch_gemm_jobs(djobs + (size_t) ph * n, n, sched, st, lowp);
            cnt[HCGB_STAGE_GEMM]++;
        }
    // Stack QR, core SVD, Q application and write-back of every update whose meta marks a compressed
    // C, on the stacks of w.
    auto recompress = [&](const Workspace &w, hcgb_update_info *inf) {
        mark(HCGB_STAGE_QR);
        // The heavy stages index updates through w.order: it must be written for every launch
        // that carries it (a single update included).
        if (w.order) launch_order(n, w, st);
        launch_qr(w, n, p.mode == 1, st);
        cnt[HCGB_STAGE_QR]++;
        mark(HCGB_STAGE_CORE_SVD);
        launch_core_svd(dups, n, w, p, st);
        cnt[HCGB_STAGE_CORE_SVD]++;
        mark(HCGB_STAGE_APPLY_Q);
        // WY form: the plain form with the tensor-core products (sides >= WY_MIN_REFLECTORS), and every
        // side in the low-precision forms; the mixed form's float-float panels are faster than either.
        if (((p.oz && p.mode == HCGB_PLAIN_FP64) || lowp) && w.off_w) {
            // Sides in full WY form: the Grams, Y = V^T X and X -= V W are products (tensor-core
            // eligible), only the small triangular solve stays on the FP64 pipe.  The others keep the
            // panel-wise kernel.
            launch_plan_wy(dups, n, w, p, djobs, st);
            launch_gemm_jobs(djobs, 4 * n, sched, st, lowp);  // Grams and Y = V^T X (independent)
            launch_wy_solve(n, w, st);
            launch_gemm_jobs(djobs + 4 * (size_t) n, 2 * n, sched, st, lowp);
        }
        launch_apply_q(dups, n, w, p.mode == 1, st);  // the sides not applied in WY form (plan_kernel zeroes META_WY)
        cnt[HCGB_STAGE_APPLY_Q]++;
        mark(HCGB_STAGE_FINALIZE);
        launch_finalize(dups, n, w, inf, st);
        cnt[HCGB_STAGE_FINALIZE]++;
    };
    const bool features = sh.any_compressed_c && ws.feat && (ctx->feature_sink || ctx->learned);
    const bool learned = ctx->learned && sh.any_compressed_c && p.fixed_rank == 0 && ws.off_sk1 && ws.pred;
    if (features) {
        mark(HCGB_STAGE_SKETCH);
        launch_features(dups, n, ws, p.accuracy, ctx->feature_sink, st);
    }
    if (learned) {
        // Randomized sketch sized by the predictor, then the plain recompression on the sketch
        // (pass A) and, for every update not sketched or whose residual test failed, on the
        // original stacks (pass B).
        mark(HCGB_STAGE_SKETCH);
        if (ctx->sk_policy == 0) launch_mlp_forward(ctx->model->m, ws.feat, n, ws.pred, st);  // y = log2(1 + r)
        launch_sketch_plan(dups, n, ws, p, ctx->sk_policy, ctx->sk_seed, djobs, st);
        launch_gemm_jobs(djobs, n, sched, st, lowp);                 // Z = V_s^T Omega
        launch_gemm_jobs(djobs + (size_t) n, n, sched, st, lowp);    // Y = U_s Z
        launch_sketch_qr(n, ws, st);
        launch_sketch_plan2(n, ws, p, djobs, st);
        launch_gemm_jobs(djobs, n, sched, st, lowp);                 // W = U_s^T Q_Y
        launch_gemm_jobs(djobs + (size_t) n, n, sched, st, lowp);    // V' = V_s W
        launch_sketch_pass(n, ws, p, 0, st);
        cnt[HCGB_STAGE_SKETCH]++;
        Workspace wsk = ws;
        wsk.off_ustack = ws.off_sk1;
        wsk.off_vstack = ws.off_sk2;
        recompress(wsk, nullptr);
        mark(HCGB_STAGE_SKETCH);
        launch_sketch_pass(n, ws, p, 1, st);
        recompress(ws, nullptr);
        mark(HCGB_STAGE_SKETCH);
        launch_sketch_pass(n, ws, p, 2, st);
        launch_learned_records(dups, n, ws, info, st);
    } else if (sh.any_compressed_c) {
        recompress(ws, info);
    } else {
        mark(HCGB_STAGE_FINALIZE);
        launch_finalize(dups, n, ws, info, st);
        cnt[HCGB_STAGE_FINALIZE]++;
    }
    mark(-1);
    if (ctx->prof) ctx->ev_pending.push_back(ev);
}

int prepare_workspace(hcgb_context *ctx, const BatchShape &sh, int n, bool ddc, Workspace *out, int mode = 0) {
    // The QR panels and the core's bookkeeping live in shared memory: refuse shapes beyond it.
    const size_t smem_limit = 227 * 1024;
    if (sh.any_compressed_c && (qr_smem_bytes(sh.ld, sh.kmax) > smem_limit || svd_smem_bytes(sh.kmax) > smem_limit))
        return fail(ctx, HCGB_POOL_TOO_SMALL, "tile too large: the QR panel or core bookkeeping exceeds shared memory");
    const bool learned = ctx->learned, features = learned || ctx->feature_sink;
    Workspace w = make_workspace_layout(sh.ld, sh.kmax, sh.rmax, ddc, ctx->oz != 0 || lowp_prec(mode) != 0, learned);
    size_t need = workspace_bytes_for(w, n, features);
    int rc = ensure_device(ctx, &ctx->ws, &ctx->ws_bytes, need);
    if (rc) return rc;
    w.base = static_cast<double *>(ctx->ws);
    w.meta = reinterpret_cast<int *>(static_cast<char *>(ctx->ws) + sizeof(double) * w.slot_doubles * (size_t) n);
    w.order = w.meta + (size_t) META_INTS * n;
    if (features) {
        const size_t fo = (sizeof(double) * w.slot_doubles * (size_t) n + sizeof(int) * (META_INTS + 1) * (size_t) n +
                           255) / 256 * 256;
        w.feat = reinterpret_cast<float *>(static_cast<char *>(ctx->ws) + fo);
        w.pred = w.feat + (size_t) MLP_IN * n;
    }
    *out = w;
    return HCGB_OK;
}

// Updates per pipeline launch for a batch of shape `sh`: at most `limit`, and few enough that the
// workspace stays within half of the device memory that is free or already held by the context.
int updates_per_launch(hcgb_context *ctx, const BatchShape &sh, int mode, int limit) {
    const bool features = ctx->learned || ctx->feature_sink;
    const Workspace w = make_workspace_layout(sh.ld, sh.kmax, sh.rmax, false, ctx->oz != 0 || lowp_prec(mode) != 0,
                                              ctx->learned);
    const size_t per = workspace_bytes_for(w, 1, features);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return limit;
    const size_t budget = (free_b + ctx->ws_bytes) / 2;
    const size_t fit = per ? budget / (per + per / 8) : (size_t) limit;
    return (int) std::max<size_t>(1, std::min<size_t>((size_t) limit, fit));
}

// Upload `n` device update descriptors and make room for 3n jobs; returns device pointers.
int upload_updates(hcgb_context *ctx, const std::vector<DevUpdate> &dv, DevUpdate **dups, GemmJob **djobs,
                   int **sched) {
    const size_t n = dv.size();
    const size_t ub = sizeof(DevUpdate) * n, jb = sizeof(GemmJob) * JOBS_PER_UPDATE * n;
    const size_t ub_al = (ub + 255) / 256 * 256, jb_al = (jb + 255) / 256 * 256;
    const size_t sb = sizeof(int) * SCHED_INTS_PER_UPDATE * n;
    int rc = ensure_device(ctx, &ctx->desc, &ctx->desc_bytes, ub_al + jb_al + sb);
    if (rc) return rc;
    rc = ensure_stage(ctx, ub);
    if (rc) return rc;
    std::memcpy(ctx->stage, dv.data(), ub);
    HCGB_CUDA(ctx, cudaMemcpyAsync(ctx->desc, ctx->stage, ub, cudaMemcpyHostToDevice, ctx->stream));
    HCGB_CUDA(ctx, cudaEventRecord(ctx->stage_done, ctx->stream));
    *dups = static_cast<DevUpdate *>(ctx->desc);
    *djobs = reinterpret_cast<GemmJob *>(static_cast<char *>(ctx->desc) + ub_al);
    *sched = reinterpret_cast<int *>(static_cast<char *>(ctx->desc) + ub_al + jb_al);
    return HCGB_OK;
}

}  // namespace

extern "C" {

int hcgb_context_create(int device, void *stream, hcgb_context **out) {
    if (!out) return HCGB_BAD_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return HCGB_CUDA_ERROR;
    if (cudaSetDevice(device) != cudaSuccess) return HCGB_CUDA_ERROR;
    auto *ctx = new hcgb_context();
    ctx->device = device;
    ctx->stream = static_cast<cudaStream_t>(stream);
    if (cudaEventCreateWithFlags(&ctx->stage_done, cudaEventDisableTiming) != cudaSuccess) {
        delete ctx;
        return HCGB_CUDA_ERROR;
    }
    *out = ctx;
    return HCGB_OK;
}

int hcgb_context_destroy(hcgb_context *ctx) {
    if (!ctx) return HCGB_BAD_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->ws) cudaFree(ctx->ws);
    if (ctx->desc) cudaFree(ctx->desc);
    if (ctx->pack_desc) cudaFree(ctx->pack_desc);
    if (ctx->tile_info) cudaFree(ctx->tile_info);
    if (ctx->be_scratch) cudaFree(ctx->be_scratch);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->capture_stream) cudaStreamDestroy(ctx->capture_stream);
    if (ctx->graph_desc) cudaFree(ctx->graph_desc);
    if (ctx->stage) cudaFreeHost(ctx->stage);
    if (ctx->stage_done) cudaEventDestroy(ctx->stage_done);
    for (auto &g : ctx->ev_pending)
        for (auto &e : g) cudaEventDestroy(e.second);
    for (auto e : ctx->ev_free) cudaEventDestroy(e);
    for (auto st : ctx->group_streams) cudaStreamDestroy(st);
    for (auto e : ctx->group_events) cudaEventDestroy(e);
    delete ctx;
    return HCGB_OK;
}

int hcgb_context_set_stream(hcgb_context *ctx, void *stream) {
    if (!ctx) return HCGB_BAD_ARG;
    ctx->stream = static_cast<cudaStream_t>(stream);
    return HCGB_OK;
}

int hcgb_sync(hcgb_context *ctx) {
    if (!ctx) return HCGB_BAD_ARG;
    HCGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HCGB_OK;
}

const char *hcgb_last_error(hcgb_context *ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

size_t hcgb_workspace_bytes(int n, int max_rows, int max_cols, int max_rank_c, int max_rank_ab) {
    if (n <= 0) return 0;
    int ld = std::max(max_rows, max_cols);
    ld = (ld + 7) / 8 * 8;
    Workspace w = make_workspace_layout(ld, max_rank_c + max_rank_ab, std::max(8, max_rank_ab), false);
    return workspace_bytes_for(w, n);
}

int hcgb_gemm_batch(hcgb_context *ctx, double alpha, double beta, int n, const hcgb_update *updates,
                    const hcgb_params *params, hcgb_update_info *info_dev) {
    if (!ctx) return HCGB_BAD_ARG;
    if (n == 0) return HCGB_OK;
    if (n < 0 || !updates) return fail(ctx, HCGB_BAD_ARG, "hcgb_gemm_batch: bad update list");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<DevUpdate> dv(n);
    for (int i = 0; i < n; i++) {
        int rc;
        if ((rc = check_tile(ctx, updates[i].a, "A")) || (rc = check_tile(ctx, updates[i].b, "B")) ||
            (rc = check_tile(ctx, updates[i].c, "C")))
            return rc;
        if (updates[i].a.kind == HCGB_DENSE && updates[i].b.kind == HCGB_DENSE &&
            compressed(updates[i].c.kind))
            return fail(ctx, HCGB_UNSUPPORTED, "hcgb_gemm_batch: DDC updates go through hcgb_tile_gemm");
        dv[i] = DevUpdate{to_dev(updates[i].a), to_dev(updates[i].b), to_dev(updates[i].c), i};
    }
    BatchShape sh = shape_of(updates, n);
    Workspace ws;
    int rc = prepare_workspace(ctx, sh, n, false, &ws, params ? params->mode : 0);
    if (rc) return rc;
    DevUpdate *dups;
    GemmJob *djobs;
    int *dsched;
    if ((rc = upload_updates(ctx, dv, &dups, &djobs, &dsched))) return rc;
    launch_pipeline(ctx, ctx->stream, dups, djobs, dsched, n, alpha, beta, ws, sh, to_params(params, ctx), info_dev);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

int hcgb_tlr_gemm(hcgb_context *ctx, int mt, int nt, int kt, double alpha, const hcgb_tile *a_grid,
                  const hcgb_tile *b_grid, double beta, const hcgb_tile *c_grid, const hcgb_params *params,
                  hcgb_update_info *info_dev) {
    if (!ctx) return HCGB_BAD_ARG;
    if (mt <= 0 || nt <= 0 || kt <= 0 || !a_grid || !b_grid || !c_grid)
        return fail(ctx, HCGB_BAD_ARG, "hcgb_tlr_gemm: bad grid");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    const int n = mt * nt;
    // Graph mode: replay the captured multiply while its arguments and the context's settings are
    // those it was captured with (and the workspace has not moved).
    std::string key;
    if (ctx->graph_mode) {
        auto put = [&](const void *p, size_t b) { key.append(static_cast<const char *>(p), b); };
        const int ints[] = {mt, nt, kt, ctx->groups, ctx->k_order, ctx->oz, ctx->learned ? 1 : 0, ctx->sk_policy,
                            ctx->oz_min, ctx->wy_min, ctx->precond_min, ctx->sk_pct};
        put(ints, sizeof(ints));
        put(&alpha, sizeof(alpha));
        put(&beta, sizeof(beta));
        hcgb_params pz{};
        if (params) pz = *params;
        put(&pz, sizeof(pz));
        const void *ptrs[] = {ctx->model, ctx->feature_sink, info_dev, ctx->stream};
        put(ptrs, sizeof(ptrs));
        put(&ctx->sk_seed, sizeof(ctx->sk_seed));
        put(a_grid, sizeof(hcgb_tile) * (size_t) mt * kt);
        put(b_grid, sizeof(hcgb_tile) * (size_t) kt * nt);
        put(c_grid, sizeof(hcgb_tile) * (size_t) n);
        if (ctx->graph_exec && key == ctx->graph_key && ctx->graph_ws == ctx->ws) {
            HCGB_CUDA(ctx, cudaGraphLaunch(ctx->graph_exec, ctx->stream));
            note_launches(ctx->graph_launches);
            return HCGB_OK;
        }
    }
    // C tiles are split into G groups (tile index mod G); each group runs its own chain of k-waves
    // on its own stream, so one slow update delays only its group, not every C tile.
    const int G = std::max(1, std::min(ctx->groups, n));
    std::vector<int> first(G + 1, 0), members;
    for (int g = 0; g < G; g++) {
        first[g] = (int) members.size();
        for (int idx = g; idx < n; idx += G) members.push_back(idx);
    }
    first[G] = n;
    // k order per C tile: the reference's ascending k, or (k_order = 1) the updates of each C tile
    // sorted by estimated recompression cost (stack width cubed), largest first, so that the
    // expensive updates of all tiles fall into the same few k-waves instead of one per wave.
    std::vector<int> korder((size_t) n * kt);
    for (int idx = 0; idx < n; idx++)
        for (int kk = 0; kk < kt; kk++) korder[(size_t) idx * kt + kk] = kk;
    if (ctx->k_order == 1) {
        auto rank_of = [&](const hcgb_tile &t, int *out) -> int {
            *out = compressed(t.kind) ? -1 : t.rows;
            return HCGB_OK;
        };
        // gather device ranks of every compressed tile with one synchronisation
        std::vector<int> ra((size_t) mt * kt), rb((size_t) kt * nt), rcv((size_t) n);
        for (size_t q = 0; q < ra.size(); q++) rank_of(a_grid[q], &ra[q]);
        for (size_t q = 0; q < rb.size(); q++) rank_of(b_grid[q], &rb[q]);
        for (size_t q = 0; q < rcv.size(); q++) rank_of(c_grid[q], &rcv[q]);
        // The device ranks of every compressed tile, gathered by one kernel and read with one copy.
        std::vector<const int *> ptrs;
        std::vector<int *> dst;
        auto collect = [&](const hcgb_tile *grid, std::vector<int> &v) {
            for (size_t q = 0; q < v.size(); q++)
                if (compressed(grid[q].kind)) {
                    ptrs.push_back(grid[q].rank);
                    dst.push_back(&v[q]);
                }
        };
        collect(a_grid, ra);
        collect(b_grid, rb);
        collect(c_grid, rcv);
        const size_t np = ptrs.size();
        if (np) {
            const size_t pb = sizeof(const int *) * np, ib = sizeof(int) * np;
            int rc0;
            if ((rc0 = ensure_device(ctx, &ctx->pack_desc, &ctx->pack_desc_bytes, pb + ib))) return rc0;
            if ((rc0 = ensure_stage(ctx, pb + ib))) return rc0;
            std::memcpy(ctx->stage, ptrs.data(), pb);
            auto *dptrs = static_cast<const int **>(ctx->pack_desc);
            int *dvals = reinterpret_cast<int *>(static_cast<char *>(ctx->pack_desc) + pb);
            HCGB_CUDA(ctx, cudaMemcpyAsync(ctx->pack_desc, ctx->stage, pb, cudaMemcpyHostToDevice, ctx->stream));
            launch_gather_ranks(dptrs, (int) np, dvals, ctx->stream);
            int *hst = reinterpret_cast<int *>(static_cast<char *>(ctx->stage) + pb);
            HCGB_CUDA(ctx, cudaMemcpyAsync(hst, dvals, ib, cudaMemcpyDeviceToHost, ctx->stream));
            HCGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (size_t q = 0; q < np; q++) *dst[q] = hst[q];
        }
        for (int idx = 0; idx < n; idx++) {
            const int i = idx % mt, j = idx / mt;
            if (!compressed(c_grid[idx].kind)) continue;
            std::vector<std::pair<double, int>> est(kt);
            for (int kk = 0; kk < kt; kk++) {
                const hcgb_tile &ta = a_grid[i + (size_t) kk * mt], &tb = b_grid[kk + (size_t) j * kt];
                const int rA = ra[i + (size_t) kk * mt], rB = rb[kk + (size_t) j * kt];
                int add;
                if (ta.kind == HCGB_DENSE && tb.kind == HCGB_DENSE) add = 0;
                else if (ta.kind == HCGB_DENSE) add = rB;
                else if (tb.kind == HCGB_DENSE) add = rA;
                else add = std::min(rA, rB);
                const double kw = (double) (rcv[idx] + add);
                est[kk] = {-kw * kw * kw, kk};
            }
            std::stable_sort(est.begin(), est.end());
            for (int kk = 0; kk < kt; kk++) korder[(size_t) idx * kt + kk] = est[kk].second;
        }
    }
    // Descriptors laid out [group][wave][member]; record uid = k * n + tile index.
    std::vector<hcgb_update> all((size_t) n * kt);
    std::vector<DevUpdate> dv((size_t) n * kt);
    for (int g = 0; g < G; g++) {
        const int ng = first[g + 1] - first[g];
        for (int kk = 0; kk < kt; kk++)
            for (int q = 0; q < ng; q++) {
                const int idx = members[first[g] + q];
                const int i = idx % mt, j = idx / mt;
                const int kx = korder[(size_t) idx * kt + kk];
                const size_t w = (size_t) first[g] * kt + (size_t) kk * ng + q;
                hcgb_update u{a_grid[i + (size_t) kx * mt], b_grid[kx + (size_t) j * kt], c_grid[idx]};
                int rc;
                if ((rc = check_tile(ctx, u.a, "A")) || (rc = check_tile(ctx, u.b, "B")) ||
                    (rc = check_tile(ctx, u.c, "C")))
                    return rc;
                if (u.a.kind == HCGB_DENSE && u.b.kind == HCGB_DENSE && compressed(u.c.kind))
                    return fail(ctx, HCGB_UNSUPPORTED, "hcgb_tlr_gemm: DDC updates are not batched");
                all[w] = u;
                dv[w] = DevUpdate{to_dev(u.a), to_dev(u.b), to_dev(u.c), kx * n + idx, i > j ? i - j : j - i};
            }
    }
    BatchShape sh = shape_of(all.data(), (int) all.size());
    Workspace ws;
    int rc = prepare_workspace(ctx, sh, n, false, &ws, params ? params->mode : 0);
    if (rc) return rc;
    const size_t ub = sizeof(DevUpdate) * dv.size(), ub_al = (ub + 255) / 256 * 256;
    const size_t jb = sizeof(GemmJob) * JOBS_PER_UPDATE * (size_t) n, jb_al = (jb + 255) / 256 * 256;
    const size_t sb = sizeof(int) * SCHED_INTS_PER_UPDATE * (size_t) n;
    void **dbuf = ctx->graph_mode ? &ctx->graph_desc : &ctx->desc;
    size_t *dbytes = ctx->graph_mode ? &ctx->graph_desc_bytes : &ctx->desc_bytes;
    if ((rc = ensure_device(ctx, dbuf, dbytes, ub_al + jb_al + sb))) return rc;
    if ((rc = ensure_stage(ctx, ub))) return rc;
    std::memcpy(ctx->stage, dv.data(), ub);
    HCGB_CUDA(ctx, cudaMemcpyAsync(*dbuf, ctx->stage, ub, cudaMemcpyHostToDevice, ctx->stream));
    HCGB_CUDA(ctx, cudaEventRecord(ctx->stage_done, ctx->stream));
    auto *dups = static_cast<DevUpdate *>(*dbuf);
    auto *djobs = reinterpret_cast<GemmJob *>(static_cast<char *>(*dbuf) + ub_al);
    auto *dsched = reinterpret_cast<int *>(static_cast<char *>(*dbuf) + ub_al + jb_al);
    const Params p = to_params(params, ctx);
    // Streams and fork/join events for the groups.
    while ((int) ctx->group_streams.size() < G) {
        cudaStream_t s;
        HCGB_CUDA(ctx, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        ctx->group_streams.push_back(s);
    }
    while ((int) ctx->group_events.size() < G + 1) {
        cudaEvent_t e;
        HCGB_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->group_events.push_back(e);
    }
    const bool single = (G == 1);
    // Graph mode: the descriptors are on the device before the capture; then every launch of the
    // multiply (all groups, all waves) is recorded into one graph and the graph is launched.
    const bool capture = ctx->graph_mode;
    const bool prof_saved = ctx->prof;
    long long launches0 = 0;
    // The stream the launches are issued on: the context's, or for a capture on the legacy default
    // stream (which cannot be captured) a stream of the context's own; the graph then runs on the
    // context's stream.
    cudaStream_t main_st = ctx->stream;
    if (capture) {
        HCGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (ctx->graph_exec) {
            cudaGraphExecDestroy(ctx->graph_exec);
            ctx->graph_exec = nullptr;
        }
        if (!main_st) {
            if (!ctx->capture_stream)
                HCGB_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking));
            main_st = ctx->capture_stream;
        }
        ctx->prof = false;  // no profiling events inside a graph
        launches0 = hcgb_kernel_launches();
        HCGB_CUDA(ctx, cudaStreamBeginCapture(main_st, cudaStreamCaptureModeThreadLocal));
    }
    if (!single) HCGB_CUDA(ctx, cudaEventRecord(ctx->group_events[0], main_st));
    std::vector<Workspace> wgs((size_t) G);
    for (int g = 0; g < G; g++) {
        cudaStream_t st = single ? main_st : ctx->group_streams[g];
        if (!single) HCGB_CUDA(ctx, cudaStreamWaitEvent(st, ctx->group_events[0], 0));
        Workspace &wg = wgs[g];
        wg = ws;
        wg.base = ws.base + ws.slot_doubles * (size_t) first[g];
        wg.meta = ws.meta + (size_t) META_INTS * first[g];
        wg.order = ws.order + first[g];
        if (ws.feat) {
            wg.feat = ws.feat + (size_t) MLP_IN * first[g];
            wg.pred = ws.pred + first[g];
        }
    }
    // Waves are issued round-robin over the groups, so every group starts at once instead of
    // waiting for the host to enqueue the earlier groups' whole chains.
    for (int kk = 0; kk < kt; kk++)
        for (int g = 0; g < G; g++) {
            const int ng = first[g + 1] - first[g];
            cudaStream_t st = single ? main_st : ctx->group_streams[g];
            const size_t off = (size_t) first[g] * kt + (size_t) kk * ng;
            BatchShape shw = shape_of(all.data() + off, ng);
            shw.ld = sh.ld;
            shw.kmax = sh.kmax;
            shw.rmax = sh.rmax;
            launch_pipeline(ctx, st, dups + off, djobs + JOBS_PER_UPDATE * (size_t) first[g],
                            dsched + SCHED_INTS_PER_UPDATE * (size_t) first[g], ng, alpha, beta, wgs[g], shw, p,
                            info_dev);
        }
    if (!single)
        for (int g = 0; g < G; g++) {
            HCGB_CUDA(ctx, cudaEventRecord(ctx->group_events[g + 1], ctx->group_streams[g]));
            HCGB_CUDA(ctx, cudaStreamWaitEvent(main_st, ctx->group_events[g + 1], 0));
        }
    if (capture) {
        ctx->prof = prof_saved;
        cudaGraph_t graph = nullptr;
        HCGB_CUDA(ctx, cudaStreamEndCapture(main_st, &graph));
        const cudaError_t e = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            ctx->graph_exec = nullptr;
            return fail(ctx, HCGB_CUDA_ERROR, std::string("hcgb_tlr_gemm: cudaGraphInstantiate: ") + cudaGetErrorString(e));
        }
        ctx->graph_key = key;
        ctx->graph_ws = ctx->ws;
        ctx->graph_launches = hcgb_kernel_launches() - launches0;
        HCGB_CUDA(ctx, cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    }
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

int hcgb_set_k_order(hcgb_context *ctx, int policy) {
    if (!ctx || policy < 0 || policy > 1) return HCGB_BAD_ARG;
    ctx->k_order = policy;
    return HCGB_OK;
}

int hcgb_set_concurrency(hcgb_context *ctx, int groups) {
    if (!ctx || groups < 1) return HCGB_BAD_ARG;
    ctx->groups = groups;
    return HCGB_OK;
}

}  // extern "C"

namespace {

// The reference's flop count of one CompressedTile<T>::Gemm on the default (ungqr, non-trmm,
// non-Cholesky) path, Compressed.cpp:335-625, including its integer arithmetic.
unsigned long long reference_recompression_flops(size_t m, size_t n, size_t crk, size_t arank, size_t rk,
                                                 bool fixed) {
    const size_t Um = m, Un = arank + crk, Vm = n, Vn = Un;
    const size_t minU = std::min(Um, Un), minV = std::min(Vm, Vn);
    const size_t sizeS = std::min(std::min(m, n), Un);
    size_t f = 0;
    f += m * crk + m * arank + m * arank;
    f += 2 * Um * Un * Un - (size_t) (2.0 * (float) Un * (float) Un * (float) Un / 3.0f) + 2 * Um * Un +
         (size_t) (17 * (float) Un / 3.0f);
    f += minU * ((Un + 1) / 2) * 2;
    f += n * crk + n * arank;
    f += 2 * Vm * Vn * Vn - (size_t) (2 * (float) Vn * (float) Vn * (float) Vn / 3.0f) + 2 * Vm * Vn +
         (size_t) (17 * (float) Vn / 3.0f);
    f += minV * ((Vn + 1) / 2) * 2;
    f += minU * minV * Un;
    f += 22 * minV * minV * minV;
    if (!fixed) f += sizeS;
    f += (8 / 3) * (size_t) ((double) minU * (double) minU) * (3 * Um - minU);
    f += Um * rk * minU;
    f += rk;
    f += (8 / 3) * (size_t) ((double) minV * (double) minV) * (3 * Vm - minV);
    f += Vm * rk * minV;
    return f;
}

struct TempTile {
    double *buf = nullptr;
    int *rank = nullptr;
};

// op(T) as an explicit tile: dense -> transposed copy; compressed (U, V) -> (V^T, U^T).
int transposed_tile(hcgb_context *ctx, const hcgb_tile &t, int rank, hcgb_tile *out, TempTile *tmp) {
    *out = t;
    out->rows = t.cols;
    out->cols = t.rows;
    if (t.kind == HCGB_DENSE) {
        HCGB_CUDA(ctx, cudaMalloc(&tmp->buf, sizeof(double) * (size_t) t.rows * t.cols));
        launch_transpose(t.data, t.rows, t.rows, t.cols, tmp->buf, t.cols, ctx->stream);
        out->data = tmp->buf;
        return HCGB_OK;
    }
    const size_t cap = (size_t) t.cols * t.max_rank + (size_t) t.max_rank * t.rows;
    HCGB_CUDA(ctx, cudaMalloc(&tmp->buf, sizeof(double) * cap));
    const double *U = t.data, *V = t.data + (size_t) t.rows * t.max_rank;
    if (t.kind == HCGB_COMPRESSED_VT) {
        // (U W^T)^T = W U^T: the factors swap places, both already in their layouts.
        if (rank > 0) {
            HCGB_CUDA(ctx, cudaMemcpyAsync(tmp->buf, V, sizeof(double) * (size_t) t.cols * rank,
                                           cudaMemcpyDeviceToDevice, ctx->stream));
            HCGB_CUDA(ctx, cudaMemcpyAsync(tmp->buf + (size_t) t.cols * t.max_rank, U,
                                           sizeof(double) * (size_t) t.rows * rank, cudaMemcpyDeviceToDevice,
                                           ctx->stream));
        }
    } else {
        // new U (cols x rank, ld cols) = V^T, new V (rank x rows, ld rank) = U^T
        launch_transpose(V, rank, rank, t.cols, tmp->buf, t.cols, ctx->stream);
        launch_transpose(U, t.rows, t.rows, rank, tmp->buf + (size_t) t.cols * t.max_rank, rank, ctx->stream);
    }
    out->data = tmp->buf;
    out->rank = t.rank;  // the rank itself is unchanged
    return HCGB_OK;
}

int read_rank(hcgb_context *ctx, const hcgb_tile &t, int *r) {
    *r = 0;
    if (!compressed(t.kind)) return HCGB_OK;
    HCGB_CUDA(ctx, cudaMemcpyAsync(r, t.rank, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    HCGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HCGB_OK;
}

}  // namespace

extern "C" int hcgb_set_tensor_products(hcgb_context *ctx, int enable) {
    if (!ctx) return HCGB_BAD_ARG;
    if (enable != 0 && enable != 1) return fail(ctx, HCGB_BAD_ARG, "hcgb_set_tensor_products: 0 or 1");
    ctx->oz = enable;
    return HCGB_OK;
}

extern "C" int hcgb_tile_gemm(hcgb_context *ctx, double alpha, const hcgb_tile *a, int op_a, const hcgb_tile *b,
                              int op_b, double beta, hcgb_tile *c, const hcgb_params *params, int *new_rank,
                              unsigned long long *flops) {
    if (!ctx) return HCGB_BAD_ARG;
    if (!a || !b || !c) return fail(ctx, HCGB_BAD_ARG, "hcgb_tile_gemm: null tile");
    if ((op_a != HCGB_NOTRANS && op_a != HCGB_TRANS) || (op_b != HCGB_NOTRANS && op_b != HCGB_TRANS))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_tile_gemm: op must be NoTrans or Trans");
    int rc;
    if ((rc = check_tile(ctx, *a, "A")) || (rc = check_tile(ctx, *b, "B")) || (rc = check_tile(ctx, *c, "C")))
        return rc;
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    int ra, rb, rcank;
    if ((rc = read_rank(ctx, *a, &ra)) || (rc = read_rank(ctx, *b, &rb)) || (rc = read_rank(ctx, *c, &rcank)))
        return rc;
    TempTile ta, tb;
    hcgb_tile A = *a, B = *b;
    if (op_a == HCGB_TRANS && (rc = transposed_tile(ctx, *a, ra, &A, &ta))) return rc;
    if (op_b == HCGB_TRANS && (rc = transposed_tile(ctx, *b, rb, &B, &tb))) return rc;
    auto cleanup = [&]() {
        cudaStreamSynchronize(ctx->stream);
        if (ta.buf) cudaFree(ta.buf);
        if (tb.buf) cudaFree(tb.buf);
    };
    if (A.cols != B.rows || A.rows != c->rows || B.cols != c->cols) {
        cleanup();
        return fail(ctx, HCGB_BAD_ARG, "hcgb_tile_gemm: shapes of op(A), op(B) and C do not match");
    }
    const size_t m = c->rows, n = c->cols, kd = A.cols;
    const bool ak = compressed(A.kind), bk = compressed(B.kind), ck = compressed(c->kind);
    unsigned long long fl = 0;
    int out_rank = 0;
    if (!ak && !bk && ck) {
        // DDC (HCore.cpp:272-299): W = alpha A B + beta Cu Cv, C <- U = W, V = I at rank min(m, n).
        const int r = (int) std::min(m, n);
        if (c->max_rank < r) {
            cleanup();
            return fail(ctx, HCGB_RANK_OVERFLOW, "hcgb_tile_gemm: DDC needs max_rank >= min(rows, cols)");
        }
        hcgb_update u{A, B, *c};
        BatchShape sh = shape_of(&u, 1);
        Workspace ws;
        if ((rc = prepare_workspace(ctx, sh, 1, true, &ws))) {
            cleanup();
            return rc;
        }
        std::vector<DevUpdate> dv{DevUpdate{to_dev(A), to_dev(B), to_dev(*c), 0}};
        DevUpdate *dups;
        GemmJob *djobs;
        int *dsched;
        if ((rc = upload_updates(ctx, dv, &dups, &djobs, &dsched))) {
            cleanup();
            return rc;
        }
        GemmJob j[3];
        std::memset(j, 0, sizeof(j));
        double *W = ws.base + ws.off_tmp2;
        const double *Cu = c->data, *Cv = c->data + m * (size_t) c->max_rank;
        const bool cvt = c->kind == HCGB_COMPRESSED_VT;  // Cv read as W^T (W: n x rank, ld n)
        j[0] = GemmJob{Cu, Cv, W, (int) m, (int) n, rcank, (int) m, cvt ? (int) n : std::max(1, rcank), ws.ld,
                       0, cvt ? 1 : 0, beta, 0.0};
        j[1] = GemmJob{A.data, B.data, W, (int) m, (int) n, (int) kd, (int) m, (int) kd, ws.ld, 0, 0, alpha, 1.0};
        if ((rc = ensure_stage(ctx, sizeof(j)))) {
            cleanup();
            return rc;
        }
        std::memcpy(ctx->stage, j, sizeof(j));
        HCGB_CUDA(ctx, cudaMemcpyAsync(djobs, ctx->stage, sizeof(j), cudaMemcpyHostToDevice, ctx->stream));
        HCGB_CUDA(ctx, cudaEventRecord(ctx->stage_done, ctx->stream));
        launch_gemm_jobs(djobs, 1, dsched, ctx->stream);
        launch_gemm_jobs(djobs + 1, 1, dsched, ctx->stream);
        launch_ddc_finalize(dups, 1, ws, ctx->stream);
        HCGB_CUDA(ctx, cudaGetLastError());
        fl = 2ull * m * n * kd + 2ull * m * n * (unsigned long long) rcank;
        out_rank = r;
    } else {
        hcgb_update u{A, B, *c};
        if (!ctx->tile_info) HCGB_CUDA(ctx, cudaMalloc(&ctx->tile_info, sizeof(hcgb_update_info)));
        hcgb_update_info *dinfo = ctx->tile_info;
        rc = hcgb_gemm_batch(ctx, alpha, beta, 1, &u, params, dinfo);
        int hstatus = HCGB_OK;
        if (rc == HCGB_OK) {
            HCGB_CUDA(ctx, cudaMemcpyAsync(&hstatus, &dinfo->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            if (ck) HCGB_CUDA(ctx, cudaMemcpyAsync(&out_rank, c->rank, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            HCGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        }
        if (rc) {
            cleanup();
            return rc;
        }
        if (hstatus != HCGB_OK && hstatus != HCGB_NOT_CONVERGED) {
            cleanup();
            return fail(ctx, hstatus, "hcgb_tile_gemm: update rejected on the device");
        }
        // Temporary dense products (Dense.cpp:66-67: 2 * m * n * A.cols each), then the recompression.
        const size_t arank = ak && bk ? (size_t) ra : (!ak && bk ? (size_t) rb : (size_t) ra);
        if (ak && bk) fl += 2ull * ra * rb * kd + 2ull * ra * n * rb;
        else if (!ak && bk) fl += 2ull * m * rb * kd;
        else if (ak && !bk) fl += 2ull * ra * n * kd;
        if (ck) fl += reference_recompression_flops(m, n, rcank, arank, out_rank, params && params->fixed_rank);
        else fl += 2ull * m * n * (ak ? (unsigned long long) ra : (bk ? rb : kd));
        if (hstatus == HCGB_NOT_CONVERGED) ctx->last_error = "hcgb_tile_gemm: Jacobi sweep limit reached";
        rc = hstatus;
    }
    cleanup();
    if (new_rank) *new_rank = ck ? out_rank : 0;
    if (flops) *flops += fl;
    return rc;
}

extern "C" int hcgb_profile_enable(hcgb_context *ctx, int enable) {
    if (!ctx) return HCGB_BAD_ARG;
    ctx->prof = enable != 0;
    return HCGB_OK;
}

extern "C" int hcgb_profile_reset(hcgb_context *ctx) {
    if (!ctx) return HCGB_BAD_ARG;
    HCGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (auto &g : ctx->ev_pending)
        for (auto &e : g) ctx->ev_free.push_back(e.second);
    ctx->ev_pending.clear();
    for (int i = 0; i < HCGB_NUM_STAGES; i++) {
        ctx->stage_ms[i] = 0.0;
        ctx->stage_launches[i] = 0;
    }
    return HCGB_OK;
}

extern "C" int hcgb_profile_read(hcgb_context *ctx, double *ms_per_stage, long long *launches_per_stage,
                                 int nstages) {
    if (!ctx || nstages < 0) return HCGB_BAD_ARG;
    HCGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (auto &g : ctx->ev_pending) {
        for (size_t i = 0; i + 1 < g.size(); i++) {
            float ms = 0.f;
            HCGB_CUDA(ctx, cudaEventElapsedTime(&ms, g[i].second, g[i + 1].second));
            if (g[i].first >= 0 && g[i].first < HCGB_NUM_STAGES) ctx->stage_ms[g[i].first] += ms;
        }
        for (auto &e : g) ctx->ev_free.push_back(e.second);
    }
    ctx->ev_pending.clear();
    for (int i = 0; i < nstages && i < HCGB_NUM_STAGES; i++) {
        if (ms_per_stage) ms_per_stage[i] = ctx->stage_ms[i];
        if (launches_per_stage) launches_per_stage[i] = ctx->stage_launches[i];
    }
    return HCGB_OK;
}

extern "C" int hcgb_fp64_peak(hcgb_context *ctx, double *dmma_tflops, double *dfma_tflops) {
    if (!ctx) return HCGB_BAD_ARG;
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    int rc = measure_fp64_peak(ctx->stream, dmma_tflops, dfma_tflops);
    if (rc) return fail(ctx, rc, "hcgb_fp64_peak: probe failed");
    return HCGB_OK;
}

namespace {

__global__ void identity_kernel(double *a, int n, int ld) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x)
        a[(e % n) + (size_t) (e / n) * ld] = (e % n) == (e / n) ? 1.0 : 0.0;
}

}  // namespace

extern "C" int hcgb_compress_tile(hcgb_context *ctx, const double *dense, int rows, int cols, hcgb_tile *out,
                                  const hcgb_params *params, int *rank) {
    if (!ctx) return HCGB_BAD_ARG;
    if (!dense || !out || rows <= 0 || cols <= 0 || !compressed(out->kind) || out->rows != rows ||
        out->cols != cols || !out->rank || out->max_rank <= 0)
        return fail(ctx, HCGB_BAD_ARG, "hcgb_compress_tile: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    // D = D * I: an update with A = the dense tile, B = I (compressed, U = V = I_cols), C = 0 (rank 0)
    // recompresses exactly the columns of D, i.e. computes its truncated SVD.
    double *ibuf = nullptr;
    int *irank = nullptr;
    const size_t n = (size_t) cols;
    HCGB_CUDA(ctx, cudaMalloc(&ibuf, sizeof(double) * 2 * n * n));
    HCGB_CUDA(ctx, cudaMalloc(&irank, sizeof(int)));
    { identity_kernel<<<64, 256, 0, ctx->stream>>>(ibuf, cols, cols); note_launch(); }
    { identity_kernel<<<64, 256, 0, ctx->stream>>>(ibuf + n * n, cols, cols); note_launch(); }
    const int ncols = cols;
    HCGB_CUDA(ctx, cudaMemcpyAsync(irank, &ncols, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    HCGB_CUDA(ctx, cudaMemsetAsync(out->rank, 0, sizeof(int), ctx->stream));
    hcgb_tile a{const_cast<double *>(dense), nullptr, rows, cols, 0, HCGB_DENSE};
    hcgb_tile b{ibuf, irank, cols, cols, cols, HCGB_COMPRESSED};
    int r = 0;
    int rc = hcgb_tile_gemm(ctx, 1.0, &a, HCGB_NOTRANS, &b, HCGB_NOTRANS, 0.0, out, params, &r, nullptr);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ibuf);
    cudaFree(irank);
    if (rank) *rank = r;
    return rc;
}

extern "C" int hcgb_compress_tiles(hcgb_context *ctx, int count, const double *const *dense, int rows, int cols,
                                   hcgb_tile *out, const hcgb_params *params, int *ranks) {
    if (!ctx) return HCGB_BAD_ARG;
    if (count < 0 || (count > 0 && (!dense || !out)) || rows <= 0 || cols <= 0)
        return fail(ctx, HCGB_BAD_ARG, "hcgb_compress_tiles: bad arguments");
    for (int i = 0; i < count; i++)
        if (!dense[i] || !compressed(out[i].kind) || out[i].rows != rows || out[i].cols != cols || !out[i].rank ||
            out[i].max_rank <= 0)
            return fail(ctx, HCGB_BAD_ARG, "hcgb_compress_tiles: bad tile " + std::to_string(i));
    if (count == 0) return HCGB_OK;
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    // Every tile is the update C_i = D_i * I with C_i at rank 0 (as in hcgb_compress_tile); the
    // identity factors are shared by the whole batch.
    double *ibuf = nullptr;
    int *irank = nullptr;
    hcgb_update_info *dinfo = nullptr;
    const size_t n = (size_t) cols;
    auto done = [&](int rc) {
        cudaStreamSynchronize(ctx->stream);
        if (ibuf) cudaFree(ibuf);
        if (irank) cudaFree(irank);
        if (dinfo) cudaFree(dinfo);
        return rc;
    };
    if (cudaMalloc(&ibuf, sizeof(double) * 2 * n * n) != cudaSuccess || cudaMalloc(&irank, sizeof(int)) != cudaSuccess)
        return done(fail(ctx, HCGB_CUDA_ERROR, "hcgb_compress_tiles: cudaMalloc failed"));
    { identity_kernel<<<64, 256, 0, ctx->stream>>>(ibuf, cols, cols); note_launch(); }
    { identity_kernel<<<64, 256, 0, ctx->stream>>>(ibuf + n * n, cols, cols); note_launch(); }
    const int ncols = cols;
    auto failed = [&](cudaError_t e) {  // a CUDA call failed: release what this call allocated
        return done(fail(ctx, HCGB_CUDA_ERROR, std::string("hcgb_compress_tiles: ") + cudaGetErrorString(e)));
    };
    cudaError_t ce = cudaMemcpyAsync(irank, &ncols, sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
    if (ce != cudaSuccess) return failed(ce);
    const hcgb_tile ident{ibuf, irank, cols, cols, cols, HCGB_COMPRESSED};
    std::vector<hcgb_update> ups(count);
    for (int i = 0; i < count; i++) {
        if ((ce = cudaMemsetAsync(out[i].rank, 0, sizeof(int), ctx->stream)) != cudaSuccess) return failed(ce);
        ups[i] = hcgb_update{hcgb_tile{const_cast<double *>(dense[i]), nullptr, rows, cols, 0, HCGB_DENSE}, ident,
                             out[i]};
    }
    const int mode = params ? params->mode : 0;
    const int chunk = updates_per_launch(ctx, shape_of(ups.data(), 1), mode, count);
    if (cudaMalloc(&dinfo, sizeof(hcgb_update_info) * (size_t) chunk) != cudaSuccess)
        return done(fail(ctx, HCGB_CUDA_ERROR, "hcgb_compress_tiles: cudaMalloc failed"));
    std::vector<hcgb_update_info> hinfo(chunk);
    bool not_converged = false;
    for (int off = 0; off < count; off += chunk) {
        const int nb = std::min(chunk, count - off);
        int rc = hcgb_gemm_batch(ctx, 1.0, 0.0, nb, ups.data() + off, params, dinfo);
        if (rc) return done(rc);
        if ((ce = cudaMemcpyAsync(hinfo.data(), dinfo, sizeof(hcgb_update_info) * (size_t) nb,
                                  cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
            (ce = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
            return failed(ce);
        for (int i = 0; i < nb; i++) {
            const int st = hinfo[i].status;
            if (st == HCGB_NOT_CONVERGED) not_converged = true;
            else if (st != HCGB_OK)
                return done(fail(ctx, st, "hcgb_compress_tiles: tile " + std::to_string(off + i) + " failed"));
            if (ranks) ranks[off + i] = hinfo[i].new_rank;
        }
    }
    return done(not_converged ? HCGB_NOT_CONVERGED : HCGB_OK);
}

extern "C" int hcgb_potrf(hcgb_context *ctx, int uplo, int n, double *A, int lda, int *info) {
    if (!ctx) return HCGB_BAD_ARG;
    if (!A || n < 0 || lda < (n > 1 ? n : 1) || (uplo != HCGB_LOWER && uplo != HCGB_UPPER))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_potrf: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    if (n == 0) {
        if (info) *info = 0;
        return HCGB_OK;
    }
    int *dinfo = nullptr;
    HCGB_CUDA(ctx, cudaMalloc(&dinfo, sizeof(int)));
    launch_potrf(A, n, lda, uplo, dinfo, ctx->stream);
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, dinfo, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(dinfo);
    if (e != cudaSuccess) return fail(ctx, HCGB_CUDA_ERROR, std::string("hcgb_potrf: ") + cudaGetErrorString(e));
    if (info) *info = h;
    return HCGB_OK;
}

extern "C" int hcgb_trsm(hcgb_context *ctx, int side, int uplo, int trans, int diag, int m, int n, double alpha,
                         const double *A, int lda, double *B, int ldb) {
    if (!ctx) return HCGB_BAD_ARG;
    const int na = side == HCGB_LEFT ? m : n;
    if (!A || !B || m < 0 || n < 0 || lda < (na > 1 ? na : 1) || ldb < (m > 1 ? m : 1) ||
        (side != HCGB_LEFT && side != HCGB_RIGHT) || (uplo != HCGB_LOWER && uplo != HCGB_UPPER) ||
        (trans != HCGB_NOTRANS && trans != HCGB_TRANS) || (diag != HCGB_NONUNIT && diag != HCGB_UNIT))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_trsm: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    if (m == 0 || n == 0) return HCGB_OK;
    launch_trsm(side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, ctx->stream);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_syrk(hcgb_context *ctx, int uplo, int trans, int n, int k, double alpha, const double *A, int lda,
                         double beta, double *C, int ldc) {
    if (!ctx) return HCGB_BAD_ARG;
    const int rows_a = trans ? k : n;
    if (!A || !C || n < 0 || k < 0 || lda < (rows_a > 1 ? rows_a : 1) || ldc < (n > 1 ? n : 1) ||
        (uplo != HCGB_LOWER && uplo != HCGB_UPPER) || (trans != HCGB_NOTRANS && trans != HCGB_TRANS))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_syrk: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    if (n == 0) return HCGB_OK;
    launch_syrk(uplo, trans, n, k, alpha, A, lda, beta, C, ldc, ctx->stream);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_fill_triangle(hcgb_context *ctx, int uplo, int n, double *A, int lda, double value) {
    if (!ctx) return HCGB_BAD_ARG;
    if (!A || n < 0 || lda < (n > 1 ? n : 1) || (uplo != HCGB_LOWER && uplo != HCGB_UPPER))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_fill_triangle: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    if (n == 0) return HCGB_OK;
    launch_fill_triangle(uplo, n, A, lda, value, ctx->stream);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

namespace {

int pack_common(hcgb_context *ctx, int count, const hcgb_tile *tiles, double *packed, long long *offsets,
                bool unpack) {
    if (!ctx) return HCGB_BAD_ARG;
    if (count < 0 || (count > 0 && (!tiles || !packed || !offsets)) || (count == 0 && !offsets))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_pack_tiles: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    if (count == 0) {
        HCGB_CUDA(ctx, cudaMemsetAsync(offsets, 0, sizeof(long long), ctx->stream));
        return HCGB_OK;
    }
    std::vector<DevTile> dv((size_t) count);
    for (int t = 0; t < count; t++) {
        int rc = check_tile(ctx, tiles[t], "tile");
        if (rc) return rc;
        dv[t] = to_dev(tiles[t]);
    }
    const size_t bytes = sizeof(DevTile) * dv.size();
    int rc = ensure_device(ctx, &ctx->pack_desc, &ctx->pack_desc_bytes, bytes);
    if (rc) return rc;
    if ((rc = ensure_stage(ctx, bytes))) return rc;
    std::memcpy(ctx->stage, dv.data(), bytes);
    HCGB_CUDA(ctx, cudaMemcpyAsync(ctx->pack_desc, ctx->stage, bytes, cudaMemcpyHostToDevice, ctx->stream));
    HCGB_CUDA(ctx, cudaEventRecord(ctx->stage_done, ctx->stream));
    launch_pack(static_cast<const DevTile *>(ctx->pack_desc), count, offsets, packed, unpack, ctx->stream);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

}  // namespace

extern "C" int hcgb_pack_tiles(hcgb_context *ctx, int count, const hcgb_tile *tiles, double *packed_dev,
                               long long *offsets_dev) {
    return pack_common(ctx, count, tiles, packed_dev, offsets_dev, false);
}

extern "C" int hcgb_unpack_tiles(hcgb_context *ctx, int count, const hcgb_tile *tiles, const double *packed_dev,
                                 long long *offsets_dev) {
    return pack_common(ctx, count, tiles, const_cast<double *>(packed_dev), offsets_dev, true);
}

extern "C" int hcgb_tile_cholesky(hcgb_context *ctx, int nt, const hcgb_tile *grid, const hcgb_params *params,
                                  int *info, hcgb_update_info *info_dev) {
    if (!ctx) return HCGB_BAD_ARG;
    if (nt <= 0 || !grid) return fail(ctx, HCGB_BAD_ARG, "hcgb_tile_cholesky: bad grid");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    const int nb = grid[0].rows;
    for (int j = 0; j < nt; j++)
        for (int i = j; i < nt; i++) {
            const hcgb_tile &t = grid[i + (size_t) j * nt];
            int rc;
            if ((rc = check_tile(ctx, t, "A"))) return rc;
            const bool want = i == j ? t.kind == HCGB_DENSE : t.kind == HCGB_COMPRESSED_VT;
            if (!want || t.rows != nb || t.cols != nb)
                return fail(ctx, HCGB_BAD_ARG,
                            "hcgb_tile_cholesky: nb x nb tiles, dense on the diagonal, compressed_vt below");
        }
    if (info) *info = 0;
    int *dinfo = nullptr;
    DevTile *dpanel = nullptr;
    HCGB_CUDA(ctx, cudaMalloc(&dinfo, sizeof(int) * (size_t) nt));
    if (cudaMalloc(&dpanel, sizeof(DevTile) * (size_t) nt) != cudaSuccess) {
        cudaFree(dinfo);
        return fail(ctx, HCGB_CUDA_ERROR, "hcgb_tile_cholesky: cudaMalloc failed");
    }
    auto done = [&](int rc) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(dinfo);
        cudaFree(dpanel);
        return rc;
    };
    const Params p = to_params(params, ctx);
    const int max_chunk = 1024;  // updates per pipeline launch (bounds the workspace)
    int uid = 0;
    auto tile = [&](int i, int j) -> const hcgb_tile & { return grid[i + (size_t) j * nt]; };
    for (int k = 0; k < nt; k++) {
        // Syrk leaves the strict upper triangle of a diagonal tile zero (HCore.cpp:555-563).
        if (k > 0) launch_fill_triangle(HCGB_UPPER, nb, tile(k, k).data, nb, 0.0, ctx->stream);
        launch_potrf(tile(k, k).data, nb, nb, HCGB_LOWER, dinfo + k, ctx->stream);
        int h = 0;
        cudaError_t e = cudaMemcpyAsync(&h, dinfo + k, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return done(fail(ctx, HCGB_CUDA_ERROR, std::string("hcgb_tile_cholesky: ") +
                                                                     cudaGetErrorString(e)));
        if (h) {
            if (info) *info = k * nb + h;
            return done(HCGB_OK);
        }
        if (k == nt - 1) break;
        // Panel: W_ik <- L_kk^-1 W_ik for every i > k.
        std::vector<DevTile> panel;
        for (int i = k + 1; i < nt; i++) panel.push_back(to_dev(tile(i, k)));
        HCGB_CUDA(ctx, cudaMemcpyAsync(dpanel, panel.data(), sizeof(DevTile) * panel.size(), cudaMemcpyHostToDevice,
                                       ctx->stream));
        launch_trsm_panel(tile(k, k).data, nb, nb, dpanel, (int) panel.size(), ctx->stream);
        HCGB_CUDA(ctx, cudaGetLastError());
        // Trailing updates A_ij -= A_ik A_jk^T (j <= i): Syrk on the diagonal, Gemm(aCholesky) below.
        // B = A_jk^T is the stored compressed_vt tile with its factors swapped (U' = W, W' = U).
        std::vector<hcgb_update> hu;
        std::vector<DevUpdate> dv;
        for (int i = k + 1; i < nt; i++)
            for (int j = k + 1; j <= i; j++) {
                const hcgb_tile &ta = tile(i, k), &tb = tile(j, k), &tc = tile(i, j);
                hcgb_tile tbt = tb;
                tbt.rows = tb.cols;
                tbt.cols = tb.rows;
                hu.push_back(hcgb_update{ta, tbt, tc});
                DevTile db = to_dev(tb);
                std::swap(db.data, db.v);
                std::swap(db.rows, db.cols);
                dv.push_back(DevUpdate{to_dev(ta), db, to_dev(tc), uid++, i - j});
            }
        const int chunk = updates_per_launch(ctx, shape_of(hu.data(), (int) hu.size()), p.mode, max_chunk);
        for (size_t off = 0; off < dv.size(); off += chunk) {
            const int n = (int) std::min<size_t>(chunk, dv.size() - off);
            std::vector<DevUpdate> part(dv.begin() + off, dv.begin() + off + n);
            BatchShape sh = shape_of(hu.data() + off, n);
            Workspace ws;
            int rc = prepare_workspace(ctx, sh, n, false, &ws, p.mode);
            if (rc) return done(rc);
            DevUpdate *dups;
            GemmJob *djobs;
            int *dsched;
            if ((rc = upload_updates(ctx, part, &dups, &djobs, &dsched))) return done(rc);
            launch_pipeline(ctx, ctx->stream, dups, djobs, dsched, n, -1.0, 1.0, ws, sh, p, info_dev);
            HCGB_CUDA(ctx, cudaGetLastError());
        }
    }
    return done(HCGB_OK);
}

// ---------------------------------------------------------------------------------------------
// Rank predictor of the learned form (no counterpart in the reference).
// ---------------------------------------------------------------------------------------------
extern "C" int hcgb_rank_model_create(hcgb_context *ctx, unsigned long long seed, hcgb_rank_model **out) {
    if (!ctx || !out) return HCGB_BAD_ARG;
    *out = nullptr;
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    auto *m = new hcgb_rank_model();
    m->m.device = ctx->device;
    const int rc = m->m.init(seed);
    if (rc) {
        m->m.release();
        delete m;
        return fail(ctx, rc, "hcgb_rank_model_create: device allocation failed");
    }
    *out = m;
    return HCGB_OK;
}

extern "C" int hcgb_rank_model_destroy(hcgb_rank_model *m) {
    if (!m) return HCGB_BAD_ARG;
    cudaSetDevice(m->m.device);
    cudaDeviceSynchronize();
    m->m.release();
    delete m;
    return HCGB_OK;
}

extern "C" int hcgb_rank_model_params(hcgb_rank_model *m, float *host_out, const float *host_in) {
    if (!m) return HCGB_BAD_ARG;
    if (cudaSetDevice(m->m.device) != cudaSuccess) return HCGB_CUDA_ERROR;
    int rc = HCGB_OK;
    if (host_in) rc = m->m.set_params(host_in);
    if (!rc && host_out) rc = m->m.get_params(host_out);
    return rc;
}

extern "C" int hcgb_rank_model_predict(hcgb_context *ctx, hcgb_rank_model *m, int n, const float *features_dev,
                                       float *out_dev) {
    if (!ctx || !m || n < 0 || (n > 0 && (!features_dev || !out_dev)))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_rank_model_predict: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    launch_mlp_forward(m->m, features_dev, n, out_dev, ctx->stream);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_rank_model_gradient(hcgb_context *ctx, hcgb_rank_model *m, int n, const float *features_dev,
                                        const float *targets_dev, float *grad_host, double *loss) {
    if (!ctx || !m || n <= 0 || !features_dev || !targets_dev || !grad_host)
        return fail(ctx, HCGB_BAD_ARG, "hcgb_rank_model_gradient: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    double *dloss = nullptr;
    HCGB_CUDA(ctx, cudaMalloc(&dloss, sizeof(double)));
    cudaMemsetAsync(dloss, 0, sizeof(double), ctx->stream);
    cudaMemsetAsync(m->m.grad, 0, sizeof(float) * MLP_PARAMS, ctx->stream);
    launch_mlp_grad(m->m, features_dev, targets_dev, nullptr, 0, n, 1.0f / (float) n, dloss, ctx->stream);
    double h = 0.0;
    cudaError_t e = cudaMemcpyAsync(grad_host, m->m.grad, sizeof(float) * MLP_PARAMS, cudaMemcpyDeviceToHost,
                                    ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, dloss, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->m.grad, 0, sizeof(float) * MLP_PARAMS, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(dloss);
    if (e != cudaSuccess) return fail(ctx, HCGB_CUDA_ERROR, std::string("hcgb_rank_model_gradient: ") + cudaGetErrorString(e));
    if (loss) *loss = h / n;
    return HCGB_OK;
}

extern "C" int hcgb_rank_model_train(hcgb_context *ctx, hcgb_rank_model *m, int n, const float *features_dev,
                                     const hcgb_update_info *records_dev, int epochs, int batch, float lr,
                                     unsigned long long seed, double *final_loss, int *samples) {
    if (!ctx || !m || n <= 0 || !features_dev || !records_dev || epochs < 0 || batch <= 0 || !(lr > 0.f))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_rank_model_train: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    float *T = nullptr;
    int *keep = nullptr, *idx = nullptr;
    double *dloss = nullptr;
    auto done = [&](int rc) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(T);
        cudaFree(keep);
        cudaFree(idx);
        cudaFree(dloss);
        return rc;
    };
    if (cudaMalloc(&T, sizeof(float) * n) != cudaSuccess || cudaMalloc(&keep, sizeof(int) * n) != cudaSuccess ||
        cudaMalloc(&idx, sizeof(int) * n) != cudaSuccess || cudaMalloc(&dloss, sizeof(double)) != cudaSuccess)
        return done(fail(ctx, HCGB_CUDA_ERROR, "hcgb_rank_model_train: cudaMalloc failed"));
    launch_targets_from_records(records_dev, n, T, keep, ctx->stream);
    std::vector<int> hk((size_t) n);
    if (cudaMemcpyAsync(hk.data(), keep, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return done(fail(ctx, HCGB_CUDA_ERROR, "hcgb_rank_model_train: record read failed"));
    std::vector<int> rows;
    for (int i = 0; i < n; i++)
        if (hk[i]) rows.push_back(i);
    const int cnt = (int) rows.size();
    if (samples) *samples = cnt;
    if (cnt == 0) return done(fail(ctx, HCGB_BAD_ARG, "hcgb_rank_model_train: no recompressed update in the records"));
    unsigned long long st = seed * 2862933555777941757ULL + 3037000493ULL;
    double last = 0.0;
    for (int ep = 0; ep < epochs; ep++) {
        // Fisher-Yates shuffle of the rows (64-bit LCG), then minibatches in that order.
        for (int i = cnt - 1; i > 0; i--) {
            st = st * 6364136223846793005ULL + 1442695040888963407ULL;
            const int j = (int) ((st >> 33) % (unsigned long long) (i + 1));
            std::swap(rows[i], rows[j]);
        }
        if (cudaMemcpyAsync(idx, rows.data(), sizeof(int) * cnt, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
            return done(fail(ctx, HCGB_CUDA_ERROR, "hcgb_rank_model_train: upload failed"));
        cudaMemsetAsync(dloss, 0, sizeof(double), ctx->stream);
        for (int off = 0; off < cnt; off += batch) {
            const int bs = cnt - off < batch ? cnt - off : batch;
            launch_mlp_grad(m->m, features_dev, T, idx, off, bs, 1.0f / (float) bs, dloss, ctx->stream);
            launch_adam(m->m, lr, ctx->stream);
        }
        double h = 0.0;
        if (cudaMemcpyAsync(&h, dloss, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess)
            return done(fail(ctx, HCGB_CUDA_ERROR, "hcgb_rank_model_train: training step failed"));
        last = h / cnt;
    }
    if (final_loss) *final_loss = last;
    return done(HCGB_OK);
}

extern "C" int hcgb_set_rank_model(hcgb_context *ctx, hcgb_rank_model *m, int policy) {
    if (!ctx || policy < 0 || policy > 1) return HCGB_BAD_ARG;
    if (m && m->m.device != ctx->device) return fail(ctx, HCGB_BAD_ARG, "hcgb_set_rank_model: model on another device");
    ctx->model = m;
    ctx->sk_policy = policy;
    ctx->learned = policy == 1 || m != nullptr;
    return HCGB_OK;
}

extern "C" int hcgb_set_feature_sink(hcgb_context *ctx, float *features_dev) {
    if (!ctx) return HCGB_BAD_ARG;
    ctx->feature_sink = features_dev;
    return HCGB_OK;
}

// ---------------------------------------------------------------------------------------------
// Per-matrix operations behind the HCoreKernels<double> backend (hcorepp_gb300/backend).
// ---------------------------------------------------------------------------------------------
namespace {

bool bad_ld(int ld, int rows) { return ld < (rows > 1 ? rows : 1); }

}  // namespace

extern "C" int hcgb_dgemm(hcgb_context *ctx, int transa, int transb, int m, int n, int k, double alpha,
                          const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc) {
    if (!ctx) return HCGB_BAD_ARG;
    if (m < 0 || n < 0 || k < 0 || (transa != 0 && transa != 1) || (transb != 0 && transb != 1) ||
        (m > 0 && n > 0 && (!C || bad_ld(ldc, m))) ||
        (m > 0 && n > 0 && k > 0 && (!A || !B || bad_ld(lda, transa ? k : m) || bad_ld(ldb, transb ? n : k))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dgemm: bad arguments");
    if (m == 0 || n == 0) return HCGB_OK;
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    GemmJob j{};
    j.A = A;
    j.B = B;
    j.C = C;
    j.M = m;
    j.N = n;
    j.K = k;
    j.lda = lda > 0 ? lda : 1;
    j.ldb = ldb > 0 ? ldb : 1;
    j.ldc = ldc;
    j.opA = transa;
    j.opB = transb;
    j.alpha = alpha;
    j.beta = beta;
    j.oz = (ctx->oz && oz_shape(m, n, k, ctx->oz_min)) ? 1 : 0;
    const size_t jb = (sizeof(GemmJob) + 255) / 256 * 256;
    int rc = ensure_device(ctx, &ctx->desc, &ctx->desc_bytes, jb + sizeof(int) * 16);
    if (rc) return rc;
    if ((rc = ensure_stage(ctx, sizeof(GemmJob)))) return rc;
    std::memcpy(ctx->stage, &j, sizeof(GemmJob));
    auto *dj = static_cast<GemmJob *>(ctx->desc);
    HCGB_CUDA(ctx, cudaMemcpyAsync(dj, ctx->stage, sizeof(GemmJob), cudaMemcpyHostToDevice, ctx->stream));
    HCGB_CUDA(ctx, cudaEventRecord(ctx->stage_done, ctx->stream));
    launch_gemm_jobs(dj, 1, reinterpret_cast<int *>(static_cast<char *>(ctx->desc) + jb), ctx->stream);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_dcopy2d(hcgb_context *ctx, int trans, int m, int n, double alpha, const double *A, int lda,
                            double *B, int ldb) {
    if (!ctx) return HCGB_BAD_ARG;
    if (m < 0 || n < 0 || (m > 0 && n > 0 && (!A || !B || bad_ld(ldb, m) || bad_ld(lda, trans ? n : m))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dcopy2d: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    be_copy(ctx->stream, trans ? 1 : 0, m, n, alpha, A, lda, B, ldb);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_dlacpy(hcgb_context *ctx, int part, int m, int n, const double *A, int lda, double *B, int ldb) {
    if (!ctx) return HCGB_BAD_ARG;
    if (part < 0 || part > 2 || m < 0 || n < 0 || (m > 0 && n > 0 && (!A || !B || bad_ld(lda, m) || bad_ld(ldb, m))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dlacpy: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    be_lacpy(ctx->stream, part, m, n, A, lda, B, ldb);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_dlaset(hcgb_context *ctx, int part, int m, int n, double offdiag, double diag, double *A, int lda) {
    if (!ctx) return HCGB_BAD_ARG;
    if (part < 0 || part > 3 || m < 0 || n < 0 || (m > 0 && n > 0 && (!A || bad_ld(lda, m))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dlaset: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    be_laset(ctx->stream, part, m, n, offdiag, diag, A, lda);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_dscale_rows(hcgb_context *ctx, int rows, int cols, const double *s, double *A, int lda) {
    if (!ctx) return HCGB_BAD_ARG;
    if (rows < 0 || cols < 0 || (rows > 0 && cols > 0 && (!s || !A || bad_ld(lda, rows))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dscale_rows: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    be_scale_rows(ctx->stream, rows, cols, s, A, lda);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_dsymmetrize(hcgb_context *ctx, int uplo, int n, double *A, int lda) {
    if (!ctx) return HCGB_BAD_ARG;
    if ((uplo != HCGB_LOWER && uplo != HCGB_UPPER) || n < 0 || (n > 0 && (!A || bad_ld(lda, n))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dsymmetrize: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    be_symmetrize(ctx->stream, uplo == HCGB_UPPER ? 1 : 2, n, A, lda);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_dgeqrf(hcgb_context *ctx, int m, int n, double *A, int lda, double *tau) {
    if (!ctx) return HCGB_BAD_ARG;
    if (m < 0 || n < 0 || (m > 0 && n > 0 && (!A || !tau || bad_ld(lda, m))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dgeqrf: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    be_geqr2(ctx->stream, m, n, A, lda, tau);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_dorgqr(hcgb_context *ctx, int m, int n, int k, double *A, int lda, const double *tau) {
    if (!ctx) return HCGB_BAD_ARG;
    if (m < 0 || n < 0 || n > m || k < 0 || k > n || (m > 0 && n > 0 && (!A || bad_ld(lda, m) || (k > 0 && !tau))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dorgqr: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    be_org2r(ctx->stream, m, n, k, A, lda, tau);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_dormqr(hcgb_context *ctx, int side, int trans, int m, int n, int k, const double *A, int lda,
                           const double *tau, double *C, int ldc) {
    if (!ctx) return HCGB_BAD_ARG;
    const int nq = side == HCGB_LEFT ? m : n;
    if ((side != HCGB_LEFT && side != HCGB_RIGHT) || (trans != HCGB_NOTRANS && trans != HCGB_TRANS) || m < 0 ||
        n < 0 || k < 0 || k > nq || (m > 0 && n > 0 && k > 0 && (!A || !tau || !C || bad_ld(lda, nq) || bad_ld(ldc, m))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dormqr: bad arguments");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    be_orm2r(ctx->stream, side == HCGB_LEFT, trans == HCGB_TRANS, m, n, k, A, lda, tau, C, ldc);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_dtrmm(hcgb_context *ctx, int side, int uplo, int trans, int diag, int m, int n, double alpha,
                          const double *A, int lda, double *B, int ldb) {
    if (!ctx) return HCGB_BAD_ARG;
    const int na = side == HCGB_LEFT ? m : n;
    if ((side != HCGB_LEFT && side != HCGB_RIGHT) || (uplo != HCGB_LOWER && uplo != HCGB_UPPER) ||
        (trans != HCGB_NOTRANS && trans != HCGB_TRANS) || (diag != HCGB_NONUNIT && diag != HCGB_UNIT) || m < 0 ||
        n < 0 || (m > 0 && n > 0 && (!A || !B || bad_ld(lda, na) || bad_ld(ldb, m))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dtrmm: bad arguments");
    if (m == 0 || n == 0) return HCGB_OK;
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    int rc = ensure_device(ctx, &ctx->be_scratch, &ctx->be_scratch_bytes, sizeof(double) * (size_t) m * n);
    if (rc) return rc;
    double *T = static_cast<double *>(ctx->be_scratch);
    be_lacpy(ctx->stream, 0, m, n, B, ldb, T, m);
    be_trmm(ctx->stream, side == HCGB_LEFT, uplo == HCGB_UPPER, trans == HCGB_TRANS, diag == HCGB_UNIT, m, n, alpha, A,
            lda, T, B, ldb);
    HCGB_CUDA(ctx, cudaGetLastError());
    return HCGB_OK;
}

extern "C" int hcgb_dgesvd(hcgb_context *ctx, int jobu, int jobvt, int m, int n, double *A, int lda, double *S,
                           double *U, int ldu, double *VT, int ldvt, int *info) {
    if (!ctx) return HCGB_BAD_ARG;
    const int kk = m < n ? m : n;
    const bool wu = jobu != HCGB_SVD_NONE, wv = jobvt != HCGB_SVD_NONE;
    if (jobu < 0 || jobu > 2 || jobvt < 0 || jobvt > 2 || m < 0 || n < 0 || (m > 0 && n > 0 && (!A || !S || bad_ld(lda, m))) ||
        (wu && m > 0 && (!U || bad_ld(ldu, m))) || (wv && n > 0 && (!VT || bad_ld(ldvt, jobvt == HCGB_SVD_ALL ? n : kk))))
        return fail(ctx, HCGB_BAD_ARG, "hcgb_dgesvd: bad arguments");
    if ((jobu == HCGB_SVD_ALL && m > n) || (jobvt == HCGB_SVD_ALL && n > m))
        return fail(ctx, HCGB_UNSUPPORTED, "hcgb_dgesvd: full U of a tall or full V^T of a wide matrix");
    if (info) *info = 0;
    if (m == 0 || n == 0) return HCGB_OK;
    if (kk > 1024) return fail(ctx, HCGB_UNSUPPORTED, "hcgb_dgesvd: min(m, n) > 1024");
    HCGB_CUDA(ctx, cudaSetDevice(ctx->device));
    // Jacobi on X = A (m >= n) or X = A^T (m < n): rows >= cols = kk.
    const bool tr = m < n;
    const int rows = tr ? n : m;
    const size_t need = sizeof(double) * ((size_t) kk * kk + (tr ? (size_t) rows * kk : 0)) + 256;
    int rc = ensure_device(ctx, &ctx->be_scratch, &ctx->be_scratch_bytes, need + sizeof(int) * 4);
    if (rc) return rc;
    double *V = static_cast<double *>(ctx->be_scratch);
    double *X = A;
    int ldx = lda;
    if (tr) {
        X = V + (size_t) kk * kk;
        ldx = rows;
        be_copy(ctx->stream, 1, rows, kk, 1.0, A, lda, X, ldx);
    }
    int *dsw = reinterpret_cast<int *>(static_cast<char *>(ctx->be_scratch) + need);
    be_jacobi_svd(ctx->stream, rows, kk, X, ldx, V, kk, 2.2204460492503131e-16 * std::sqrt((double) rows), dsw);
    be_svd_finish(ctx->stream, rows, kk, X, ldx, V, kk, S, U, ldu, VT, ldvt, kk, wu ? 1 : 0, wv ? 1 : 0, tr ? 1 : 0);
    int sw = 0;
    HCGB_CUDA(ctx, cudaMemcpyAsync(&sw, dsw, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    HCGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (sw < 0) {
        if (info) *info = 1;
        return fail(ctx, HCGB_NOT_CONVERGED, "hcgb_dgesvd: Jacobi sweep limit reached");
    }
    return HCGB_OK;
}

extern "C" int hcgb_set_graph(hcgb_context *ctx, int enable) {
    if (!ctx || (enable != 0 && enable != 1)) return HCGB_BAD_ARG;
    ctx->graph_mode = enable != 0;
    if (!enable && ctx->graph_exec) {
        cudaStreamSynchronize(ctx->stream);
        cudaGraphExecDestroy(ctx->graph_exec);
        ctx->graph_exec = nullptr;
        ctx->graph_key.clear();
    }
    return HCGB_OK;
}

extern "C" int hcgb_set_tuning(hcgb_context *ctx, int oz_min_outputs, int wy_min_reflectors) {
    if (!ctx || oz_min_outputs < 1 || wy_min_reflectors < 1) return HCGB_BAD_ARG;
    ctx->oz_min = oz_min_outputs;
    ctx->wy_min = wy_min_reflectors;
    return HCGB_OK;
}

extern "C" int hcgb_set_sketch_limit(hcgb_context *ctx, int percent) {
    if (!ctx || percent < 0 || percent > 100) return HCGB_BAD_ARG;
    ctx->sk_pct = percent ? percent : SKETCH_MAX_PCT;
    return HCGB_OK;
}

extern "C" int hcgb_set_precond(hcgb_context *ctx, int min_cols) {
    if (!ctx || min_cols < 0) return HCGB_BAD_ARG;
    ctx->precond_min = min_cols ? min_cols : PRECOND_MIN_COLS;
    return HCGB_OK;
}
