// hcgb_tile_gemm_noalloc: one tile update that allocates nothing.
//
// Who needs it: code that runs where it may not allocate device memory of its own.  Task
// runtimes that move tiles between workers (the StarPU/PaRSEC-style runtimes HCore++ tiles are
// designed for) own the device memory and call a codelet with buffers they already placed; a
// codelet that calls cudaMalloc there competes with the runtime's allocator, and cudaMalloc /
// cudaFree can synchronise the device in the middle of other workers' kernels.  Real-time or
// embedded callers may also forbid allocation after start-up.  This entry point takes the
// caller's tile buffers and stream and uses only a fixed scratch array that is part of the
// library image.
//
// The scratch: a file-scope __device__ array of HCGB_NOALLOC_SCRATCH_DOUBLES doubles (8 MiB).
// Every GPU that loads the library holds one copy of it until the process exits.  All calls on
// a device share it, so calls that overlap on the GPU (different streams, or host threads that
// do not order their streams) race on it: order such calls yourself.  Nothing in it has to
// start at zero: every call writes each scratch region before it reads it.
//
// Host code never dereferences `g_noalloc_scratch`: on the host that name is a stand-in, not a
// device address.  The device address is obtained once per device with cudaGetSymbolAddress,
// with that device current, on the first call made on that device; make that first call
// before any stream capture begins.  The address is kept for the life of the process, so a
// device reset (cudaDeviceReset, which unloads the module) after the first call is not
// supported: the kept address would then be stale.
#include <cstring>
#include <mutex>

#include "internal.cuh"

namespace hcgb {

namespace {

constexpr size_t HCGB_NOALLOC_SCRATCH_DOUBLES = size_t(1) << 20;  // 8 MiB
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_scratch[HCGB_NOALLOC_SCRATCH_DOUBLES];

std::mutex g_setup_mutex;
void *g_scratch_addr[MAX_DEVICES] = {nullptr};

// Copies the update descriptor (passed by value) into the scratch array.
__global__ void noalloc_set_update(DevUpdate *dst, DevUpdate u) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = u;
}

int scratch_address(int device, double **out) {
    if (device < 0 || device >= MAX_DEVICES) return HCGB_BAD_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        // The current device is `device` here (the caller's stream belongs to it).
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return HCGB_CUDA_ERROR;
        g_scratch_addr[device] = p;
    }
    *out = static_cast<double *>(g_scratch_addr[device]);
    return HCGB_OK;
}

size_t round_up_bytes(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

}  // namespace hcgb

using namespace hcgb;

extern "C" int hcgb_tile_gemm_noalloc(double alpha, const hcgb_tile *a, const hcgb_tile *b, double beta,
                                      hcgb_tile *c, const hcgb_params *params, void *stream,
                                      hcgb_update_info *info_dev) {
    if (!a || !b || !c) return HCGB_BAD_ARG;
    const hcgb_tile *tiles[3] = {a, b, c};
    for (const hcgb_tile *t : tiles) {
        if (!t->data || t->rows <= 0 || t->cols <= 0) return HCGB_BAD_ARG;
        if (t->kind != HCGB_DENSE && t->kind != HCGB_COMPRESSED) return HCGB_BAD_ARG;
        if (t->kind == HCGB_COMPRESSED && (!t->rank || t->max_rank <= 0)) return HCGB_BAD_ARG;
    }
    if (a->cols != b->rows || a->rows != c->rows || b->cols != c->cols) return HCGB_BAD_ARG;
    const bool ak = a->kind == HCGB_COMPRESSED, bk = b->kind == HCGB_COMPRESSED, ck = c->kind == HCGB_COMPRESSED;
    if (!ak && !bk && ck) return HCGB_UNSUPPORTED;  // DDC re-shapes the tile: hcgb_tile_gemm only
    if (params && params->mode != HCGB_PLAIN_FP64 && params->mode != HCGB_MIXED)
        return HCGB_UNSUPPORTED;  // the low-precision forms apply Q in WY form: hcgb_tile_gemm only

    // Scratch layout for this update, same as one slot of the batched path.
    const int ra = ak ? a->max_rank : 0, rb = bk ? b->max_rank : 0, rc = ck ? c->max_rank : 0;
    int ld = c->rows;
    if (c->cols > ld) ld = c->cols;
    if (a->cols > ld) ld = a->cols;
    ld = (ld + 7) / 8 * 8;
    int rmax = ra > rb ? ra : rb;
    if (rmax < 8) rmax = 8;
    int kmax = 8;
    if (ck) kmax = rc + (ak && bk ? rmax : (bk ? rb : ra));
    if (kmax < 8) kmax = 8;
    Workspace ws = make_workspace_layout(ld, kmax, rmax, false);
    ws.order = nullptr;  // a single update: no ordering
    const size_t slot_bytes = round_up_bytes(sizeof(double) * ws.slot_doubles);
    const size_t meta_bytes = round_up_bytes(sizeof(int) * META_INTS);
    const size_t desc_bytes = round_up_bytes(sizeof(DevUpdate));
    const size_t job_bytes = round_up_bytes(sizeof(GemmJob) * 3);
    const size_t sched_bytes = round_up_bytes(sizeof(int) * 8);  // three tile lists of one job
    if (slot_bytes + meta_bytes + desc_bytes + job_bytes + sched_bytes > sizeof(double) * HCGB_NOALLOC_SCRATCH_DOUBLES)
        return HCGB_POOL_TOO_SMALL;
    // The QR panels and the core's bookkeeping live in shared memory: the same per-CTA limit as the
    // allocating entry points, checked before anything is launched so that C stays untouched.
    const size_t smem_limit = 227 * 1024;
    if (ck && (qr_smem_bytes(ld, kmax) > smem_limit || svd_smem_bytes(kmax) > smem_limit))
        return HCGB_POOL_TOO_SMALL;

    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return HCGB_CUDA_ERROR;
    double *scratch = nullptr;
    int rcode = scratch_address(device, &scratch);
    if (rcode != HCGB_OK) return rcode;
    char *p = reinterpret_cast<char *>(scratch);
    ws.base = reinterpret_cast<double *>(p);
    ws.meta = reinterpret_cast<int *>(p + slot_bytes);
    auto *dup = reinterpret_cast<DevUpdate *>(p + slot_bytes + meta_bytes);
    auto *jobs = reinterpret_cast<GemmJob *>(p + slot_bytes + meta_bytes + desc_bytes);
    auto *sched = reinterpret_cast<int *>(p + slot_bytes + meta_bytes + desc_bytes + job_bytes);

    auto dev_tile = [](const hcgb_tile *t) {
        DevTile d;
        d.data = t->data;
        d.rank = t->rank;
        d.rows = t->rows;
        d.cols = t->cols;
        d.max_rank = t->kind == HCGB_COMPRESSED ? t->max_rank : 0;
        d.kind = t->kind == HCGB_COMPRESSED ? 1 : 0;
        d.v = t->kind == HCGB_COMPRESSED ? t->data + (size_t) t->rows * t->max_rank : nullptr;
        return d;
    };
    DevUpdate u{dev_tile(a), dev_tile(b), dev_tile(c), 0};
    Params prm;
    prm.accuracy = params ? params->accuracy : 1e-9;
    prm.truncated = params ? params->truncated_svd : 0;
    prm.fixed_rank = params ? params->fixed_rank : 0;
    prm.side_mode = 1;
    prm.mode = params ? params->mode : 0;
    prm.oz = 1;
    prm.oz_min = OZ_MIN_OUTPUTS;
    prm.wy_min = WY_MIN_REFLECTORS;
    prm.precond_min = PRECOND_MIN_COLS;
    prm.sk_pct = SKETCH_MAX_PCT;

    // GEMM grid bounds from the tile kinds and capacities (ranks are read on the device).
    int pm[3] = {0, 0, 0}, pn[3] = {0, 0, 0};
    const int m = c->rows, n = c->cols;
    if (ck) {
        if (ak && bk) {
            pm[0] = ra; pn[0] = rb;
            pm[1] = m > n ? m : n; pn[1] = rmax;
        } else if (bk) {
            pm[0] = m; pn[0] = rb;
        } else {
            pm[0] = n; pn[0] = ra;
        }
    } else {
        if (ak && bk) {
            pm[0] = ra; pn[0] = rb;
            pm[1] = ra > m ? ra : m; pn[1] = n > rb ? n : rb;
        } else if (bk) {
            pm[0] = m; pn[0] = rb;
        } else if (ak) {
            pm[0] = ra; pn[0] = n;
        }
        pm[2] = m; pn[2] = n;
    }

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    { noalloc_set_update<<<1, 32, 0, st>>>(dup, u); note_launch(); }
    launch_plan(dup, 1, alpha, beta, ws, prm, jobs, st);
    if (ck) launch_stack(dup, 1, alpha, beta, ws, st);
    for (int ph = 0; ph < 3; ph++)
        if (pm[ph] > 0 && pn[ph] > 0) launch_gemm_jobs(jobs + ph, 1, sched, st);
    if (ck) {
        launch_qr(ws, 1, prm.mode == 1, st);
        launch_core_svd(dup, 1, ws, prm, st);
        launch_apply_q(dup, 1, ws, prm.mode == 1, st);
    }
    launch_finalize(dup, 1, ws, info_dev, st);
    return cudaGetLastError() == cudaSuccess ? HCGB_OK : HCGB_CUDA_ERROR;
}
