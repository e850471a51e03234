// FP64 factor products on the fifth-generation tensor cores by error-free splitting (the Ozaki
// scheme), with tcgen05.mma (kind::f16, FP32 accumulation in tensor memory).
//
// The GB300's FP64 pipe (SIMT or DMMA) delivers ~1.1 TFLOP/s, its FP16 tensor cores ~2 PFLOP/s.
// A product C = op(A) op(B) is computed exactly enough for FP64 work as follows:
//   * every row i of op(A) gets the exponent e_i with max_k |A_ik| < 2^e_i, every column j of
//     op(B) the exponent f_j with max_k |B_kj| < 2^f_j;
//   * each element becomes a 56-bit fixed-point integer relative to its group's exponent (rounded
//     to nearest; the rounding error is 2^-57 of the group maximum) and is cut into S = 8 balanced
//     base-128 digits, A = sum_s 2^(e_i - 7 (s + 1)) A^(s), |A^(s)| <= 64 for s > 0 and <= 128 for
//     s = 0, all exact in FP16;
//   * the plane products A^(s) B^(t) are integers; the pairs of one level L = s + t (at most 8
//     per k, each below 2^13 but the (0, 0) one) sum to less than 2^15 per k, so over 128 k the
//     FP32 accumulators of a level hold them exactly (< 2^22) and an FP32 add of 1.5 * 2^23 exposes
//     them as integers in the low mantissa bits;
//   * levels L = s + t <= S - 1 are kept (36 plane pairs; the dropped ones are below 2^-56 of
//     max|A_i| max|B_j| per k, under FP64's own worst-case bound); every 128 k the eight level
//     accumulators are read out of tensor memory and added into two 64-bit integers (levels 0-3 and
//     4-7, each shifted to a common scale), which stay exact for k up to 2^16, and the tile ends with
//     C_ij = 2^(e_i + f_j) (hi 2^-35 + lo 2^-63).
// Tensor memory holds the eight level accumulators of a 128 x 64 output tile (512 columns); one
// thread issues the 72 MMAs (36 pairs x 2 k-steps of 16) of a 32-wide K chunk while the others cut
// the next chunk into digit planes in the second shared-memory stage.  The splitting and combining
// is integer work; an output element costs 4 FP64 instructions (two conversions, two scalings)
// plus the epilogue.
#include <cuda_fp16.h>

#include "internal.cuh"
#include "tcgen05.cuh"

namespace hcgb {

namespace {

constexpr int OZ_S = 8;                 // digit planes per operand
constexpr int OZ_B = 7;                 // bits per digit
constexpr int OZ_W = OZ_S * OZ_B;       // fixed-point width (56 bits)
static_assert(OZ_W >= 53, "the digit planes must cover a double's 53-bit significand");
constexpr int OZ_TM = 128, OZ_TN = 64;  // output tile per CTA (UMMA M = 128, N = 64)
constexpr int OZ_KC = 32;               // K elements per shared-memory stage (64 bytes per row and plane)
constexpr int OZ_KB = OZ_KC * 2 / 16;   // core matrices along K per stage (4)
constexpr int OZ_FLUSH = 4;             // stages per exact read-out of the level accumulators (128 k)
constexpr int OZ_THREADS = 256;         // 8 warps
constexpr int OZ_A_PLANE = OZ_TM * OZ_KC * 2;   // 8 KB
constexpr int OZ_B_PLANE = OZ_TN * OZ_KC * 2;   // 4 KB
constexpr int OZ_STAGE = OZ_S * (OZ_A_PLANE + OZ_B_PLANE);  // 96 KB
constexpr int OZ_SMEM = 2 * OZ_STAGE + 1024;
constexpr int OZ_TMEM_COLS = OZ_S * OZ_TN;  // 512: one 64-column accumulator per level
constexpr int OZ_NOGROUP = -1100;       // exponent of an all-zero group

__device__ unsigned int g_oz_wait_timeouts = 0;

// Biased exponent field of |x| (0 for zero and subnormals).
__device__ __forceinline__ int exp_field(double x) {
    return (int) ((__double_as_longlong(x) >> 52) & 0x7ff);
}

// Balanced digits of x relative to the group exponent e (|x| < 2^e): digit s has weight
// 2^(e - 7 (s + 1)), d[1..7] in [-64, 63], d[0] in [-128, 128].  Subnormals count as zero.
__device__ __forceinline__ void oz_digits(double x, int e, int (&d)[OZ_S]) {
    const long long bits = __double_as_longlong(x);
    const int E = (int) ((bits >> 52) & 0x7ff);
    long long u = 0;
    if (E != 0 && e > OZ_NOGROUP) {
        const long long M = (bits & 0xfffffffffffffLL) | (1LL << 52);
        const int sh = E - 1019 - e;  // x * 2^(56 - e) = M * 2^sh, sh <= 3
        if (sh >= 0) u = M << sh;
        else if (sh > -64) u = (M + (1LL << (-sh - 1))) >> (-sh);
    }
    long long v = bits < 0 ? -u : u;
#pragma unroll
    for (int s = OZ_S - 1; s > 0; s--) {
        long long r = v & 127;
        if (r >= 64) r -= 128;
        d[s] = (int) r;
        v = (v - r) >> OZ_B;
    }
    d[0] = (int) v;
}

// Byte offset of (row r, K element kk of the stage) inside one plane (core-matrix layout, 2-byte
// elements, OZ_KB core matrices along K).
__device__ __forceinline__ int oz_off(int r, int kk) {
    return ((r >> 3) * OZ_KB + (kk >> 3)) * 128 + (r & 7) * 16 + (kk & 7) * 2;
}

__device__ __forceinline__ uint32_t pack_h2(int lo, int hi) {
    const __half a = __int2half_rn(lo), b = __int2half_rn(hi);
    return (uint32_t) __half_as_ushort(a) | ((uint32_t) __half_as_ushort(b) << 16);
}

// 2^ex as a double (0 below the normal range).
__device__ __forceinline__ double pow2(int ex) {
    if (ex < -1022) return 0.0;
    if (ex > 1023) ex = 1023;
    return __hiloint2double((ex + 1023) << 20, 0);
}

// Cuts rows [0, R) x K elements [k0, k0 + 32) of op(X) (a = true: op(A) with the row exponents;
// false: op(B)^T with the column exponents) into the stage's digit planes, two K elements per
// 32-bit store.
template <bool IS_A>
__device__ void split_chunk(const GemmJob &jb, int base, int R, int k0, const int *ex, unsigned char *planes,
                            int plane_bytes) {
    constexpr int PAIRS = OZ_KC / 2;
    const bool kfast = IS_A ? jb.opA != 0 : jb.opB == 0;  // consecutive K contiguous in memory
    const int lim = IS_A ? jb.M : jb.N;
    for (int e = threadIdx.x; e < R * PAIRS; e += OZ_THREADS) {
        int r, kp;
        if (kfast) {
            kp = e % PAIRS;
            r = e / PAIRS;
        } else {
            r = e % R;
            kp = e / R;
        }
        const int g = base + r, k = k0 + 2 * kp;
        double v0 = 0.0, v1 = 0.0;
        if (g < lim) {
            if (IS_A) {
                if (k < jb.K) v0 = job_a(jb, g, k);
                if (k + 1 < jb.K) v1 = job_a(jb, g, k + 1);
            } else {
                if (k < jb.K) v0 = job_b(jb, k, g);
                if (k + 1 < jb.K) v1 = job_b(jb, k + 1, g);
            }
        }
        int d0[OZ_S], d1[OZ_S];
        oz_digits(v0, ex[r], d0);
        oz_digits(v1, ex[r], d1);
        const int off = oz_off(r, 2 * kp);
#pragma unroll
        for (int s = 0; s < OZ_S; s++)
            *reinterpret_cast<uint32_t *>(planes + s * plane_bytes + off) = pack_h2(d0[s], d1[s]);
    }
}

// One 128 x 64 output tile of one job.
__device__ void oz_tile(const GemmJob &jb, int tile, unsigned char *stage0, uint32_t tmem, uint32_t mbar0,
                        uint32_t (&phase)[2], bool (&pending)[2], int *ea, int *eb) {
    const int ntm = (jb.M + OZ_TM - 1) / OZ_TM;
    const int m0 = (tile % ntm) * OZ_TM, n0 = (tile / ntm) * OZ_TN;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr uint32_t IDESC = tc::instr_desc(tc::FMT_F16, OZ_TM, OZ_TN);

    // 1. Group exponents over all of K: PA threads per row of op(A), PB per column of op(B).
    {
        constexpr int PA = OZ_THREADS / OZ_TM, PB = OZ_THREADS / OZ_TN;
        const int gi = m0 + tid / PA, pa = tid % PA;
        int ma = 0;
        if (gi < jb.M)
            for (int k = pa; k < jb.K; k += PA) ma = max(ma, exp_field(job_a(jb, gi, k)));
#pragma unroll
        for (int o = 1; o < PA; o <<= 1) ma = max(ma, __shfl_xor_sync(0xffffffffu, ma, o));
        if (pa == 0) ea[tid / PA] = ma ? ma - 1022 : OZ_NOGROUP;
        const int gj = n0 + tid / PB, pb = tid % PB;
        int mb = 0;
        if (gj < jb.N)
            for (int k = pb; k < jb.K; k += PB) mb = max(mb, exp_field(job_b(jb, k, gj)));
#pragma unroll
        for (int o = 1; o < PB; o <<= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
        if (pb == 0) eb[tid / PB] = mb ? mb - 1022 : OZ_NOGROUP;
    }
    __syncthreads();

    // This thread's share of the read-out: TMEM lanes 32 (warp % 4) .. (rows), columns 32 (warp / 4) ..
    const int q = warp & 3, h = warp >> 2;
    long long hi[32], lo[32];  // levels 0-3 at scale 2^-35, levels 4-7 at scale 2^-63
#pragma unroll
    for (int j = 0; j < 32; j++) hi[j] = lo[j] = 0;
    bool ok = true;
    auto drain = [&]() {  // every committed MMA complete (each commit waited for exactly once)
        for (int b = 0; b < 2; b++)
            if (pending[b]) {
                ok &= tc::mbar_wait(mbar0 + 8 * b, phase[b]);
                phase[b] ^= 1;
                pending[b] = false;
            }
        tc::fence_after();
    };
    auto readout = [&]() {
#pragma unroll 1
        for (int l = 0; l < OZ_S; l++) {
            float v[32];
            tc::tmem_ld32(tmem + ((uint32_t) (q * 32) << 16) + (uint32_t) (l * OZ_TN + h * 32), v);
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const long long iv = (long long) (__float_as_int(v[j] + 12582912.0f) - 0x4B400000);
                if (l < 4) hi[j] += iv << (OZ_B * (3 - l));
                else lo[j] += iv << (OZ_B * (7 - l));
            }
        }
        tc::fence_before();
        __syncthreads();  // the next MMAs overwrite the accumulators only after every read-out
    };

    const int nchunks = (jb.K + OZ_KC - 1) / OZ_KC;
    for (int c = 0; c < nchunks; c++) {
        const int buf = c & 1;
        unsigned char *sa = stage0 + buf * OZ_STAGE, *sb = sa + OZ_S * OZ_A_PLANE;
        if (pending[buf]) {  // the MMAs of chunk c - 2 have read this stage
            ok &= tc::mbar_wait(mbar0 + 8 * buf, phase[buf]);
            phase[buf] ^= 1;
            pending[buf] = false;
        }
        split_chunk<true>(jb, m0, OZ_TM, c * OZ_KC, ea, sa, OZ_A_PLANE);
        split_chunk<false>(jb, n0, OZ_TN, c * OZ_KC, eb, sb, OZ_B_PLANE);
        tc::fence_smem_to_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            const uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
            const bool first = (c % OZ_FLUSH) == 0;  // accumulators restart after every read-out
#pragma unroll
            for (int ks = 0; ks < OZ_KC / 16; ks++)
#pragma unroll
                for (int s = 0; s < OZ_S; s++)
#pragma unroll
                    for (int t = 0; t < OZ_S - s; t++) {
                        const uint64_t ad = tc::smem_desc(a0 + s * OZ_A_PLANE + ks * 256, 128, OZ_KB * 128);
                        const uint64_t bd = tc::smem_desc(b0 + t * OZ_B_PLANE + ks * 256, 128, OZ_KB * 128);
                        // The first MMA into level L of a read-out window overwrites it: in this order
                        // that is the pair (0, L) of the window's first k-step.
                        const bool overwrite = first && ks == 0 && s == 0;
                        tc::mma_f16(tmem + (uint32_t) ((s + t) * OZ_TN), ad, bd, IDESC, overwrite ? 0u : 1u);
                    }
            tc::commit(mbar0 + 8 * buf);
        }
        pending[buf] = true;
        if ((c + 1) % OZ_FLUSH == 0 || c + 1 == nchunks) {
            drain();
            readout();
        }
    }
    if (!ok && tid == 0) atomicAdd(&g_oz_wait_timeouts, 1u);

    // Epilogue: C = alpha * product + beta * C, one row per thread, 32 columns.
    const int row_l = q * 32 + lane, row = m0 + row_l;
    if (row < jb.M) {
        const bool scale = jb.alpha != 1.0, accum = jb.beta != 0.0;
#pragma unroll
        for (int j = 0; j < 32; j++) {
            const int cl = h * 32 + j, col = n0 + cl;
            if (col < jb.N) {
                double *cp = jb.C + row + (size_t) col * jb.ldc;
                const int eab = ea[row_l] + eb[cl];
                double prod = 0.0;
                if (jb.K > 0) prod = fma((double) hi[j], pow2(eab - 35), (double) lo[j] * pow2(eab - 63));
                double v = scale ? jb.alpha * prod : prod;
                if (accum) v = fma(jb.beta, *cp, v);
                *cp = v;
            }
        }
    }
    __syncthreads();  // ea / eb are rewritten by the next tile
}

// Tiles of the jobs marked oz, compacted (sched: exclusive prefix of tiles per job, njobs + 1
// entries); a grid sized to the GPU strides over them.
__global__ void __launch_bounds__(OZ_THREADS, 1) oz_gemm_jobs_kernel(const GemmJob *jobs, int njobs, const int *sched) {
    extern __shared__ __align__(1024) unsigned char oz_smem_raw[];
    __shared__ __align__(8) unsigned long long mbar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int ea[OZ_TM], eb[OZ_TN];
    unsigned char *stage0 = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(oz_smem_raw) + 1023) & ~uintptr_t(1023));
    const int total = sched[njobs];
    if (blockIdx.x >= total) return;  // whole CTA leaves before any TMEM or barrier is set up
    const uint32_t mbar0 = tc::smem_u32(&mbar[0]);
    if (threadIdx.x == 0) {
        tc::mbar_init(mbar0, 1);
        tc::mbar_init(mbar0 + 8, 1);
    }
    if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(tc::smem_u32(&tmem_slot), OZ_TMEM_COLS);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    uint32_t phase[2] = {0u, 0u};
    bool pending[2] = {false, false};
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        int lo = 0, hi = njobs;  // sched[lo] <= w < sched[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (sched[mid] <= w) lo = mid;
            else hi = mid;
        }
        const GemmJob jb = jobs[lo];
        oz_tile(jb, w - sched[lo], stage0, tmem, mbar0, phase, pending, ea, eb);
    }
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tc::tmem_free(tmem, OZ_TMEM_COLS);
}

}  // namespace

void launch_oz_gemm_jobs(const GemmJob *jobs, int njobs, const int *sched, int sms, cudaStream_t st) {
    if (njobs <= 0) return;
    cudaFuncSetAttribute(oz_gemm_jobs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM);
    { oz_gemm_jobs_kernel<<<sms, OZ_THREADS, OZ_SMEM, st>>>(jobs, njobs, sched); note_launch(); }
}

unsigned int oz_wait_timeouts() {
    unsigned int v = 0;
    cudaMemcpyFromSymbol(&v, g_oz_wait_timeouts, sizeof(v));
    return v;
}

}  // namespace hcgb
