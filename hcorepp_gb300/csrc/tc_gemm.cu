// Factor products and Q-application products in TF32 or BF16 on the fifth-generation tensor
// cores (tcgen05.mma, FP32 accumulation in tensor memory), for the low-precision recompression
// forms.  Operands are FP64 in global memory; each row of op(A) and each column of op(B) is first
// scaled by an exact power of two so its largest entry lies in [1/2, 1) (per-row / per-column
// power-of-two scaling), rounded to TF32 (cvt.rna) or BF16, and staged in shared memory in the
// K-major core-matrix layout (tcgen05.cuh); one thread issues the MMAs of a K chunk while the
// others convert the next chunk into the second buffer.  The epilogue reads the accumulator
// rows from TMEM (warp w reads lanes 32 (w % 4) ..), undoes the scaling in FP64 and applies
// C = alpha * product + beta * C.
//
// Work split: persistent CTAs stride over the compacted output tiles of a job list
// (128 x 64 per tile: UMMA M = 128, N = the tile's columns rounded up to 16).
#include <cuda_bf16.h>

#include "internal.cuh"
#include "tcgen05.cuh"

namespace hcgb {

namespace {

constexpr int TC_M = 128, TC_N = 64;
constexpr int TC_THREADS = 256;
constexpr int TC_KBYTES = 128;                  // bytes of K per row per stage (8 core matrices)
constexpr int TC_KB = TC_KBYTES / 16;           // core matrices along K per stage
constexpr int TC_A_BYTES = TC_M * TC_KBYTES;    // 16 KB
constexpr int TC_B_BYTES = TC_N * TC_KBYTES;    // 8 KB
constexpr int TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;
constexpr int TC_SMEM = 2 * TC_STAGE_BYTES + 1024;  // two stages + alignment slack
constexpr int TC_NOGROUP = -1100;

__device__ unsigned int g_tc_wait_timeouts = 0;

__device__ __forceinline__ int exp_field(double x) { return (int) ((__double_as_longlong(x) >> 52) & 0x7ff); }

__device__ __forceinline__ double pow2(int ex) {
    if (ex < -1022) return 0.0;
    if (ex > 1023) ex = 1023;
    return __hiloint2double((ex + 1023) << 20, 0);
}

// Byte offset of element (row r, byte kb within the stage's K bytes) in the core-matrix layout.
__device__ __forceinline__ int cm_off(int r, int kbyte) {
    return ((r >> 3) * TC_KB + (kbyte >> 4)) * 128 + (r & 7) * 16 + (kbyte & 15);
}

__device__ __forceinline__ uint32_t to_tf32(float f) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(f));
    return r;
}

// One 128 x 64 output tile of one job.  PREC 1: TF32 (4 bytes per element, 32 per stage);
// PREC 2: BF16 (2 bytes, 64 per stage).
template <int PREC>
__device__ void tc_tile(const GemmJob &jb, int tile, unsigned char *stage0, uint32_t tmem, uint32_t mbar0,
                        uint32_t (&phase)[2], int *ea, int *eb) {
    constexpr int ESZ = PREC == 1 ? 4 : 2;
    constexpr int KC = TC_KBYTES / ESZ;  // K elements per stage
    const int ntm = (jb.M + TC_M - 1) / TC_M;
    const int m0 = (tile % ntm) * TC_M, n0 = (tile / ntm) * TC_N;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ncols = min(TC_N, jb.N - n0);
    const int nmma = (ncols + 15) & ~15;  // UMMA N for M = 128: a multiple of 16
    const uint32_t idesc = tc::instr_desc(PREC == 1 ? tc::FMT_TF32 : tc::FMT_BF16, TC_M, nmma);

    // 1. Power-of-two scale of every row of op(A) and column of op(B) over all of K.
    {
        constexpr int PA = TC_THREADS / TC_M, PB = TC_THREADS / TC_N;
        const int gi = m0 + tid / PA, pa = tid % PA;
        int ma = 0;
        if (gi < jb.M)
            for (int k = pa; k < jb.K; k += PA) ma = max(ma, exp_field(job_a(jb, gi, k)));
#pragma unroll
        for (int o = 1; o < PA; o <<= 1) ma = max(ma, __shfl_xor_sync(0xffffffffu, ma, o));
        if (pa == 0) ea[tid / PA] = ma ? ma - 1022 : TC_NOGROUP;
        const int gj = n0 + tid / PB, pb = tid % PB;
        int mb = 0;
        if (gj < jb.N)
            for (int k = pb; k < jb.K; k += PB) mb = max(mb, exp_field(job_b(jb, k, gj)));
#pragma unroll
        for (int o = 1; o < PB; o <<= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
        if (pb == 0) eb[tid / PB] = mb ? mb - 1022 : TC_NOGROUP;
    }
    __syncthreads();

    // 2. K chunks: convert into stage c % 2 (after the MMAs of chunk c - 2 have read it), then one
    //    thread issues the chunk's MMAs and commits them to the stage's barrier.
    const int nchunks = (jb.K + KC - 1) / KC;
    bool ok = true;
    for (int c = 0; c < nchunks; c++) {
        const int buf = c & 1;
        unsigned char *sa = stage0 + buf * TC_STAGE_BYTES, *sb = sa + TC_A_BYTES;
        if (c >= 2) {
            ok &= tc::mbar_wait(mbar0 + 8 * buf, phase[buf]);
            phase[buf] ^= 1;
        }
        const int k0 = c * KC;
        for (int e = tid; e < TC_M * KC; e += TC_THREADS) {
            int i, kk;
            if (jb.opA == 0) {
                i = e % TC_M;
                kk = e / TC_M;
            } else {
                kk = e % KC;
                i = e / KC;
            }
            const int gi = m0 + i, gk = k0 + kk;
            const int ex = ea[i];
            const double v = (gi < jb.M && gk < jb.K && ex > TC_NOGROUP) ? job_a(jb, gi, gk) * pow2(-ex) : 0.0;
            if (PREC == 1) *reinterpret_cast<uint32_t *>(sa + cm_off(i, kk * 4)) = to_tf32((float) v);
            else *reinterpret_cast<__nv_bfloat16 *>(sa + cm_off(i, kk * 2)) = __double2bfloat16(v);
        }
        for (int e = tid; e < TC_N * KC; e += TC_THREADS) {
            int j, kk;
            if (jb.opB == 0) {
                kk = e % KC;
                j = e / KC;
            } else {
                j = e % TC_N;
                kk = e / TC_N;
            }
            const int gj = n0 + j, gk = k0 + kk;
            const int ex = eb[j];
            const double v = (gj < jb.N && gk < jb.K && ex > TC_NOGROUP) ? job_b(jb, gk, gj) * pow2(-ex) : 0.0;
            if (PREC == 1) *reinterpret_cast<uint32_t *>(sb + cm_off(j, kk * 4)) = to_tf32((float) v);
            else *reinterpret_cast<__nv_bfloat16 *>(sb + cm_off(j, kk * 2)) = __double2bfloat16(v);
        }
        tc::fence_smem_to_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            const uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
#pragma unroll
            for (int s = 0; s < TC_KBYTES / 32; s++) {
                const uint64_t ad = tc::smem_desc(a0 + s * 256, 128, TC_KB * 128);
                const uint64_t bd = tc::smem_desc(b0 + s * 256, 128, TC_KB * 128);
                if (PREC == 1) tc::mma_tf32(tmem, ad, bd, idesc, (c > 0 || s > 0) ? 1u : 0u);
                else tc::mma_f16(tmem, ad, bd, idesc, (c > 0 || s > 0) ? 1u : 0u);
            }
            tc::commit(mbar0 + 8 * buf);
        }
    }
    // 3. The last one or two chunks' MMAs complete (every commit is waited for exactly once).
    for (int c = nchunks > 2 ? nchunks - 2 : 0; c < nchunks; c++) {
        const int buf = c & 1;
        ok &= tc::mbar_wait(mbar0 + 8 * buf, phase[buf]);
        phase[buf] ^= 1;
    }
    if (!ok && tid == 0) atomicAdd(&g_tc_wait_timeouts, 1u);
    tc::fence_after();

    // 4. Epilogue: warp w reads TMEM lanes 32 (w % 4) .. (rows) and columns 32 (w / 4) ..
    const int q = warp & 3, h = warp >> 2;
    const int row_l = q * 32 + lane, col0 = h * 32;
    if (col0 < ncols) {
        float v[32];
        tc::tmem_ld32(tmem + ((uint32_t) (q * 32) << 16) + (uint32_t) col0, v);
        const int row = m0 + row_l;
        if (row < jb.M && jb.K > 0) {
            const bool accum = jb.beta != 0.0;
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const int cl = col0 + j;
                if (cl < ncols) {
                    double *cp = jb.C + row + (size_t) (n0 + cl) * jb.ldc;
                    const double prod = (double) v[j] * pow2(ea[row_l] + eb[cl]);
                    double out = jb.alpha * prod;
                    if (accum) out = fma(jb.beta, *cp, out);
                    *cp = out;
                }
            }
        } else if (row < jb.M) {  // K = 0: C = beta C
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const int cl = col0 + j;
                if (cl < ncols) {
                    double *cp = jb.C + row + (size_t) (n0 + cl) * jb.ldc;
                    *cp = jb.beta != 0.0 ? jb.beta * *cp : 0.0;
                }
            }
        }
    }
    tc::fence_before();
    __syncthreads();
}

// Tiles of the jobs marked for TF32 / BF16 (prec 1 / 2), compacted (sched: exclusive prefix of
// tiles per job, njobs + 1 entries); a grid sized to the GPU strides over them.
__global__ void __launch_bounds__(TC_THREADS) tc_gemm_jobs_kernel(const GemmJob *jobs, int njobs, const int *sched) {
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    __shared__ __align__(8) unsigned long long mbar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int ea[TC_M], eb[TC_N];
    unsigned char *stage0 = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
    const int total = sched[njobs];
    if (blockIdx.x >= total) return;  // whole CTA leaves before any TMEM or barrier is set up
    const uint32_t mbar0 = tc::smem_u32(&mbar[0]);
    if (threadIdx.x == 0) {
        tc::mbar_init(mbar0, 1);
        tc::mbar_init(mbar0 + 8, 1);
    }
    if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(tc::smem_u32(&tmem_slot), TC_N);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    uint32_t phase[2] = {0u, 0u};
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        int lo = 0, hi = njobs;  // sched[lo] <= w < sched[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (sched[mid] <= w) lo = mid;
            else hi = mid;
        }
        const GemmJob jb = jobs[lo];
        if (jb.prec == 1) tc_tile<1>(jb, w - sched[lo], stage0, tmem, mbar0, phase, ea, eb);
        else tc_tile<2>(jb, w - sched[lo], stage0, tmem, mbar0, phase, ea, eb);
    }
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tc::tmem_free(tmem, TC_N);
}

}  // namespace

void launch_tc_gemm_jobs(const GemmJob *jobs, int njobs, const int *sched, int sms, cudaStream_t st) {
    if (njobs <= 0) return;
    cudaFuncSetAttribute(tc_gemm_jobs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    { tc_gemm_jobs_kernel<<<2 * sms, TC_THREADS, TC_SMEM, st>>>(jobs, njobs, sched); note_launch(); }
}

unsigned int tc_wait_timeouts() {
    unsigned int v = 0;
    cudaMemcpyFromSymbol(&v, g_tc_wait_timeouts, sizeof(v));
    return v;
}

}  // namespace hcgb
