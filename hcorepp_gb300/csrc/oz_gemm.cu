// FP64 factor products on the 16-bit tensor cores by error-free splitting (the Ozaki scheme).
//
// The GB300's FP64 pipe (SIMT or DMMA) delivers ~1.1 TFLOP/s, its FP16 tensor cores ~600 TFLOP/s
// through mma.sync.  A product C = op(A) op(B) is computed exactly enough for FP64 work as follows:
//   * every row i of op(A) gets the exponent e_i with max_k |A_ik| < 2^e_i, every column j of
//     op(B) the exponent f_j with max_k |B_kj| < 2^f_j;
//   * each element becomes a 56-bit fixed-point integer relative to its group's exponent (rounded
//     to nearest; the rounding error is 2^-57 of the group maximum) and is cut into S = 8 signed
//     7-bit digits, A = sum_s 2^(e_i - 7 s) A^(s) with integer planes |A^(s)| <= 127, exact in FP16;
//   * the plane products A^(s) B^(t) are integers; over a k-chunk of 32 every partial sum of a
//     level L = s + t (at most 8 terms of 127 * 127 per k) stays below 2^22, so the FP32
//     accumulators of the tensor cores hold them exactly and an FP32 add of 1.5 * 2^23 exposes
//     them as integers in the low mantissa bits;
//   * levels s + t <= S + 1 are kept (the dropped ones sum to < 2^-44 of max|A_i| max|B_j| for
//     k <= 512, the order of FP64's own worst-case bound); after every chunk the levels are added
//     into two 64-bit integers (levels 2-5 and 6-9, each shifted to a common scale), which stay
//     exact for k up to 2^14, and the tile ends with C_ij = 2^(e_i + f_j) (hi 2^-35 + lo 2^-63).
// All of the splitting and combining is integer work; an output element costs 4 FP64
// instructions (two conversions, two scalings) plus the epilogue.
#include <cuda_fp16.h>

#include "internal.cuh"

namespace hcgb {

namespace {

constexpr int OZ_S = 8;                 // digit planes per operand
constexpr int OZ_B = 7;                 // bits per digit
constexpr int OZ_W = OZ_S * OZ_B;       // fixed-point width (56 bits)
constexpr int OZ_TM = 64, OZ_TN = 32;   // output tile per CTA
constexpr int OZ_KC = 32;               // k-chunk staged in shared memory
constexpr int OZ_LDS = 40;              // padded row of a plane in halves (conflict-free fragment loads)
constexpr int OZ_THREADS = 256;         // 8 warps (4 x 2), each a 16 x 16 piece of the tile
constexpr int OZ_NOGROUP = -1100;       // exponent of an all-zero group

// Biased exponent field of |x| (0 for zero and subnormals).
__device__ __forceinline__ int exp_field(double x) {
    return (int) ((__double_as_longlong(x) >> 52) & 0x7ff);
}

// Digits of x relative to the group exponent e (|x| < 2^e): plane s receives the signed digit of
// weight 2^(e - 7 (s + 1)).  Subnormals (far below any group maximum here) count as zero.
__device__ __forceinline__ void oz_digits(double x, int e, __half *dst, int plane_stride) {
    const long long bits = __double_as_longlong(x);
    const int E = (int) ((bits >> 52) & 0x7ff);
    unsigned long long u = 0;
    if (E != 0 && e > OZ_NOGROUP) {
        const unsigned long long M = (unsigned long long) (bits & 0xfffffffffffffLL) | (1ULL << 52);
        const int sh = E - 1019 - e;  // x * 2^(56 - e) = M * 2^sh, sh <= 3
        if (sh >= 0) u = M << sh;
        else if (sh > -64) u = (M + (1ULL << (-sh - 1))) >> (-sh);
    }
    const bool neg = bits < 0;
#pragma unroll
    for (int s = 0; s < OZ_S; s++) {
        const int d = (int) ((u >> (OZ_W - OZ_B * (s + 1))) & 127u);
        dst[s * plane_stride] = __int2half_rn(neg ? -d : d);
    }
}

// 2^ex as a double (0 below the normal range).
__device__ __forceinline__ double pow2(int ex) {
    if (ex < -1022) return 0.0;
    if (ex > 1023) ex = 1023;
    return __hiloint2double((ex + 1023) << 20, 0);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ double load_a(const GemmJob &jb, int i, int k) { return job_a(jb, i, k); }
__device__ __forceinline__ double load_b(const GemmJob &jb, int k, int j) { return job_b(jb, k, j); }

// One 64 x 32 output tile of one job.
__device__ void oz_tile(const GemmJob &jb, int tile, __half *As, __half *Bs, int *ea, int *eb) {
    const int ntm = (jb.M + OZ_TM - 1) / OZ_TM;
    const int m0 = (tile % ntm) * OZ_TM, n0 = (tile / ntm) * OZ_TN;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // 1. Group exponents over all of K: PA threads per row of op(A), PB per column of op(B).
    {
        constexpr int PA = OZ_THREADS / OZ_TM, PB = OZ_THREADS / OZ_TN;
        const int gi = m0 + tid / PA, pa = tid % PA;
        int ma = 0;
        if (gi < jb.M)
            for (int k = pa; k < jb.K; k += PA) ma = max(ma, exp_field(load_a(jb, gi, k)));
#pragma unroll
        for (int o = 1; o < PA; o <<= 1) ma = max(ma, __shfl_xor_sync(0xffffffffu, ma, o));
        if (pa == 0) ea[tid / PA] = ma ? ma - 1022 : OZ_NOGROUP;
        const int gj = n0 + tid / PB, pb = tid % PB;
        int mb = 0;
        if (gj < jb.N)
            for (int k = pb; k < jb.K; k += PB) mb = max(mb, exp_field(load_b(jb, k, gj)));
#pragma unroll
        for (int o = 1; o < PB; o <<= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
        if (pb == 0) eb[tid / PB] = mb ? mb - 1022 : OZ_NOGROUP;
    }
    __syncthreads();

    const int g = lane >> 2, c = lane & 3;
    const int wm = warp & 3, wn = warp >> 2;  // 4 x 2 warps, 16 x 16 each
    float acc[OZ_S][2][4];
    long long hi[2][4], lo[2][4];  // levels 2-5 at scale 2^-35, levels 6-9 at scale 2^-63
#pragma unroll
    for (int l = 0; l < OZ_S; l++)
#pragma unroll
        for (int t = 0; t < 2; t++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[l][t][q] = 0.f;
#pragma unroll
    for (int t = 0; t < 2; t++)
#pragma unroll
        for (int q = 0; q < 4; q++) hi[t][q] = lo[t][q] = 0;
    // group-exponent sums of this thread's eight outputs
    int ebase[2][4];
#pragma unroll
    for (int t = 0; t < 2; t++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int rl = wm * 16 + g + (q >= 2 ? 8 : 0), cl = wn * 16 + t * 8 + 2 * c + (q & 1);
            ebase[t][q] = ea[rl] + eb[cl];
        }

    int chunk = 0;
    for (int k0 = 0; k0 < jb.K; k0 += OZ_KC, chunk++) {
        // 2. Split the chunk of op(A) (64 x 32) and op(B) (32 x 32) into digit planes.
        for (int e = tid; e < OZ_TM * OZ_KC; e += OZ_THREADS) {
            int i, kk;
            if (jb.opA == 0) {
                i = e % OZ_TM;
                kk = e / OZ_TM;
            } else {
                kk = e % OZ_KC;
                i = e / OZ_KC;
            }
            const int gi = m0 + i, gk = k0 + kk;
            const double v = (gi < jb.M && gk < jb.K) ? load_a(jb, gi, gk) : 0.0;
            oz_digits(v, ea[i], As + i * OZ_LDS + kk, OZ_TM * OZ_LDS);
        }
        for (int e = tid; e < OZ_TN * OZ_KC; e += OZ_THREADS) {
            int j, kk;
            if (jb.opB == 0) {
                kk = e % OZ_KC;
                j = e / OZ_KC;
            } else {
                j = e % OZ_TN;
                kk = e / OZ_TN;
            }
            const int gj = n0 + j, gk = k0 + kk;
            const double v = (gj < jb.N && gk < jb.K) ? load_b(jb, gk, gj) : 0.0;
            oz_digits(v, eb[j], Bs + j * OZ_LDS + kk, OZ_TN * OZ_LDS);
        }
        __syncthreads();
        // 3. Plane products, level by level, on the tensor cores (exact in FP32).
#pragma unroll
        for (int ks = 0; ks < OZ_KC; ks += 16) {
#pragma unroll
            for (int s = 0; s < OZ_S; s++) {
                const __half *ap = As + s * OZ_TM * OZ_LDS + (wm * 16 + g) * OZ_LDS + ks + 2 * c;
                unsigned a[4];
                a[0] = *reinterpret_cast<const unsigned *>(ap);
                a[1] = *reinterpret_cast<const unsigned *>(ap + 8 * OZ_LDS);
                a[2] = *reinterpret_cast<const unsigned *>(ap + 8);
                a[3] = *reinterpret_cast<const unsigned *>(ap + 8 * OZ_LDS + 8);
#pragma unroll
                for (int t = 0; t < OZ_S - s; t++) {
                    const __half *bp = Bs + t * OZ_TN * OZ_LDS + (wn * 16 + g) * OZ_LDS + ks + 2 * c;
                    const unsigned b00 = *reinterpret_cast<const unsigned *>(bp);
                    const unsigned b01 = *reinterpret_cast<const unsigned *>(bp + 8);
                    const unsigned b10 = *reinterpret_cast<const unsigned *>(bp + 8 * OZ_LDS);
                    const unsigned b11 = *reinterpret_cast<const unsigned *>(bp + 8 * OZ_LDS + 8);
                    mma16816(acc[s + t][0], a, b00, b01);
                    mma16816(acc[s + t][1], a, b10, b11);
                }
            }
        }
        __syncthreads();
        // 4. Levels into the 64-bit integers (exact: |level| < 2^22 per chunk).
#pragma unroll
        for (int l = 0; l < OZ_S; l++)
#pragma unroll
            for (int t = 0; t < 2; t++)
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const long long v = (long long) (__float_as_int(acc[l][t][q] + 12582912.0f) - 0x4B400000);
                    if (l < 4) hi[t][q] += v << (OZ_B * (3 - l));
                    else lo[t][q] += v << (OZ_B * (7 - l));
                    acc[l][t][q] = 0.f;
                }
    }
    // 5. Epilogue: C = alpha * product + beta * C.
    const bool scale = jb.alpha != 1.0, accum = jb.beta != 0.0;
#pragma unroll
    for (int t = 0; t < 2; t++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int row = m0 + wm * 16 + g + (q >= 2 ? 8 : 0);
            const int col = n0 + wn * 16 + t * 8 + 2 * c + (q & 1);
            if (row < jb.M && col < jb.N) {
                double *cp = jb.C + row + (size_t) col * jb.ldc;
                const double prod = fma((double) hi[t][q], pow2(ebase[t][q] - 35),
                                        (double) lo[t][q] * pow2(ebase[t][q] - 63));
                double v = scale ? jb.alpha * prod : prod;
                if (accum) v = fma(jb.beta, *cp, v);
                *cp = v;
            }
        }
}

// Tiles of the jobs marked oz, compacted (sched: exclusive prefix of tiles per job, njobs + 1
// entries); a grid sized to the GPU strides over them.
__global__ void __launch_bounds__(OZ_THREADS) oz_gemm_jobs_kernel(const GemmJob *jobs, int njobs, const int *sched) {
    extern __shared__ __align__(16) unsigned char oz_smem[];
    __half *As = reinterpret_cast<__half *>(oz_smem);  // [plane][row][k]
    __half *Bs = As + OZ_S * OZ_TM * OZ_LDS;            // [plane][col][k]
    __shared__ int ea[OZ_TM], eb[OZ_TN];
    const int total = sched[njobs];
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        int lo = 0, hi = njobs;  // sched[lo] <= w < sched[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (sched[mid] <= w) lo = mid;
            else hi = mid;
        }
        const GemmJob jb = jobs[lo];
        oz_tile(jb, w - sched[lo], As, Bs, ea, eb);
        __syncthreads();
    }
}

}  // namespace

void launch_oz_gemm_jobs(const GemmJob *jobs, int njobs, const int *sched, int sms, cudaStream_t st) {
    if (njobs <= 0) return;
    const int smem = (int) (sizeof(__half) * OZ_S * (OZ_TM + OZ_TN) * OZ_LDS);
    cudaFuncSetAttribute(oz_gemm_jobs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    { oz_gemm_jobs_kernel<<<sms, OZ_THREADS, smem, st>>>(jobs, njobs, sched); note_launch(); }
}

}  // namespace hcgb
