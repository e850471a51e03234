// Rank predictor of the learned recompression form: an MLP 12 -> 64 -> 64 -> 1 with GELU
// activations, BF16 weights and FP32 accumulation, trained with mean squared error on the log of
// the post-recompression rank (target log2(1 + r)).  Everything here is hand-written: inference
// (one thread per sample, weights staged in shared memory as floats), the backward pass (per
// sample activations in shared memory, per-block gradient sums added atomically into an FP32
// gradient), and Adam on an FP32 master copy that is re-rounded to the BF16 weights after every
// step (the weights the forward and backward passes read).
//
// No counterpart in the reference: HCore++ sizes every recompression by the full QR + SVD
// (src/operators/concrete/Compressed.cpp:441-527); this model only chooses the sketch width of
// the learned form, and the plain recompression stays the fallback.
#include <cuda_bf16.h>

#include <cstring>
#include <vector>

#include "internal.cuh"

namespace hcgb {

namespace {

constexpr int F = MLP_IN, H = MLP_HIDDEN;
// Parameter layout (floats): W1 [H][F] row-major, b1 [H], W2 [H][H] row-major, b2 [H], w3 [H], b3.
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * F, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H;
static_assert(OFF_B3 + 1 == MLP_PARAMS, "parameter layout");

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
// d/dx GELU(x) = Phi(x) + x phi(x)
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__device__ void load_weights(const __nv_bfloat16 *w, float *s) {
    for (int i = threadIdx.x; i < MLP_PARAMS; i += blockDim.x) s[i] = __bfloat162float(w[i]);
    __syncthreads();
}

// Forward pass of one sample from the weights in shared memory; optionally keeps the hidden
// activations and the GELU derivatives (for the backward pass).
__device__ float forward_one(const float *s, const float *x, float *h1, float *g1, float *h2, float *g2) {
    float h[H];
#pragma unroll
    for (int j = 0; j < H; j++) {
        float acc = s[OFF_B1 + j];
#pragma unroll
        for (int i = 0; i < F; i++) acc = fmaf(s[OFF_W1 + j * F + i], x[i], acc);
        h[j] = gelu(acc);
        if (h1) {
            h1[j] = h[j];
            g1[j] = gelu_grad(acc);
        }
    }
    float y = s[OFF_B3];
    for (int j = 0; j < H; j++) {
        float acc = s[OFF_B2 + j];
#pragma unroll
        for (int i = 0; i < H; i++) acc = fmaf(s[OFF_W2 + j * H + i], h[i], acc);
        const float hj = gelu(acc);
        if (h2) {
            h2[j] = hj;
            g2[j] = gelu_grad(acc);
        }
        y = fmaf(s[OFF_W3 + j], hj, y);
    }
    return y;
}

__global__ void __launch_bounds__(128) mlp_forward_kernel(const __nv_bfloat16 *w, const float *X, int n, float *Y) {
    __shared__ float s[MLP_PARAMS];
    load_weights(w, s);
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        float x[F];
#pragma unroll
        for (int i = 0; i < F; i++) x[i] = X[(size_t) idx * F + i];
        Y[idx] = forward_one(s, x, nullptr, nullptr, nullptr, nullptr);
    }
}

// Gradient of L = (1 / n_total) sum_s (y_s - t_s)^2 over the samples [off, off + n) of a batch
// (rows idx[off ..] of X, T when idx != nullptr), added into grad (MLP_PARAMS floats); the
// loss sum (not divided) is added into *loss.  One sample per thread for the forward and
// per-sample backward parts, then one parameter per thread for the block's sums.
constexpr int GB = 64;  // samples per block
struct GradSmem {
    float w[MLP_PARAMS];
    float x[GB][F];
    float h1[GB][H], g1[GB][H], h2[GB][H], g2[GB][H];
    float da2[GB][H], da1[GB][H];
    float dy[GB];
};

__global__ void __launch_bounds__(GB) mlp_grad_kernel(const __nv_bfloat16 *w, const float *X, const float *T,
                                                     const int *idx, int off, int n, float inv_total,
                                                     float *grad, double *loss) {
    extern __shared__ __align__(16) unsigned char gsm_raw[];
    GradSmem &S = *reinterpret_cast<GradSmem *>(gsm_raw);
    load_weights(w, S.w);
    const int s = threadIdx.x;
    const int q = blockIdx.x * GB + s;  // sample within [0, n)
    const bool act = q < n;
    float err = 0.f;
    if (act) {
        const int row = idx ? idx[off + q] : off + q;
#pragma unroll
        for (int i = 0; i < F; i++) S.x[s][i] = X[(size_t) row * F + i];
        const float y = forward_one(S.w, S.x[s], S.h1[s], S.g1[s], S.h2[s], S.g2[s]);
        err = y - T[row];
        const float dy = 2.0f * err * inv_total;
        S.dy[s] = dy;
        for (int j = 0; j < H; j++) S.da2[s][j] = dy * S.w[OFF_W3 + j] * S.g2[s][j];
        for (int i = 0; i < H; i++) {
            float acc = 0.f;
            for (int j = 0; j < H; j++) acc = fmaf(S.w[OFF_W2 + j * H + i], S.da2[s][j], acc);
            S.da1[s][i] = acc * S.g1[s][i];
        }
    } else {
        for (int i = 0; i < F; i++) S.x[s][i] = 0.f;
        S.dy[s] = 0.f;
        for (int j = 0; j < H; j++) S.h1[s][j] = S.h2[s][j] = S.da1[s][j] = S.da2[s][j] = 0.f;
    }
    // block loss
    float e2 = err * err;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, (double) e2);
    __syncthreads();
    for (int p = threadIdx.x; p < MLP_PARAMS; p += blockDim.x) {
        float acc = 0.f;
        if (p < OFF_B1) {
            const int j = p / F, i = p % F;
            for (int t = 0; t < GB; t++) acc = fmaf(S.da1[t][j], S.x[t][i], acc);
        } else if (p < OFF_W2) {
            const int j = p - OFF_B1;
            for (int t = 0; t < GB; t++) acc += S.da1[t][j];
        } else if (p < OFF_B2) {
            const int j = (p - OFF_W2) / H, i = (p - OFF_W2) % H;
            for (int t = 0; t < GB; t++) acc = fmaf(S.da2[t][j], S.h1[t][i], acc);
        } else if (p < OFF_W3) {
            const int j = p - OFF_B2;
            for (int t = 0; t < GB; t++) acc += S.da2[t][j];
        } else if (p < OFF_B3) {
            const int j = p - OFF_W3;
            for (int t = 0; t < GB; t++) acc = fmaf(S.dy[t], S.h2[t][j], acc);
        } else {
            for (int t = 0; t < GB; t++) acc += S.dy[t];
        }
        if (acc != 0.f) atomicAdd(&grad[p], acc);
    }
}

// Adam (Kingma & Ba) on the FP32 master parameters, then the BF16 weights re-rounded from them;
// the gradient is cleared for the next step.
__global__ void adam_kernel(float *master, __nv_bfloat16 *w, float *grad, float *m1, float *m2, float lr, float b1,
                            float b2, float eps, float bc1, float bc2) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < MLP_PARAMS; p += gridDim.x * blockDim.x) {
        const float g = grad[p];
        const float a = b1 * m1[p] + (1.f - b1) * g;
        const float v = b2 * m2[p] + (1.f - b2) * g * g;
        m1[p] = a;
        m2[p] = v;
        const float step = lr * (a / bc1) / (sqrtf(v / bc2) + eps);
        const float nm = master[p] - step;
        master[p] = nm;
        w[p] = __float2bfloat16(nm);
        grad[p] = 0.f;
    }
}

__global__ void round_weights_kernel(const float *master, __nv_bfloat16 *w) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < MLP_PARAMS; p += gridDim.x * blockDim.x)
        w[p] = __float2bfloat16(master[p]);
}

// Targets log2(1 + new rank) and the rows kept for training (recompressed updates with status OK
// or NOT_CONVERGED) from the per-update records; keep[i] = 1 / 0.
__global__ void targets_from_records_kernel(const hcgb_update_info *info, int n, float *T, int *keep) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const hcgb_update_info r = info[i];
        const bool ok = (r.status == HCGB_OK || r.status == HCGB_NOT_CONVERGED) && r.k > 0;
        keep[i] = ok ? 1 : 0;
        T[i] = ok ? log2f(1.0f + (float) r.new_rank) : 0.f;
    }
}

size_t grad_smem() { return sizeof(GradSmem); }

}  // namespace

// ---------------------------------------------------------------------------------------------
// RankModel: device parameters of one predictor.
// ---------------------------------------------------------------------------------------------
int RankModel::init(unsigned long long seed) {
    if (cudaMalloc(&master, sizeof(float) * MLP_PARAMS * 4) != cudaSuccess) return HCGB_CUDA_ERROR;
    grad = master + MLP_PARAMS;
    m1 = grad + MLP_PARAMS;
    m2 = m1 + MLP_PARAMS;
    if (cudaMalloc(&w, sizeof(__nv_bfloat16) * MLP_PARAMS) != cudaSuccess) return HCGB_CUDA_ERROR;
    // Glorot-uniform initialisation from a 64-bit LCG (host side), biases zero.
    std::vector<float> p(MLP_PARAMS, 0.f);
    unsigned long long st = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto uni = [&]() {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        return (float) ((st >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
    };
    auto fill = [&](int off, int fan_in, int fan_out, int count) {
        const float a = sqrtf(6.f / (float) (fan_in + fan_out));
        for (int i = 0; i < count; i++) p[off + i] = a * uni();
    };
    fill(OFF_W1, F, H, H * F);
    fill(OFF_W2, H, H, H * H);
    fill(OFF_W3, H, 1, H);
    return set_params(p.data());
}

int RankModel::set_params(const float *host) {
    if (cudaMemcpy(master, host, sizeof(float) * MLP_PARAMS, cudaMemcpyHostToDevice) != cudaSuccess)
        return HCGB_CUDA_ERROR;
    if (cudaMemset(grad, 0, sizeof(float) * MLP_PARAMS * 3) != cudaSuccess) return HCGB_CUDA_ERROR;
    { round_weights_kernel<<<8, 256>>>(master, w); note_launch(); }
    adam_t = 0;
    return cudaDeviceSynchronize() == cudaSuccess ? HCGB_OK : HCGB_CUDA_ERROR;
}

int RankModel::get_params(float *host) const {
    return cudaMemcpy(host, master, sizeof(float) * MLP_PARAMS, cudaMemcpyDeviceToHost) == cudaSuccess
               ? HCGB_OK
               : HCGB_CUDA_ERROR;
}

void RankModel::release() {
    if (master) cudaFree(master);
    if (w) cudaFree(w);
    master = nullptr;
    w = nullptr;
}

void launch_mlp_forward(const RankModel &m, const float *X, int n, float *Y, cudaStream_t st) {
    if (n <= 0) return;
    const int blocks = (n + 127) / 128 < 1024 ? (n + 127) / 128 : 1024;
    { mlp_forward_kernel<<<blocks, 128, 0, st>>>(m.w, X, n, Y); note_launch(); }
}

void launch_mlp_grad(const RankModel &m, const float *X, const float *T, const int *idx, int off, int n,
                     float inv_total, double *loss, cudaStream_t st) {
    if (n <= 0) return;
    static const bool attr = [] {
        return cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int) grad_smem()) == cudaSuccess;
    }();
    (void) attr;
    { mlp_grad_kernel<<<(n + GB - 1) / GB, GB, grad_smem(), st>>>(m.w, X, T, idx, off, n, inv_total, m.grad, loss); note_launch(); }
}

void launch_adam(RankModel &m, float lr, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f;
    m.adam_t++;
    const float bc1 = 1.f - powf(b1, (float) m.adam_t), bc2 = 1.f - powf(b2, (float) m.adam_t);
    { adam_kernel<<<8, 256, 0, st>>>(m.master, m.w, m.grad, m.m1, m.m2, lr, b1, b2, 1e-8f, bc1, bc2); note_launch(); }
}

void launch_targets_from_records(const hcgb_update_info *info, int n, float *T, int *keep, cudaStream_t st) {
    if (n > 0) { targets_from_records_kernel<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, st>>>(info, n, T, keep); note_launch(); }
}

}  // namespace hcgb
