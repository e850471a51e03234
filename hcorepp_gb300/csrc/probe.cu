// FP64 throughput probes: the roofline denominators of the FP64 path (the measured peaks that
// come with the machine cover only HBM copy bandwidth and bf16 tensor throughput).
#include "internal.cuh"

namespace hcgb {

namespace {

constexpr int PROBE_ITERS = 4096;

__global__ void __launch_bounds__(256) dmma_probe_kernel(double *sink, double seed) {
    const int lane = threadIdx.x & 31;
    const double a = seed * (1 + lane), b = 1.0 - seed * lane;
    double c[8][2];
#pragma unroll
    for (int i = 0; i < 8; i++) c[i][0] = c[i][1] = 0.0;
    for (int it = 0; it < PROBE_ITERS; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) dmma(c[i][0], c[i][1], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += c[i][0] + c[i][1];
    if (s == 1.2345) sink[threadIdx.x] = s;  // never true; keeps the work alive
}

__global__ void __launch_bounds__(256) dfma_probe_kernel(double *sink, double a, double b) {
    double x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x + i;
    for (int it = 0; it < PROBE_ITERS; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = fma(x[i], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    if (s == 1.2345) sink[threadIdx.x] = s;
}

}  // namespace

int measure_fp64_peak(cudaStream_t st, double *dmma_tflops, double *dfma_tflops) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HCGB_CUDA_ERROR;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return HCGB_CUDA_ERROR;
    double *sink = nullptr;
    if (cudaMalloc(&sink, 256 * sizeof(double)) != cudaSuccess) return HCGB_CUDA_ERROR;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 4, threads = 256;
    float ms = 0.f;
    // DMMA: each warp-level m8n8k4 is 8*8*4 FMAs.
    { dmma_probe_kernel<<<blocks, threads, 0, st>>>(sink, 1e-3); note_launch(); }
    cudaEventRecord(e0, st);
    { dmma_probe_kernel<<<blocks, threads, 0, st>>>(sink, 1e-3); note_launch(); }
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    const double dmma_flops = 2.0 * 256.0 * 8 * PROBE_ITERS * (double) blocks * (threads / 32);
    if (dmma_tflops) *dmma_tflops = dmma_flops / (ms * 1e-3) / 1e12;
    { dfma_probe_kernel<<<blocks, threads, 0, st>>>(sink, 0.999999, 1e-7); note_launch(); }
    cudaEventRecord(e0, st);
    { dfma_probe_kernel<<<blocks, threads, 0, st>>>(sink, 0.999999, 1e-7); note_launch(); }
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    const double dfma_flops = 2.0 * 8 * PROBE_ITERS * (double) blocks * threads;
    if (dfma_tflops) *dfma_tflops = dfma_flops / (ms * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    return cudaGetLastError() == cudaSuccess ? HCGB_OK : HCGB_CUDA_ERROR;
}

}  // namespace hcgb
