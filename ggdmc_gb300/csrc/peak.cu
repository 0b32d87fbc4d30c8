// peak.cu -- throughput probes for the roofline denominators of the
// likelihood kernel, which is bound by the FP32 FMA pipe and the MUFU
// (special-function) unit rather than by HBM or the tensor cores.
#include <cuda_runtime.h>

#include "../../include/ggdmc_gpu.h"

namespace {

constexpr int kProbeIters = 4096;

// 8 independent FMA chains per thread: 2 flops per FMA.
__global__ void k_fma_probe(float *out, float a, float b)
{
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = threadIdx.x * 1e-3f + j;
    for (int i = 0; i < kProbeIters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = fmaf(x[j], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    if (s == 12345.678f) out[0] = s;   // keeps the chains live
}

// 8 independent ex2.approx chains per thread (one MUFU op each).
__global__ void k_mufu_probe(float *out, float a)
{
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = -1e-3f * (threadIdx.x + j);
    for (int i = 0; i < kProbeIters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            float y;
            asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[j]));
            x[j] = y * a;
        }
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    if (s == 12345.678f) out[0] = s;
}

}  // namespace

extern "C" ggdmc_status ggdmc_probe_peaks(double *fp32_tflops, double *mufu_tops)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *d = nullptr;
    if (cudaMalloc(&d, sizeof(float))) return GGDMC_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256;
    float best_fma = 1e30f, best_mufu = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        float ms = 0.f;
        cudaEventRecord(e0);
        k_fma_probe<<<blocks, threads>>>(d, 1.0000001f, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep && ms < best_fma) best_fma = ms;
        cudaEventRecord(e0);
        k_mufu_probe<<<blocks, threads>>>(d, 0.999f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep && ms < best_mufu) best_mufu = ms;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (err) return GGDMC_ERR_CUDA;
    const double ops = (double)blocks * threads * kProbeIters * 8;
    if (fp32_tflops) *fp32_tflops = 2.0 * ops / (best_fma * 1e-3) / 1e12;
    if (mufu_tops) *mufu_tops = ops / (best_mufu * 1e-3) / 1e12;
    return GGDMC_OK;
}
