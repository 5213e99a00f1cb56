// peaks.cu -- throughput probes of the FP32 FMA pipe and the MUFU (SFU) pipe.
//
// The roofline of the sinc accumulation is compute-bound on these two pipes;
// the measured peaks cover only HBM and bf16 tensor throughput, so the
// library measures FP32 and MUFU peaks on the device it runs on.
#include <cuda_runtime.h>

namespace gpurir {

constexpr int kProbeChains = 8;

__global__ void __launch_bounds__(1024) probe_fma_kernel(float *out, int iters, float a, float b) {
    float x[kProbeChains];
#pragma unroll
    for (int c = 0; c < kProbeChains; c++) x[c] = threadIdx.x * 1e-7f + c;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kProbeChains; c++) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kProbeChains; c++) s += x[c];
    if (s == 12345.678f) out[threadIdx.x] = s;   // keeps the chains live
}

__global__ void __launch_bounds__(1024) probe_mufu_kernel(float *out, int iters) {
    float x[kProbeChains];
#pragma unroll
    for (int c = 0; c < kProbeChains; c++) x[c] = 1.0f + threadIdx.x * 1e-7f + c;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kProbeChains; c++) {
            float r;
            asm volatile("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x[c]));
            x[c] = r + 0.5f;   // keeps rcp(rcp(x)) from folding; x stays in [1.5, 2.2]
        }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kProbeChains; c++) s += x[c];
    if (s == 12345.678f) out[threadIdx.x] = s;
}

// Returns FP32 FLOP/s (2 per FMA) and MUFU op/s measured with CUDA events.
// The MUFU chain carries one FADD per reciprocal, which the FP32 pipe absorbs
// at 1/8 of its rate, so the chain is MUFU-bound.
cudaError_t probe_peaks(double *fp32_flops, double *mufu_ops, cudaStream_t st) {
    int dev, sms;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    float *buf;
    if ((e = cudaMalloc(&buf, 1024 * sizeof(float))) != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 2, threads = 1024;
    const int it_fma = 16384, it_mufu = 2048;
    float ms = 0.f, best_fma = 1e30f, best_mufu = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(a, st);
        probe_fma_kernel<<<blocks, threads, 0, st>>>(buf, it_fma, 0.9999f, 1e-6f);
        cudaEventRecord(b, st);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best_fma) best_fma = ms;
        cudaEventRecord(a, st);
        probe_mufu_kernel<<<blocks, threads, 0, st>>>(buf, it_mufu);
        cudaEventRecord(b, st);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best_mufu) best_mufu = ms;
    }
    e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    const double n = (double)blocks * threads * kProbeChains;
    *fp32_flops = 2.0 * n * it_fma / (best_fma * 1e-3);
    *mufu_ops = n * it_mufu / (best_mufu * 1e-3);
    return e;
}

}  // namespace gpurir
