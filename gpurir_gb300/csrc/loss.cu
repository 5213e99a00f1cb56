// loss.cu -- the L2 loss of a differentiable step and its gradient in one pass.
//
// For a training loop that fits RIRs to a target (the inverse problem: walls
// and positions from measured responses), loss = scale * sum (y - t)^2 and
// dL/dy = 2 scale (y - t) are formed by one kernel that reads y and t once
// and writes the gradient the adjoint kernel consumes; a second one-block
// kernel adds the per-block partial sums in a fixed order (deterministic).
// gpuRIR has no counterpart (it is not differentiable).
#include <cuda_runtime.h>

namespace gpurir {

constexpr int kLossThreads = 256;

__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kLossThreads / 32; w++) s += red[w];
    return s;   // valid in thread 0
}

// g = 2 scale (y - t); partial[block] = sum over the block's elements of (y - t)^2.
__global__ void __launch_bounds__(kLossThreads) l2_grad_kernel(const float *__restrict__ y,
                                                               const float *__restrict__ t, long n,
                                                               float scale, float *__restrict__ g,
                                                               double *__restrict__ partial) {
    __shared__ double red[kLossThreads / 32];
    const float two_s = 2.0f * scale;
    float acc = 0.0f;
    const long stride = (long)gridDim.x * kLossThreads;
    const long n4 = n / 4;
    const float4 *y4 = reinterpret_cast<const float4 *>(y);
    const float4 *t4 = reinterpret_cast<const float4 *>(t);
    float4 *g4 = reinterpret_cast<float4 *>(g);
    for (long i = (long)blockIdx.x * kLossThreads + threadIdx.x; i < n4; i += stride) {
        const float4 a = __ldg(&y4[i]), b = __ldg(&t4[i]);
        const float4 d = make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
        acc = fmaf(d.x, d.x, fmaf(d.y, d.y, fmaf(d.z, d.z, fmaf(d.w, d.w, acc))));
        g4[i] = make_float4(two_s * d.x, two_s * d.y, two_s * d.z, two_s * d.w);
    }
    if (blockIdx.x == 0)
        for (long i = 4 * n4 + threadIdx.x; i < n; i += kLossThreads) {
            const float d = y[i] - t[i];
            acc = fmaf(d, d, acc);
            g[i] = two_s * d;
        }
    const double s = block_sum((double)acc, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kLossThreads) l2_final_kernel(const double *__restrict__ partial, int n_part,
                                                                float scale, float *__restrict__ loss) {
    __shared__ double red[kLossThreads / 32];
    double v = 0.0;
    for (int i = threadIdx.x; i < n_part; i += kLossThreads) v += partial[i];
    const double s = block_sum(v, red);
    if (threadIdx.x == 0) *loss = (float)(s * (double)scale);
}

// Blocks of l2_grad_kernel for n elements (fixed for a given n: the sum order, and so
// the loss, does not change between calls).
int l2_grad_blocks(long n) {
    long b = (n / 4 + 4 * kLossThreads - 1) / (4 * kLossThreads);
    if (b < 1) b = 1;
    if (b > 1024) b = 1024;
    return (int)b;
}

// y, t, g must be 16-byte aligned; partial holds l2_grad_blocks(n) doubles.
cudaError_t l2_grad_launch(const float *y, const float *t, long n, float scale, float *g, double *partial,
                           float *loss, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int blocks = l2_grad_blocks(n);
    l2_grad_kernel<<<blocks, kLossThreads, 0, st>>>(y, t, n, scale, g, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    l2_final_kernel<<<1, kLossThreads, 0, st>>>(partial, blocks, scale, loss);
    return cudaGetLastError();
}

}  // namespace gpurir
