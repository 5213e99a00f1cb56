// tail.cu -- diffuse reverberation tail for sm_103a.
//
// Replaces envPred_kernel (src/gpuRIR_cuda.cu:415-443), the cuRAND uniform
// fill (:874) and diffRev_kernel (:445-461) by one kernel: each block predicts
// the envelope of its RIR from the last <=10 ms of the early part (already in
// the output row), then writes its chunk of the tail from a counter-based
// Philox4x32-10 stream keyed by (seed, call offset, global RIR index), so the
// noise is reproducible and needs no generator state or extra HBM pass.
#include "gpurir_internal.cuh"

namespace gpurir {

constexpr int kTailThreads = 256;
constexpr int kTailChunk = kTailThreads * 16;   // samples per block (4 Philox blocks/thread)

struct TailLaunch {
    const RoomDesc *rooms;
    const IsmItem *rirs;     // one entry per RIR (t_lo/t_hi unused)
    int n_rir;
    const float *pos_src, *pos_rcv;
    float *out;
    uint64_t seed, offset;
    const uint64_t *offset_ptr;   // if set, the call offset is read here (captured graphs)
    int noise_kind;          // 0 logistic (reference), 1 Gaussian (Box-Muller)
    float *env_out;          // optional [n_rir][3]: A, alpha, tau_dp
};

// Direct-path delay in samples, same float-float arithmetic as the ISM kernel
// applies to the image with clust = refl = 0 (src/gpuRIR_cuda.cu:368-369).
__device__ __forceinline__ float direct_tau(const RoomDesc &R, const float *ps, const float *pr) {
    ff v0 = ff_two_sum(ps[0], -pr[0]);
    ff v1 = ff_two_sum(ps[1], -pr[1]);
    ff v2 = ff_two_sum(ps[2], -pr[2]);
    ff d2 = ff_add(ff_add(ff_sqr(v0), ff_sqr(v1)), ff_sqr(v2));
    ff tau = ff_mul(ff_sqrt(d2), ff{R.kh, R.kl});
    return tau.hi + tau.lo;
}

__global__ void __launch_bounds__(kTailThreads) tail_kernel(TailLaunch P) {
    const int rir = blockIdx.x;
    if (rir >= P.n_rir) return;
    const IsmItem it = P.rirs[rir];
    const RoomDesc &R = P.rooms[it.room];
    const int n_ism = R.n_ism, n_diff = R.n_total - R.n_ism;
    const int s0 = blockIdx.y * kTailChunk;
    if (s0 >= n_diff) return;
    float *row = P.out + it.out_row;

    __shared__ float red[kTailThreads / 32];
    __shared__ float envA, envB;
    const float tau_dp = direct_tau(R, P.pos_src + 3 * it.src, P.pos_rcv + 3 * it.rcv);
    // envelope window, src/gpuRIR_cuda.cu:419-428
    const float w_sz = 10e-3f * R.fs;
    const float lo = fmaxf((float)n_ism - w_sz, tau_dp);
    const int w_start = (int)ceilf(lo);
    const int cnt = n_ism - w_start;
    float p = 0.0f;
    for (int t = w_start + threadIdx.x; t < n_ism; t += kTailThreads) {
        float v = row[t];
        p = fmaf(v, v, p);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = p;
    __syncthreads();
    if (threadIdx.x == 0) {
        float tot = 0.0f;
        for (int w = 0; w < kTailThreads / 32; w++) tot += red[w];
        const float alpha = -13.8155f / (R.T60 * R.fs);   // log(1e-6) / (T60 Fs)
        float A = 0.0f;
        if (cnt > 0) {
            const float w_center = (float)w_start + (float)cnt * 0.5f;
            A = (tot / (float)cnt) / expf(alpha * (w_center - tau_dp));
        }
        // out = sqrt(A exp(alpha (n_ism + s - tau_dp))) * noise = exp(B + 0.5 alpha s) * noise
        envA = 0.5f * alpha;
        envB = (A > 0.0f) ? 0.5f * logf(A) + 0.5f * alpha * ((float)n_ism - tau_dp) : -INFINITY;
        if (P.env_out && blockIdx.y == 0) {
            P.env_out[3 * rir] = A;
            P.env_out[3 * rir + 1] = alpha;
            P.env_out[3 * rir + 2] = tau_dp;
        }
    }
    __syncthreads();
    const float ea = envA, eb = envB;
    const uint2 key = make_uint2((uint32_t)P.seed, (uint32_t)(P.seed >> 32));
    const uint64_t offset = P.offset_ptr ? *P.offset_ptr : P.offset;
    const uint32_t off_lo = (uint32_t)offset, off_hi = (uint32_t)(offset >> 32);
    const uint32_t gidx = (uint32_t)it.rir;
    float *trow = row + n_ism;
#pragma unroll 1
    for (int q = 0; q < kTailChunk / (4 * kTailThreads); q++) {
        const int s = s0 + 4 * (q * kTailThreads + threadIdx.x);
        if (s >= n_diff) break;
        const uint4 w = philox4x32_10(make_uint4((uint32_t)(s >> 2), gidx, off_lo, off_hi), key);
        float z[4];
        if (P.noise_kind == 0) {
            // logistic noise of unit variance, src/gpuRIR_cuda.cu:454-455
            const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float u = u01(ww[e]);
                z[e] = 0.551329f * __logf(u / (1.0f - u + 1e-6f));
            }
        } else {
            const float r0 = sqrtf(-2.0f * __logf(u01(w.x)));
            const float r1 = sqrtf(-2.0f * __logf(u01(w.z)));
            float sn0, cs0, sn1, cs1;
            sincospif(2.0f * u01(w.y), &sn0, &cs0);
            sincospif(2.0f * u01(w.w), &sn1, &cs1);
            z[0] = r0 * cs0; z[1] = r0 * sn0; z[2] = r1 * cs1; z[3] = r1 * sn1;
        }
#pragma unroll
        for (int e = 0; e < 4; e++) {
            if (s + e < n_diff) trow[s + e] = __expf(fmaf(ea, (float)(s + e), eb)) * z[e];
        }
    }
}

cudaError_t tail_launch(const RoomDesc *rooms, const IsmItem *rirs, int n_rir, int max_n_diff,
                        const float *pos_src, const float *pos_rcv, float *out, uint64_t seed,
                        uint64_t offset, const uint64_t *offset_ptr, int noise_kind, float *env_out,
                        cudaStream_t st) {
    if (n_rir <= 0 || max_n_diff <= 0) return cudaSuccess;
    TailLaunch p;
    p.rooms = rooms; p.rirs = rirs; p.n_rir = n_rir;
    p.pos_src = pos_src; p.pos_rcv = pos_rcv; p.out = out;
    p.seed = seed; p.offset = offset; p.offset_ptr = offset_ptr; p.noise_kind = noise_kind;
    p.env_out = env_out;
    const long chunks = ((long)max_n_diff + kTailChunk - 1) / kTailChunk;
    if (chunks > 65535) return cudaErrorInvalidValue;
    dim3 grid(n_rir, (unsigned)chunks);
    tail_kernel<<<grid, kTailThreads, 0, st>>>(p);
    return cudaGetLastError();
}

// One thread: the call offset of a captured graph advances by one per replay.
__global__ void advance_counter_kernel(uint64_t *counter) { *counter += 1; }

cudaError_t advance_counter_launch(uint64_t *counter, cudaStream_t st) {
    advance_counter_kernel<<<1, 1, 0, st>>>(counter);
    return cudaGetLastError();
}

// Raw Philox words of the tail stream of one RIR (bit-exact check against the
// host replay oracle/ism_oracle.c:orc_tail_stream).
__global__ void philox_stream_kernel(uint32_t *out, long n, uint64_t seed, uint64_t offset,
                                     uint32_t rir) {
    const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (4 * j >= n) return;
    const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    const uint4 w = philox4x32_10(
        make_uint4((uint32_t)j, rir, (uint32_t)offset, (uint32_t)(offset >> 32)), key);
    const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
    for (int e = 0; e < 4 && 4 * j + e < n; e++) out[4 * j + e] = ww[e];
}

cudaError_t philox_stream_launch(uint32_t *out, long n, uint64_t seed, uint64_t offset,
                                 uint32_t rir, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    long blocks = ((n + 3) / 4 + 255) / 256;
    philox_stream_kernel<<<(unsigned)blocks, 256, 0, st>>>(out, n, seed, offset, rir);
    return cudaGetLastError();
}

}  // namespace gpurir
