// tail.cu -- diffuse reverberation tail for sm_103a.
//
// Replaces envPred_kernel (src/gpuRIR_cuda.cu:415-443), the cuRAND uniform
// fill (:874) and diffRev_kernel (:445-461) by one kernel: each block predicts
// the envelope of its RIR from the last <=10 ms of the early part (already in
// the output row), then writes its chunk of the tail from a counter-based
// Philox4x32-10 stream keyed by (seed, call offset, global RIR index), so the
// noise is reproducible and needs no generator state or extra HBM pass.
#include "gpurir_internal.cuh"
#include "tail_common.cuh"

namespace gpurir {

constexpr int kTailThreads = kPowerThreads;
constexpr int kTailChunk = kTailThreads * 8;   // samples per block (2 Philox blocks/thread)

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
    const unsigned char *pre;   // optional [rir]: 1 = silent tail written elsewhere (TailArgs::pre)
};

__global__ void __launch_bounds__(kTailThreads) tail_kernel(TailLaunch P) {
    const int rir = blockIdx.x;
    if (rir >= P.n_rir) return;
    const IsmItem it = P.rirs[rir];
    if (it.t_hi < 0) return;   // this RIR's tail was written by the ISM kernel's epilogue
    const RoomDesc &R = P.rooms[it.room];
    const int n_ism = R.n_ism, n_diff = R.n_total - R.n_ism;
    const int s0 = blockIdx.y * kTailChunk;
    if (s0 >= n_diff) return;
    float *row = P.out + it.out_row;

    __shared__ float red[kTailThreads / 32];
    __shared__ float envA, envB;
    const float tau_dp = direct_tau(R, P.pos_src + 3 * it.src, P.pos_rcv + 3 * it.rcv);
    const int w_start = envelope_start(R, tau_dp);
    float p = 0.0f;
    for (int t0 = (w_start / (4 * kTailThreads)) * (4 * kTailThreads) + 4 * threadIdx.x; t0 < n_ism;
         t0 += 4 * kTailThreads) {
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int t = t0 + e;
            if (t >= w_start && t < n_ism) {
                const float v = row[t];
                p = fmaf(v, v, p);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = p;
    __syncthreads();
    if (threadIdx.x == 0) {
        float tot = 0.0f;
        for (int w = 0; w < kTailThreads / 32; w++) tot += red[w];
        const TailEnv e = tail_envelope(R, tot, w_start, tau_dp);
        envA = e.ea;
        envB = e.eb;
        if (P.env_out && blockIdx.y == 0) {
            P.env_out[3 * rir] = e.A;
            P.env_out[3 * rir + 1] = e.alpha;
            P.env_out[3 * rir + 2] = tau_dp;
        }
    }
    __syncthreads();
    if (P.pre && P.pre[it.rir]) return;   // silent (A = 0 above) and streamed by the caller
    const uint64_t offset = P.offset_ptr ? *P.offset_ptr : P.offset;
    tail_fill(row + n_ism, n_diff, s0, s0 + kTailChunk, threadIdx.x, kTailThreads, envA, envB, P.seed,
              offset, (uint32_t)it.rir, P.noise_kind);
}

cudaError_t tail_launch(const RoomDesc *rooms, const IsmItem *rirs, int n_rir, int max_n_diff,
                        const float *pos_src, const float *pos_rcv, float *out, uint64_t seed,
                        uint64_t offset, const uint64_t *offset_ptr, int noise_kind, float *env_out,
                        cudaStream_t st, const unsigned char *pre) {
    if (n_rir <= 0 || max_n_diff <= 0) return cudaSuccess;
    TailLaunch p;
    p.rooms = rooms; p.rirs = rirs; p.n_rir = n_rir;
    p.pos_src = pos_src; p.pos_rcv = pos_rcv; p.out = out;
    p.seed = seed; p.offset = offset; p.offset_ptr = offset_ptr; p.noise_kind = noise_kind;
    p.env_out = env_out;
    p.pre = pre;
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
