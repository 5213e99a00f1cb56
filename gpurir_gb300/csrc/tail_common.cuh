// tail_common.cuh -- diffuse-tail pieces shared by the tail kernel and the
// fused epilogue of the ISM kernel: direct-path delay, envelope parameters
// (envPred_kernel, src/gpuRIR_cuda.cu:415-443) and Philox-driven noise
// samples (diffRev_kernel, src/gpuRIR_cuda.cu:445-461).
#pragma once

#include "gpurir_internal.cuh"

namespace gpurir {

// Threads that sum the envelope-window power.  Thread j adds the squares of the
// samples t >= w_start of the groups of four t / 4 = j (mod kPowerThreads), in
// increasing t; warps then combine by an xor butterfly and thread 0 adds the warp
// sums in order.  The tail kernel and the ISM epilogue both follow this order, so
// an RIR's tail is the same bits whichever of them writes it.
constexpr int kPowerThreads = 512;

// Direct-path delay in samples, the float-float arithmetic the ISM kernel
// applies to the image with clust = refl = 0 (src/gpuRIR_cuda.cu:368-369).
__device__ __forceinline__ float direct_tau(const RoomDesc &R, const float *ps, const float *pr) {
    if (R.ref_delay) {   // the reference's float32 tau_dp (:368-369)
        const float d2 = ref_dist2(ref_axis_component(0, 0, R.L[0], ps[0], pr[0]),
                                   ref_axis_component(0, 0, R.L[1], ps[1], pr[1]),
                                   ref_axis_component(0, 0, R.L[2], ps[2], pr[2]),
                                   R.spkr != P_OMNI || R.mic != P_OMNI);
        return ref_tau(d2, R.c, R.fs);
    }
    ff v0 = ff_two_sum(ps[0], -pr[0]);
    ff v1 = ff_two_sum(ps[1], -pr[1]);
    ff v2 = ff_two_sum(ps[2], -pr[2]);
    ff d2 = ff_add(ff_add(ff_sqr(v0), ff_sqr(v1)), ff_sqr(v2));
    ff tau = ff_mul(ff_sqrt(d2), ff{R.kh, R.kl});
    return tau.hi + tau.lo;
}

// First sample of the envelope window: ceil(max(nISM - 10 ms, tau_dp)) (:419-421).
__device__ __forceinline__ int envelope_start(const RoomDesc &R, float tau_dp) {
    const float w_sz = 10e-3f * R.fs;
    return (int)ceilf(fmaxf((float)R.n_ism - w_sz, tau_dp));
}

struct TailEnv {
    float ea, eb;          // sample s of the tail: exp(eb + ea s) * noise
    float A, alpha;
};

// Envelope from the summed power of the window samples (:426-441).  An empty
// window (tau_dp >= nISM) gives A = 0: a silent tail.
__device__ __forceinline__ TailEnv tail_envelope(const RoomDesc &R, float power, int w_start,
                                                 float tau_dp) {
    TailEnv e;
    const int n_ism = R.n_ism, cnt = n_ism - w_start;
    e.alpha = -13.8155f / (R.T60 * R.fs);   // log(1e-6) / (T60 Fs)
    e.A = 0.0f;
    if (cnt > 0) {
        const float w_center = (float)w_start + (float)cnt * 0.5f;
        e.A = (power / (float)cnt) / expf(e.alpha * (w_center - tau_dp));
    }
    // sqrt(A exp(alpha (nISM + s - tau_dp))) = exp(B + alpha s / 2)
    e.ea = 0.5f * e.alpha;
    e.eb = (e.A > 0.0f) ? 0.5f * logf(e.A) + 0.5f * e.alpha * ((float)n_ism - tau_dp) : -INFINITY;
    return e;
}

// Tail samples [s_begin, s_end) of one RIR (s_begin a multiple of 4), blocks of
// four samples dealt to threads tid, tid + nthreads, ...  Counter block
// (s/4, rir, call_lo, call_hi), key (seed_lo, seed_hi).
__device__ __forceinline__ void tail_fill(float *trow, int n_diff, int s_begin, int s_end, int tid,
                                          int nthreads, float ea, float eb, uint64_t seed,
                                          uint64_t offset, uint32_t rir, int noise_kind) {
    const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    const uint32_t off_lo = (uint32_t)offset, off_hi = (uint32_t)(offset >> 32);
    const bool vec4 = ((reinterpret_cast<uintptr_t>(trow) & 15) == 0);
    const float step = __expf(ea);   // envelope ratio between consecutive samples
    const int end = min(s_end, n_diff);
    if (eb == -INFINITY) {
        // silent envelope (A = 0: no image energy in the envelope window): every sample is
        // 0 * finite noise, so the noise is not drawn
#pragma unroll 1
        for (int s = s_begin + 4 * tid; s < end; s += 4 * nthreads) {
            if (vec4 && s + 3 < end) {
                *reinterpret_cast<float4 *>(trow + s) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            } else {
#pragma unroll
                for (int e = 0; e < 4; e++)
                    if (s + e < end) trow[s + e] = 0.0f;
            }
        }
        return;
    }
#pragma unroll 1
    for (int s = s_begin + 4 * tid; s < end; s += 4 * nthreads) {
        const uint4 w = philox4x32_10(make_uint4((uint32_t)(s >> 2), rir, off_lo, off_hi), key);
        float z[4];
        if (noise_kind == 0) {
            // logistic noise of unit variance, src/gpuRIR_cuda.cu:454-455
            const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float u = u01(ww[e]);
                z[e] = 0.551329f * __logf(__fdividef(u, 1.0f - u + 1e-6f));
            }
        } else {
            const float r0 = sqrtf(-2.0f * __logf(u01(w.x)));
            const float r1 = sqrtf(-2.0f * __logf(u01(w.z)));
            float sn0, cs0, sn1, cs1;
            sincospif(2.0f * u01(w.y), &sn0, &cs0);
            sincospif(2.0f * u01(w.w), &sn1, &cs1);
            z[0] = r0 * cs0; z[1] = r0 * sn0; z[2] = r1 * cs1; z[3] = r1 * sn1;
        }
        float env = __expf(fmaf(ea, (float)s, eb));
        float v[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            v[e] = env * z[e];
            env *= step;
        }
        if (vec4 && s + 3 < end) {
            *reinterpret_cast<float4 *>(trow + s) = make_float4(v[0], v[1], v[2], v[3]);
        } else {
#pragma unroll
            for (int e = 0; e < 4; e++)
                if (s + e < end) trow[s + e] = v[e];
        }
    }
}

}  // namespace gpurir
