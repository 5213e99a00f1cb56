// ism_forward.cu -- fused image-source-method forward kernel for sm_103a.
//
// Replaces three stages of gpuRIR (src/gpuRIR_cuda.cu):
//   calcAmpTau_kernel   (:245-375)  image amplitudes / delays
//   generateRIR_kernel  (:377-390)  brute-force sinc evaluation over all t
//   reduceRIR_kernel    (:392-413)  tree reduction of 512-image partial sums
// by one persistent kernel that never materialises amplitudes or partial sums
// in HBM and evaluates only the taps inside the 8 ms Hann window.
//
// Work item = one RIR x one segment [t_lo, t_hi) of its early part.  Per item:
//   1. images are generated in chunks of kChunk: geometry in float-float so
//      that delays are exact to ~1e-10 samples, amplitude in FP32;
//   2. the chunk is stably counting-sorted by sub-range of the segment
//      (sub-range = SUB samples, keyed by floor(tau));
//   3. warps pull sub-ranges from a shared-memory queue; each image's taps are
//      spread over the 32 lanes (TPL taps per lane) and accumulated into a
//      buffer private to the sub-range, so no two warps touch the same word;
//   4. the segment is the sum of the (<=2) sub-range buffers covering each t,
//      in a fixed order -- results are bitwise reproducible.
// Tap value: amp * w(x) * sinc(x) with x = t - tau, written as
//   a * (-1)^k * cos^2(pi x / Tw) / x,  a = -amp sin(pi f)/pi,  tau = n0 + f,
// since sin(pi (k - f)) = -(-1)^k sin(pi f): one sinpi per image, one MUFU.RCP
// per tap, and the Hann window as an FMA polynomial (image_sample, :116-121).
#include "gpurir_internal.cuh"

namespace gpurir {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kChunk = 2048;                        // images per chunk
constexpr int kPerWarp = kChunk / kWarps;           // images per warp and chunk
constexpr int kRounds = kPerWarp / 32;              // 32-image rounds per warp and chunk
constexpr int kMaxSub = 64;                         // sub-ranges per item

struct IsmLaunch {
    const RoomDesc *rooms;
    const IsmItem *items;
    int n_items;
    const float *pos_src, *pos_rcv;   // [*, 3]
    const float *orv_src, *orv_rcv;   // [*, 3] (unused for omni rooms)
    float *out;
    int *work_counter;                // reset to 0 before every launch
    int *status;                      // device error word
    int em;                           // pad words before/after the buffers
    int max_nsub;                     // sub-ranges this launch's smem holds
    int clamp;                        // taps may fall outside |x| < H: clamp the window
};

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Taps of one image into its sub-range buffer: lane l owns taps
// k = k_lo + l + 32 i, i < TPL, at p[32 i].
template <int TPL, bool CLAMP>
__device__ __forceinline__ void scatter_taps(float *p, const float (&kf)[TPL], float al, float f,
                                             float H2, float wc0, float wc1, float wc2, float wc3) {
#pragma unroll
    for (int i = 0; i < TPL; i++) {
        const float x = kf[i] - f;
        const float z = x * x;
        float d = H2 - z;
        if (CLAMP) d = fmaxf(d, 0.0f);
        const float poly = fmaf(fmaf(fmaf(wc3, z, wc2), z, wc1), z, wc0);
        const float cw = d * poly;                  // cos(pi x / Tw)
        const float v = (cw * cw) * rcp_approx(x);  // Hann window / x
        p[32 * i] = fmaf(al, v, p[32 * i]);
    }
}

template <int TPL, bool CLAMP>
__device__ __forceinline__ void scatter_list(float *bs, int origin, const float4 *rec,
                                             const unsigned short *perm, int j0, int j1,
                                             const float (&kf)[TPL], float lane_sign, float H2,
                                             float wc0, float wc1, float wc2, float wc3) {
    if (j0 >= j1) return;
    float4 r = rec[perm[j0]];
#pragma unroll 1
    for (int j = j0; j < j1; j++) {
        const float4 cur = r;
        if (j + 1 < j1) r = rec[perm[j + 1]];   // fetch the next record while this one computes
        scatter_taps<TPL, CLAMP>(bs + (__float_as_int(cur.z) - origin), kf, cur.x * lane_sign,
                                 cur.y, H2, wc0, wc1, wc2, wc3);
    }
}

template <int TPL>
__global__ void __launch_bounds__(kThreads, 2) ism_forward_kernel(IsmLaunch P) {
    constexpr int KS = 32 * TPL;   // taps per image, rounded up to the warp
    constexpr int SUB = KS;        // sub-range length
    constexpr int BUF = SUB + KS;  // words per sub-range buffer

    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *rec = reinterpret_cast<float4 *>(smem_raw);                       // [kChunk]
    unsigned short *perm = reinterpret_cast<unsigned short *>(rec + kChunk);  // [kChunk]
    int *hist = reinterpret_cast<int *>(perm + kChunk);                        // [kWarps][kMaxSub]
    int *sub_start = hist + kWarps * kMaxSub;
    int *sub_cnt = sub_start + kMaxSub;
    int *order = sub_cnt + kMaxSub;
    int *ctl = order + kMaxSub;                                                // [0] item, [1] queue
    float *buf = reinterpret_cast<float *>(ctl + 4);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;

    for (;;) {
        if (tid == 0) ctl[0] = atomicAdd(P.work_counter, 1);
        __syncthreads();
        const int item_id = ctl[0];
        if (item_id >= P.n_items) break;
        const IsmItem it = P.items[item_id];
        const RoomDesc &R = P.rooms[it.room];
        const int t_lo = it.t_lo, t_hi = it.t_hi;
        const int nsub = (t_hi - t_lo + SUB - 1) / SUB;
        if (nsub > P.max_nsub || nsub <= 0) {   // host guarantees this; never index past smem
            if (tid == 0) atomicExch(P.status, DEV_BAD_ITEM);
            __syncthreads();
            continue;
        }
        const int buf_words = 2 * P.em + nsub * BUF;
        for (int i = tid; i < buf_words; i += kThreads) buf[i] = 0.0f;

        // Room and pair constants (uniform across the block).
        const float L0 = R.L[0], L1 = R.L[1], L2 = R.L[2];
        const int N0 = R.nb[0], N1 = R.nb[1], N2 = R.nb[2];
        const int n_img = R.n_img;
        const float H = R.H, H2 = R.H2;
        const float wc0 = R.wc[0], wc1 = R.wc[1], wc2 = R.wc[2], wc3 = R.wc[3];
        const int k_lo = (int)floorf(-H) + 1;
        const int spkr = R.spkr, mic = R.mic;
        const ff kfs = {R.kh, R.kl};
        const float sx = P.pos_src[3 * it.src], sy = P.pos_src[3 * it.src + 1],
                    sz = P.pos_src[3 * it.src + 2];
        const float rx = P.pos_rcv[3 * it.rcv], ry = P.pos_rcv[3 * it.rcv + 1],
                    rz = P.pos_rcv[3 * it.rcv + 2];
        float os0 = 0.f, os1 = 0.f, os2 = 0.f, or0 = 0.f, or1 = 0.f, or2 = 0.f;
        if (spkr != P_OMNI) {
            os0 = P.orv_src[3 * it.src]; os1 = P.orv_src[3 * it.src + 1]; os2 = P.orv_src[3 * it.src + 2];
            float inv = rsqrtf(os0 * os0 + os1 * os1 + os2 * os2);
            os0 *= inv; os1 *= inv; os2 *= inv;
        }
        if (mic != P_OMNI) {
            or0 = P.orv_rcv[3 * it.rcv]; or1 = P.orv_rcv[3 * it.rcv + 1]; or2 = P.orv_rcv[3 * it.rcv + 2];
            float inv = rsqrtf(or0 * or0 + or1 * or1 + or2 * or2);
            or0 *= inv; or1 *= inv; or2 *= inv;
        }
        const float keep_lo = (float)t_lo - H, keep_hi = (float)t_hi + H;

        // Per-lane tap constants: k = k_lo + lane + 32 i, sign (-1)^k.
        float kf[TPL];
#pragma unroll
        for (int i = 0; i < TPL; i++) kf[i] = (float)(k_lo + lane + 32 * i);
        const float lane_sign = ((k_lo + lane) & 1) ? -1.0f : 1.0f;
        int *my_hist = hist + warp * kMaxSub;

        for (int cbase = 0; cbase < n_img; cbase += kChunk) {
            // ---- pass 1: geometry of this warp's images, per-warp histogram
            for (int s = lane; s < nsub; s += 32) my_hist[s] = 0;
            __syncwarp();
#pragma unroll 1
            for (int r = 0; r < kRounds; r++) {
                const int local = warp * kPerWarp + r * 32 + lane;
                const int i = cbase + local;
                int sub = -1;
                float a = 0.f, f = 0.f;
                int n0 = 0;
                if (i < n_img) {
                    const int q = i / N2;
                    const int m2 = i - q * N2;
                    const int m0 = q / N1;
                    const int m1 = q - m0 * N1;
                    int c0, r0, c1, r1, c2, r2;
                    image_axis(m0, N0, c0, r0);
                    image_axis(m1, N1, c1, r1);
                    image_axis(m2, N2, c2, r2);
                    const float att = __ldg(&R.pw[0][abs(c0 - r0)]) * __ldg(&R.pw[1][abs(c0)]) *
                                      __ldg(&R.pw[2][abs(c1 - r1)]) * __ldg(&R.pw[3][abs(c1)]) *
                                      __ldg(&R.pw[4][abs(c2 - r2)]) * __ldg(&R.pw[5][abs(c2)]);
                    // vector receiver -> image, float-float (src/gpuRIR_cuda.cu:353)
                    const ff v0 = ff_add(ff_two_prod((float)(2 * c0), L0), ff_two_sum(r0 ? -sx : sx, -rx));
                    const ff v1 = ff_add(ff_two_prod((float)(2 * c1), L1), ff_two_sum(r1 ? -sy : sy, -ry));
                    const ff v2 = ff_add(ff_two_prod((float)(2 * c2), L2), ff_two_sum(r2 ? -sz : sz, -rz));
                    const ff d2 = ff_add(ff_add(ff_sqr(v0), ff_sqr(v1)), ff_sqr(v2));
                    const ff dist = ff_sqrt(d2);
                    const ff tau = ff_mul(dist, kfs);
                    const float inv_d = 1.0f / dist.hi;
                    float amp = att * (0.0795774715459476679f * inv_d);   // 1/(4 pi dist)
                    if (spkr != P_OMNI) {
                        // doa = image -> receiver = -vec; axis mirrored per reflection (:357-362)
                        float ct = -((r0 ? -os0 : os0) * v0.hi + (r1 ? -os1 : os1) * v1.hi +
                                     (r2 ? -os2 : os2) * v2.hi) * inv_d;
                        amp *= pattern_gain(ct, spkr);
                    }
                    if (mic != P_OMNI) {
                        float ct = (or0 * v0.hi + or1 * v1.hi + or2 * v2.hi) * inv_d;   // (:363)
                        amp *= pattern_gain(ct, mic);
                    }
                    float fl = floorf(tau.hi);
                    n0 = (int)fl;
                    f = __fadd_rn(__fsub_rn(tau.hi, fl), tau.lo);
                    if (f < 0.0f) { n0 -= 1; f += 1.0f; }
                    if (f >= 1.0f) { n0 += 1; f -= 1.0f; }
                    f = fmaxf(f, 9.094947017729282e-13f);   // 2^-40: keeps x = k - f != 0
                    a = -amp * sinpif(f) * 0.318309886183790672f;
                    if (amp != 0.0f && tau.hi > keep_lo && tau.hi < keep_hi) {
                        int rel = n0 - t_lo;
                        sub = rel < 0 ? 0 : min(rel / SUB, nsub - 1);
                    }
                }
                rec[local] = make_float4(a, f, __int_as_float(n0), __int_as_float(sub));
                const unsigned peers = __match_any_sync(0xffffffffu, sub);
                if (sub >= 0 && (peers & lt_mask) == 0) my_hist[sub] += __popc(peers);
                __syncwarp();
            }
            __syncthreads();
            // ---- warp 0: stable offsets per (warp, sub-range), starts, longest-first order
            if (warp == 0) {
                int cnt2[2], st2[2];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int s = lane + 32 * h;
                    int run = 0;
                    if (s < nsub)
                        for (int w = 0; w < kWarps; w++) {
                            const int c = hist[w * kMaxSub + s];
                            hist[w * kMaxSub + s] = run;
                            run += c;
                        }
                    cnt2[h] = run;
                }
                int x0 = cnt2[0], x1 = cnt2[1];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y0 = __shfl_up_sync(0xffffffffu, x0, o);
                    const int y1 = __shfl_up_sync(0xffffffffu, x1, o);
                    if (lane >= o) { x0 += y0; x1 += y1; }
                }
                const int tot0 = __shfl_sync(0xffffffffu, x0, 31);
                st2[0] = x0 - cnt2[0];
                st2[1] = tot0 + x1 - cnt2[1];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int s = lane + 32 * h;
                    if (s < nsub) {
                        sub_start[s] = st2[h];
                        sub_cnt[s] = cnt2[h];
                        for (int w = 0; w < kWarps; w++) hist[w * kMaxSub + s] += st2[h];
                    }
                }
                // rank by (count desc, index asc): the queue hands out heavy sub-ranges first
                int rk0 = 0, rk1 = 0;
                for (int t = 0; t < 64; t++) {
                    const int ct = __shfl_sync(0xffffffffu, cnt2[t >> 5], t & 31);
                    if (t < nsub) {
                        rk0 += (ct > cnt2[0]) || (ct == cnt2[0] && t < lane);
                        rk1 += (ct > cnt2[1]) || (ct == cnt2[1] && t < lane + 32);
                    }
                }
                if (lane < nsub) order[rk0] = lane;
                if (lane + 32 < nsub) order[rk1] = lane + 32;
                if (lane == 0) ctl[1] = 0;
            }
            __syncthreads();
            // ---- pass 2: stable permutation into sub-range order
#pragma unroll 1
            for (int r = 0; r < kRounds; r++) {
                const int local = warp * kPerWarp + r * 32 + lane;
                const int sub = __float_as_int(rec[local].w);
                const unsigned peers = __match_any_sync(0xffffffffu, sub);
                if (sub >= 0) perm[my_hist[sub] + __popc(peers & lt_mask)] = (unsigned short)local;
                __syncwarp();
                if (sub >= 0 && (peers & lt_mask) == 0) my_hist[sub] += __popc(peers);
                __syncwarp();
            }
            __syncthreads();
            // ---- pass 3: warps pull sub-ranges (heaviest first), scatter taps into private buffers
            for (;;) {
                int q = 0;
                if (lane == 0) q = atomicAdd(&ctl[1], 1);
                q = __shfl_sync(0xffffffffu, q, 0);
                if (q >= nsub) break;
                const int s = order[q];
                const int j0 = sub_start[s], j1 = j0 + sub_cnt[s];
                float *bs = buf + P.em + s * BUF + lane;
                const int origin = t_lo + s * SUB;
                if (P.clamp)
                    scatter_list<TPL, true>(bs, origin, rec, perm, j0, j1, kf, lane_sign, H2, wc0, wc1, wc2, wc3);
                else
                    scatter_list<TPL, false>(bs, origin, rec, perm, j0, j1, kf, lane_sign, H2, wc0, wc1, wc2, wc3);
            }
            __syncthreads();
        }
        // ---- output: sum of the covering sub-range buffers, ascending s
        float *orow = P.out + it.out_row;
        for (int t = t_lo + tid; t < t_hi; t += kThreads) {
            const int rel = t - t_lo;
            int s_max = (rel - k_lo) / SUB;
            if (s_max > nsub - 1) s_max = nsub - 1;
            int num = rel - k_lo - BUF + 1;   // buffer s covers rel in [s*SUB + k_lo, s*SUB + k_lo + BUF)
            int s_min = num <= 0 ? 0 : (num + SUB - 1) / SUB;
            float acc = 0.0f;
            for (int s = s_min; s <= s_max; s++) acc += buf[P.em + s * BUF + rel - s * SUB - k_lo];
            orow[t] = acc;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
size_t ism_forward_smem_bytes(int tpl, int em, int max_nsub) {
    const int ks = 32 * tpl;
    size_t fixed = kChunk * (sizeof(float4) + sizeof(unsigned short)) +
                   (kWarps * kMaxSub + 3 * kMaxSub + 4) * sizeof(int);
    return fixed + (size_t)(2 * em + max_nsub * 2 * ks) * sizeof(float);
}

int ism_forward_max_nsub(int tpl, int em, size_t smem_budget) {
    const int ks = 32 * tpl;
    size_t fixed = ism_forward_smem_bytes(tpl, em, 0);
    if (smem_budget <= fixed) return 0;
    long n = (long)((smem_budget - fixed) / (sizeof(float) * 2 * ks));
    return (int)(n < kMaxSub ? n : kMaxSub);
}

static const int kTplList[] = {2, 4, 8, 12, 16, 24};

int ism_forward_pick_tpl(float H) {
    const int k_lo = (int)floorf(-H) + 1;
    const int nk = (int)floorf(H) - k_lo + 1;
    for (int t : kTplList)
        if (32 * t >= nk) return t;
    return -1;
}

template <int TPL>
static cudaError_t launch_tpl(const IsmLaunch &p, int grid, size_t smem, cudaStream_t st) {
    static bool attr_set = false;   // per process; the attribute is per function
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(ism_forward_kernel<TPL>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    ism_forward_kernel<TPL><<<grid, kThreads, smem, st>>>(p);
    return cudaGetLastError();
}

int ism_forward_blocks_per_sm(int tpl, size_t smem) {
    int n = 0;
    switch (tpl) {
#define OCC(T) case T: cudaFuncSetAttribute(ism_forward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ism_forward_kernel<T>, kThreads, smem); break;
        OCC(2) OCC(4) OCC(8) OCC(12) OCC(16) OCC(24)
#undef OCC
    default: return 0;
    }
    return n;
}

cudaError_t ism_forward_launch(int tpl, const RoomDesc *rooms, const IsmItem *items, int n_items,
                               const float *pos_src, const float *pos_rcv, const float *orv_src,
                               const float *orv_rcv, float *out, int *work_counter, int *status,
                               int em, int max_nsub, int clamp, int grid, cudaStream_t st) {
    IsmLaunch p;
    p.rooms = rooms; p.items = items; p.n_items = n_items;
    p.pos_src = pos_src; p.pos_rcv = pos_rcv; p.orv_src = orv_src; p.orv_rcv = orv_rcv;
    p.out = out; p.work_counter = work_counter; p.status = status;
    p.em = em; p.max_nsub = max_nsub; p.clamp = clamp;
    size_t smem = ism_forward_smem_bytes(tpl, em, max_nsub);
    cudaError_t e = cudaMemsetAsync(work_counter, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    switch (tpl) {
    case 2: return launch_tpl<2>(p, grid, smem, st);
    case 4: return launch_tpl<4>(p, grid, smem, st);
    case 8: return launch_tpl<8>(p, grid, smem, st);
    case 12: return launch_tpl<12>(p, grid, smem, st);
    case 16: return launch_tpl<16>(p, grid, smem, st);
    case 24: return launch_tpl<24>(p, grid, smem, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace gpurir
