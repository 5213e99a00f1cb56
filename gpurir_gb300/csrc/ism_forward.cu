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
// per tap, and the Hann window by the angle-sum identity from per-lane
// constants and a per-image (cos, sin) pair (image_sample, :116-121).
#include <cuda_fp16.h>

#include <map>
#include <mutex>

#include "gpurir_internal.cuh"
#include "tail_common.cuh"

namespace gpurir {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kChunk = 2048;                        // images per chunk
constexpr int kPerWarp = kChunk / kWarps;           // images per warp and chunk
constexpr int kRounds = kPerWarp / 32;              // 32-image rounds per warp and chunk
constexpr int kMaxSub = 64;                         // sub-ranges per item
constexpr int kPool = kWarps;                       // extra slices of heavy sub-ranges per chunk
constexpr int kMaxItems = 128;                      // >= kMaxSub + kPool queue entries
constexpr short kNoImage = -32768;                  // record of an image outside the segment
static_assert(kPerWarp <= 256, "ranks within a warp's bucket are stored in 8 bits");
static_assert(kThreads == kPowerThreads, "the fused tail sums the window power in the tail kernel's order");

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
    int tw;                           // window length in samples (LUT mode table)
    // diffuse tail written by the epilogue of single-segment items (see TailArgs)
    uint64_t seed, offset;
    const uint64_t *offset_ptr;
    int noise_kind;
    float *env_out;
    int fuse_tail;
    // per-axis image terms of the current item, one region of axis_cap entries per block
    // (global memory, L1-resident): {v^2 hi, v^2 lo, v hi, attenuation} for m < N0, then
    // N1, then N2 entries.  nullptr: computed per image instead.
    float4 *axis_tab;
    int axis_cap;
    float *partial;   // partial segments of items holding a part of an RIR's images
    const unsigned char *skip;   // per item: 1 = no image reaches its segment (nullptr: none)
    const unsigned char *tail_pre;   // per RIR: 1 = silent tail written elsewhere (TailArgs::pre)
};

// Evaluation modes of the taps (template parameter MODE):
//   kModeF32  FP32 Hann window by the angle-sum identity (default)
//   kModeMP   mixed precision: the window evaluated in packed half2, reciprocal
//             and accumulation in FP32 (gpuRIR's activateMixedPrecision,
//             src/gpuRIR_cuda.cu:488-553 evaluates in half2 and also accumulates in half2)
//   kModeLUT  gpuRIR's lookup table (src/gpuRIR_cuda.cu:236-239, 578-616): Hann x sinc
//             sampled 16x per sample, fetched at gpuRIR's float coordinate with the
//             linear filter of a GB300 texture unit (8-bit weight, rounded half up),
//             support |x| < floor(Tw/2)
constexpr int kModeF32 = 0, kModeMP = 1, kModeLUT = 2;
// Flag added to a mode: compensated accumulation across chunks.  Each chunk's taps
// still go into the FP32 sub-range buffers (few terms per sample per chunk), and
// after the chunk every touched word is added into a running (hi, lo) pair by
// TwoSum (Knuth TAOCP vol. 2, 4.2.2) and cleared, so the error of a late, dense
// sample stops growing with the number of images that reach it.  Used for the
// lookup-table mode on long RIRs, and on request in mixed precision (capi.cu
// gpurir_set_compensation).
constexpr int kModeComp = 4;
constexpr int kLutOversamp = 16;

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Taps of one image into its sub-range buffer: lane l owns taps
// k = k_lo + l + 32 i, i < TPL, at p[32 i].  With x = k - f the Hann window is
//   0.5 (1 + cos(2 pi x / Tw)) = 0.5 + [0.5 cos(2 pi k/Tw)] cos(phi) + [0.5 sin(2 pi k/Tw)] sin(phi),
// phi = 2 pi f / Tw: the bracketed factors are per-lane constants (ck, sk) and
// (cos phi, sin phi) comes with the image.  In FP32 mode the image's amplitude is
// folded in as well: the record holds (a, f, a cos phi, a sin phi), ck and sk carry
// the lane's sign (-1)^k, and al = 0.5 a (-1)^k, so a tap is
//   acc += (al + ck (a cos phi) + sk (a sin phi)) / x:
// one FADD, two FFMA, one MUFU.RCP, one FFMA and the shared-memory read and write.
template <int TPL, bool CLAMP, int MODE>
__device__ __forceinline__ void scatter_taps(float *p, const float (&kf)[TPL], const float (&ck)[TPL],
                                             const float (&sk)[TPL], float al, float4 r, float H,
                                             const float2 *lut, int lut_cols) {
    const float f = r.y;
    if (MODE == kModeF32 && (TPL % 2) == 0 && TPL <= 12) {   // (more taps per lane: register spills)
        // taps i and i + 1 of the lane in packed FP32 (Blackwell's two-wide FADD/FFMA,
        // each half rounded as the scalar instruction): the image's values are
        // duplicated once, the lane constants pair up as they lie in registers
        const float2 f2 = make_float2(-f, -f), ac2 = make_float2(r.z, r.z), as2 = make_float2(r.w, r.w);
        const float2 al2 = make_float2(al, al);
#pragma unroll
        for (int i = 0; i < TPL; i += 2) {
            const float2 x = __fadd2_rn(make_float2(kf[i], kf[i + 1]), f2);
            float2 u = __ffma2_rn(make_float2(ck[i], ck[i + 1]), ac2,
                                  __ffma2_rn(make_float2(sk[i], sk[i + 1]), as2, al2));
            if (CLAMP) {
                u.x = fabsf(x.x) < H ? u.x : 0.0f;
                u.y = fabsf(x.y) < H ? u.y : 0.0f;
            }
            const float2 acc = __ffma2_rn(u, make_float2(rcp_approx(x.x), rcp_approx(x.y)),
                                          make_float2(p[32 * i], p[32 * (i + 1)]));
            p[32 * i] = acc.x;
            p[32 * (i + 1)] = acc.y;
        }
    } else if (MODE == kModeF32) {
        const float ac = r.z, as = r.w;   // a cos phi, a sin phi
#pragma unroll
        for (int i = 0; i < TPL; i++) {
            const float x = kf[i] - f;
            float u = fmaf(ck[i], ac, fmaf(sk[i], as, al));
            if (CLAMP) u = fabsf(x) < H ? u : 0.0f;
            p[32 * i] = fmaf(u, rcp_approx(x), p[32 * i]);
        }
    } else if (MODE == kModeMP) {
        const __half2 cphi = __float2half2_rn(r.z), sphi = __float2half2_rn(r.w);
        const __half2 half = __float2half2_rn(0.5f);
#pragma unroll
        for (int i = 0; i < TPL; i += 2) {
            const __half2 ck2 = __floats2half2_rn(ck[i], ck[i + 1]);
            const __half2 sk2 = __floats2half2_rn(sk[i], sk[i + 1]);
            const float2 w = __half22float2(__hfma2(ck2, cphi, __hfma2(sk2, sphi, half)));
            const float x0 = kf[i] - f, x1 = kf[i + 1] - f;
            float v0 = w.x * rcp_approx(x0), v1 = w.y * rcp_approx(x1);
            if (CLAMP) { v0 = fabsf(x0) < H ? v0 : 0.0f; v1 = fabsf(x1) < H ? v1 : 0.0f; }
            p[32 * i] = fmaf(al, v0, p[32 * i]);
            p[32 * (i + 1)] = fmaf(al, v1, p[32 * (i + 1)]);
        }
    } else {
        // gpuRIR's fetch (image_sample_lut, src/gpuRIR_cuda.cu:236-239) in its float
        // arithmetic: record al = amp, r.y = f with tau = n0 + f exactly in float32, so
        // x = k - f rounds as the reference's t - tau does; texel position
        // __fmaf_rz(x, 16, 8 Tw + 0.5) - 0.5; the upper texel's weight on 8 fractional
        // bits rounded half up, as GB300 texture units filter; border texels are 0.
        // Without CLAMP every tap has -H < x <= H = Tw/2 (window of exactly 32 TPL taps),
        // so the texel index lies in [0, 16 Tw] and its clamp changes nothing; the support
        // test stays (x = H when tau is an integer).
        const float lut_c = (float)(kLutOversamp / 2 * (lut_cols - 1)) + 0.5f;
        const int j_max = kLutOversamp * (lut_cols - 1);
#pragma unroll
        for (int i = 0; i < TPL; i++) {
            const float x = kf[i] - f;
            const float xb = __fmaf_rz(x, (float)kLutOversamp, lut_c) - 0.5f;
            const float jf = floorf(xb);
            const float y = (xb - jf) * 256.0f;   // exact
            // round half up to 8 bits: floor(y + 1/2), the sum rounded down so that an
            // inexact y + 1/2 never reaches the next integer
            const float w = floorf(__fadd_rd(y, 0.5f)) * (1.0f / 256.0f);
            int j = (int)jf;
            if (CLAMP) j = min(max(j, 0), j_max);
            const float2 t = lut[(j & (kLutOversamp - 1)) * lut_cols + (j >> 4)];
            float v = fmaf(w, t.y - t.x, t.x);
            v = fabsf(x) < H ? v : 0.0f;
            p[32 * i] = fmaf(al, v, p[32 * i]);
        }
    }
}

template <int TPL, bool CLAMP, int MODE>
__device__ __forceinline__ void scatter_list(float *bs, int origin, const float4 *rec, const short *rec_n0,
                                             int j0, int j1,
                                             const float (&kf)[TPL], const float (&ck)[TPL],
                                             const float (&sk)[TPL], float lane_sign, float H,
                                             const float2 *lut, int lut_cols) {
    int j = j0;
#pragma unroll 1
    for (; j + 1 < j1; j += 2) {   // two images per trip: half the loop bookkeeping
        const float4 a = rec[j], b = rec[j + 1];
        const int na = rec_n0[j], nb = rec_n0[j + 1];
        scatter_taps<TPL, CLAMP, MODE>(bs + (na - origin), kf, ck, sk, a.x * lane_sign, a, H, lut, lut_cols);
        scatter_taps<TPL, CLAMP, MODE>(bs + (nb - origin), kf, ck, sk, b.x * lane_sign, b, H, lut, lut_cols);
    }
    if (j < j1) {
        const float4 a = rec[j];
        scatter_taps<TPL, CLAMP, MODE>(bs + (rec_n0[j] - origin), kf, ck, sk, a.x * lane_sign, a, H, lut,
                                       lut_cols);
    }
}

template <int TPL, int MODE_ARG>
__global__ void __launch_bounds__(kThreads, 2) ism_forward_kernel(IsmLaunch P) {
    constexpr int MODE = MODE_ARG & 3;                  // tap evaluation
    constexpr bool COMP = (MODE_ARG & kModeComp) != 0;  // compensated accumulation across chunks
    constexpr int KS = 32 * TPL;   // taps per image, rounded up to the warp
    constexpr int SUB = KS;        // sub-range length
    constexpr int BUF = SUB + KS;  // words per sub-range buffer

    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *rec = reinterpret_cast<float4 *>(smem_raw);            // [kChunk] a, f, cos phi, sin phi
    short *rec_n0 = reinterpret_cast<short *>(rec + kChunk);        // [kChunk] floor(tau) - t_lo
    // [kChunk] rank of the image among its warp's images of the same sub-range (< kPerWarp)
    unsigned char *rec_rank = reinterpret_cast<unsigned char *>(rec_n0 + kChunk);
    int *hist = reinterpret_cast<int *>(rec_rank + kChunk);         // [kWarps][kMaxSub]
    int *sub_start = hist + kWarps * kMaxSub;
    int *sub_cnt = sub_start + kMaxSub;
    int *pool_base = sub_cnt + kMaxSub;                                        // first pool slot of s
    int *order = pool_base + kMaxSub;                                          // [kMaxItems] s | k << 8
    int *slot_sub = order + kMaxItems;                                         // [kPool]
    int *ctl = slot_sub + kPool;   // [0] item, [1] queue, [2] queue length, [3] pool slots, [4] cap
    float *buf = reinterpret_cast<float *>(ctl + 8);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    // LUT mode: the table after the largest buffers + pool of this launch, rows of
    // (T[16 col + row], T[16 col + row + 1]) pairs so that lanes read consecutive words.
    const int lut_cols = P.tw + 1;
    // compensated mode: running sums (hi) and their errors (lo), laid out as buf
    const int comp_words = COMP ? 2 * P.em + P.max_nsub * BUF : 0;
    float *hi = buf + 2 * P.em + P.max_nsub * BUF + kPool * (2 * P.em + BUF);
    float *lo = hi + comp_words;
    float2 *lut = reinterpret_cast<float2 *>(
        buf + ((2 * P.em + P.max_nsub * BUF + kPool * (2 * P.em + BUF) + 2 * comp_words + 1) & ~1));
    if (MODE == kModeLUT) {
        // T[j] = Hann x sinc at (j - 8 Tw) / 16, as src/gpuRIR_cuda.cu:578-592 tabulates it
        const int center = 8 * P.tw, lut_len = 16 * P.tw + 1;
        const float PIf = 3.141592654f, twf = (float)P.tw;
        for (int e = tid; e < kLutOversamp * lut_cols; e += kThreads) {
            const int row = e / lut_cols, col = e - row * lut_cols;
            float v[2];
            for (int u = 0; u < 2; u++) {
                const int j = kLutOversamp * col + row + u;
                v[u] = 0.0f;
                if (j < lut_len) {
                    const float x = (float)abs(j - center) / (float)kLutOversamp;
                    const float sc = (x == 0.0f) ? 1.0f : sinf(PIf * x) / (PIf * x);
                    v[u] = 0.5f * (1.0f + cosf(2.0f * PIf * x / twf)) * sc;
                }
            }
            lut[row * lut_cols + col] = make_float2(v[0], v[1]);
        }
        __syncthreads();
    }
    const float h_lut = (float)(P.tw / 2);   // gpuRIR's LUT support |t - tau| < Tw/2 (integer)

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
        const int slot_words = 2 * P.em + BUF;
        float *pool = buf + buf_words;   // kPool slots of [em | BUF | em]
        for (int i = tid; i < buf_words + kPool * slot_words; i += kThreads) buf[i] = 0.0f;
        if (COMP)
            for (int i = tid; i < buf_words; i += kThreads) hi[i] = lo[i] = 0.0f;

        // Room and pair constants (uniform across the block).
        const float L0 = R.L[0], L1 = R.L[1], L2 = R.L[2];
        const int N0 = R.nb[0], N1 = R.nb[1], N2 = R.nb[2];
        const int n_img = R.n_img;
        const float H = R.H;
        const float inv_h = 1.0f / H;
        const float rN1 = 1.0f / (float)N1, rN2 = 1.0f / (float)N2;
        // delays in the reference's float32 arithmetic instead of the exact ones
        const bool ref_delay = R.ref_delay != 0;
        const bool ref_dir = R.spkr != P_OMNI || R.mic != P_OMNI;
        const bool small_phi = inv_h <= 0.0625f;   // window angle f / H <= 1/16: polynomials
        // per-axis terms once per item: an image's squared distance is then two
        // float-float additions (the same operations, in the same order, as per image)
        // an item whose segment no image of its pair reaches (the zeros after the last
        // image of a long RIR) only writes zeros: no axis table, no chunks (flags from
        // item_skip_kernel, launched before this kernel when the plan has later segments)
        const bool miss = P.skip != nullptr && P.skip[item_id] != 0;
        float4 *tab = P.axis_tab ? P.axis_tab + (size_t)blockIdx.x * P.axis_cap : nullptr;
        const bool use_tab = tab && N0 + N1 + N2 <= P.axis_cap && !miss;
        if (use_tab) {
            for (int e = tid; e < N0 + N1 + N2; e += kThreads) {
                const int a = e < N0 ? 0 : (e < N0 + N1 ? 1 : 2);
                const int m = e - (a == 0 ? 0 : (a == 1 ? N0 : N0 + N1));
                const int Na = a == 0 ? N0 : (a == 1 ? N1 : N2);
                const float La = a == 0 ? L0 : (a == 1 ? L1 : L2);
                const float sa = a == 0 ? P.pos_src[3 * it.src] : (a == 1 ? P.pos_src[3 * it.src + 1] : P.pos_src[3 * it.src + 2]);
                const float ra = a == 0 ? P.pos_rcv[3 * it.rcv] : (a == 1 ? P.pos_rcv[3 * it.rcv + 1] : P.pos_rcv[3 * it.rcv + 2]);
                int ca, fa;
                image_axis(m, Na, ca, fa);
                const float att = R.pw[2 * a][abs(ca - fa)] * R.pw[2 * a + 1][abs(ca)];
                if (ref_delay) {   // the reference's float32 component; its square only bounds
                    const float v = ref_axis_component(ca, fa, La, sa, ra);
                    tab[e] = make_float4(v * v, 0.0f, v, att);
                } else {
                    const ff v = ff_add(ff_two_prod((float)(2 * ca), La), ff_two_sum(fa ? -sa : sa, -ra));
                    const ff sq = ff_sqr(v);
                    tab[e] = make_float4(sq.hi, sq.lo, v.hi, att);
                }
            }
            __syncthreads();
        }
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

        // a partial item writes its segment at part_off (sample t_lo first)
        float *orow = it.part_off >= 0 ? P.partial + it.part_off - t_lo : P.out + it.out_row;
        const bool fuse = P.fuse_tail && it.part_off < 0 && t_lo == 0 && t_hi == R.n_ism &&
                          R.n_total > R.n_ism;
        float tau_dp = 0.0f;
        int w_start = t_hi;
        if (fuse) {
            tau_dp = direct_tau(R, P.pos_src + 3 * it.src, P.pos_rcv + 3 * it.rcv);
            w_start = envelope_start(R, tau_dp);
        }
        // When no image of the pair can reach the envelope window [w_start, nISM), the
        // window's samples are exact zeros, the envelope is A = 0 and the tail is silent
        // whatever the rest of the early part holds.  An item of the first wave (the
        // first gridDim.x handed out) writes such a tail now, the same values as after
        // the early part: while the first items compute nothing else is being stored,
        // so these stores (over the host link when the caller's buffer is in host
        // memory) overlap the tap work.  Later items keep the tail for the end, where
        // earlier items' stores already keep the link busy (mic_array into host memory:
        // 0.79 ms instead of 0.83 ms; no change into HBM).
        bool tail_written = false;
        if (fuse && P.tail_pre && P.tail_pre[it.rir]) {
            // the caller streams this silent tail itself: only its envelope (A = 0) here
            const TailEnv e = tail_envelope(R, 0.0f, w_start, tau_dp);
            if (tid == 0 && P.env_out) {
                P.env_out[3 * it.rir] = e.A;
                P.env_out[3 * it.rir + 1] = e.alpha;
                P.env_out[3 * it.rir + 2] = tau_dp;
            }
            tail_written = true;
        } else if (fuse && item_id < (int)gridDim.x) {
            const float s3[3] = {sx, sy, sz}, r3[3] = {rx, ry, rz};
            if (images_miss_segment(R.L, R.nb, s3, r3, R.kh, H, w_start, R.n_ism)) {
                const TailEnv e = tail_envelope(R, 0.0f, w_start, tau_dp);
                if (tid == 0 && P.env_out) {
                    P.env_out[3 * it.rir] = e.A;
                    P.env_out[3 * it.rir + 1] = e.alpha;
                    P.env_out[3 * it.rir + 2] = tau_dp;
                }
                const uint64_t offset = P.offset_ptr ? *P.offset_ptr : P.offset;
                tail_fill(orow + R.n_ism, R.n_total - R.n_ism, 0, R.n_total - R.n_ism, tid, kThreads, e.ea,
                          e.eb, P.seed, offset, (uint32_t)it.rir, P.noise_kind);
                tail_written = true;
            }
        }

        // Per-lane tap constants: k = k_lo + lane + 32 i, sign (-1)^k.
        float kf[TPL], ck[TPL], sk[TPL];
#pragma unroll
        for (int i = 0; i < TPL; i++) {
            kf[i] = (float)(k_lo + lane + 32 * i);
            float sn, cs;
            sincospif(kf[i] * inv_h, &sn, &cs);   // 2 pi k / Tw = pi k / H
            ck[i] = 0.5f * cs;
            sk[i] = 0.5f * sn;
            if (MODE == kModeF32 && ((k_lo + lane) & 1)) { ck[i] = -ck[i]; sk[i] = -sk[i]; }
        }
        // (-1)^k of the lane's taps, times 1/2 in FP32 mode (the window's constant term)
        const float lane_sign = (((k_lo + lane) & 1) ? -1.0f : 1.0f) * (MODE == kModeF32 ? 0.5f : 1.0f);
        int *my_hist = hist + warp * kMaxSub;

        // Chunks whose rows (fixed m0, m1) all lie farther from the receiver than the
        // segment's latest delay reaches, in the xy-plane alone, hold no image of the
        // segment: skipped whole (a conservative test on the tables' leading parts).
        const float d_hi = (keep_hi + 2.0f) / kfs.hi + 0.01f;
        const float dhi2 = d_hi * d_hi;
        // |component| <= (|k| + 1) L on each axis: when even the farthest row is within
        // reach, nothing can be skipped and the test is not made
        const float x_max = (float)(N0 / 2 + 1) * L0, y_max = (float)(N1 / 2 + 1) * L1;
        const bool may_skip = use_tab && x_max * x_max + y_max * y_max > dhi2;
        const int i_end = miss ? it.i_lo : min(it.i_hi, n_img);   // this item's images: [i_lo, i_end)
        for (int cbase = it.i_lo; cbase < i_end; cbase += kChunk) {
            if (may_skip) {
                const int q_first = cbase / N2, q_last = (min(cbase + kChunk, i_end) - 1) / N2;
                int hit = 0;
                for (int q = q_first + tid; q <= q_last && !hit; q += kThreads) {
                    int m0, m1;
                    divmod_small(q, N1, rN1, m0, m1);
                    hit = tab[m0].x + tab[N0 + m1].x <= dhi2;
                }
                if (!__syncthreads_or(hit)) continue;
            }
            // ---- pass 1: geometry of this warp's images, per-warp histogram
            for (int s = lane; s < nsub; s += 32) my_hist[s] = 0;
            __syncwarp();
#pragma unroll 2
            for (int r = 0; r < kRounds; r++) {
                const int local = warp * kPerWarp + r * 32 + lane;
                const int i = cbase + local;
                int sub = -1;
                float a = 0.f, f = 0.f, sphi = 0.f, cphi = 1.f;
                int n0 = 0;
                if (i < i_end) {
                    int q, m2, m0, m1;
                    divmod_small(i, N2, rN2, q, m2);
                    divmod_small(q, N1, rN1, m0, m1);
                    int c0, r0, c1, r1, c2, r2;
                    image_axis(m0, N0, c0, r0);
                    image_axis(m1, N1, c1, r1);
                    image_axis(m2, N2, c2, r2);
                    // vector receiver -> image, float-float (src/gpuRIR_cuda.cu:353)
                    ff d2;
                    float v0h, v1h, v2h, att_t = 0.0f;
                    if (use_tab) {
                        const float4 t0 = tab[m0], t1 = tab[N0 + m1], t2 = tab[N0 + N1 + m2];
                        d2 = ff_add(ff_add(ff{t0.x, t0.y}, ff{t1.x, t1.y}), ff{t2.x, t2.y});
                        v0h = t0.z; v1h = t1.z; v2h = t2.z;
                        att_t = t0.w * t1.w * t2.w;
                        if (ref_delay) d2 = ff{ref_dist2(v0h, v1h, v2h, ref_dir), 0.0f};
                    } else if (ref_delay) {
                        v0h = ref_axis_component(c0, r0, L0, sx, rx);
                        v1h = ref_axis_component(c1, r1, L1, sy, ry);
                        v2h = ref_axis_component(c2, r2, L2, sz, rz);
                        d2 = ff{ref_dist2(v0h, v1h, v2h, ref_dir), 0.0f};
                    } else {
                        const ff v0 = ff_add(ff_two_prod((float)(2 * c0), L0), ff_two_sum(r0 ? -sx : sx, -rx));
                        const ff v1 = ff_add(ff_two_prod((float)(2 * c1), L1), ff_two_sum(r1 ? -sy : sy, -ry));
                        const ff v2 = ff_add(ff_two_prod((float)(2 * c2), L2), ff_two_sum(r2 ? -sz : sz, -rz));
                        d2 = ff_add(ff_add(ff_sqr(v0), ff_sqr(v1)), ff_sqr(v2));
                        v0h = v0.hi; v1h = v1.hi; v2h = v2.hi;
                    }
                    // approximate distance first: images whose delay is far outside this
                    // segment (a third of them in a room's corner regions) stop here
                    const float rs0 = rsqrtf(d2.hi);
                    const float s0 = d2.hi * rs0;
                    const float tau_est = s0 * kfs.hi;
                    if (tau_est > keep_lo - 1.0f && tau_est < keep_hi + 1.0f) {
                        const float att = use_tab ? att_t :
                                          __ldg(&R.pw[0][abs(c0 - r0)]) * __ldg(&R.pw[1][abs(c0)]) *
                                          __ldg(&R.pw[2][abs(c1 - r1)]) * __ldg(&R.pw[3][abs(c1)]) *
                                          __ldg(&R.pw[4][abs(c2 - r2)]) * __ldg(&R.pw[5][abs(c2)]);
                        // distance = s0 + (d2 - s0^2) / (2 s0): one Newton step in float-float
                        // (the residual by FMA is exact to ~1e-14 of d2)
                        float inv_d;
                        const ff dist = ff_dist_newton(d2, rs0, s0, inv_d);
                        const ff tau = ref_delay ? ff{ref_tau(d2.hi, R.c, R.fs), 0.0f} : ff_mul(dist, kfs);
                        float amp = att * (0.0795774715459476679f * inv_d);   // 1/(4 pi dist)
                        if (spkr != P_OMNI) {
                            // doa = image -> receiver = -vec; axis mirrored per reflection (:357-362)
                            float ct = -((r0 ? -os0 : os0) * v0h + (r1 ? -os1 : os1) * v1h +
                                         (r2 ? -os2 : os2) * v2h) * inv_d;
                            amp *= pattern_gain(ct, spkr);
                        }
                        if (mic != P_OMNI) {
                            float ct = (or0 * v0h + or1 * v1h + or2 * v2h) * inv_d;   // (:363)
                            amp *= pattern_gain(ct, mic);
                        }
                        float fl = floorf(tau.hi);
                        n0 = (int)fl;
                        f = __fadd_rn(__fsub_rn(tau.hi, fl), tau.lo);
                        if (f < 0.0f) { n0 -= 1; f += 1.0f; }
                        if (f >= 1.0f) { n0 += 1; f -= 1.0f; }
                        f = fmaxf(f, 9.094947017729282e-13f);   // 2^-40: keeps x = k - f != 0
                        if (MODE == kModeLUT) {
                            // the reference stores tau as a float: split its nearest float
                            fl = floorf(tau.hi);
                            n0 = (int)fl;
                            f = tau.hi - fl;   // exact
                            a = amp;
                        } else {
                            a = -amp * sinpi_unit(f) * 0.318309886183790672f;
                            if (small_phi) sincospi_small(f * inv_h, sphi, cphi);   // phi = 2 pi f / Tw
                            else sincospif(f * inv_h, &sphi, &cphi);
                            if (MODE == kModeF32) { cphi *= a; sphi *= a; }   // record a cos phi, a sin phi
                        }
                        if (amp != 0.0f && tau.hi > keep_lo && tau.hi < keep_hi) {
                            int rel = n0 - t_lo;
                            sub = rel < 0 ? 0 : min(rel / SUB, nsub - 1);
                        }
                    }
                }
                rec[local] = make_float4(a, f, cphi, sphi);
                // n0 - t_lo (|.| < 2^15: host caps segments), kNoImage for images outside
                rec_n0[local] = (short)(sub >= 0 ? n0 - t_lo : kNoImage);
                const unsigned peers = __match_any_sync(0xffffffffu, sub);
                const int rank = sub >= 0 ? my_hist[sub] + __popc(peers & lt_mask) : 0;
                __syncwarp();
                if (sub >= 0 && (peers & lt_mask) == 0) my_hist[sub] += __popc(peers);
                rec_rank[local] = (unsigned char)rank;
                __syncwarp();
            }
            __syncthreads();
            // ---- warp 0: stable offsets per (warp, sub-range); split sub-ranges heavier than a
            //      warp's share into slices; queue full slices first, then the rest by size
            if (warp == 0) {
                int cnt2[2], st2[2];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int s = lane + 32 * h;
                    int run = 0;
                    if (s < nsub) {
                        int c[kWarps];   // independent loads, then the running sum in registers
#pragma unroll
                        for (int w = 0; w < kWarps; w++) c[w] = hist[w * kMaxSub + s];
#pragma unroll
                        for (int w = 0; w < kWarps; w++) {
                            hist[w * kMaxSub + s] = run;
                            run += c[w];
                        }
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
                const int total = tot0 + __shfl_sync(0xffffffffu, x1, 31);
                st2[0] = x0 - cnt2[0];
                st2[1] = tot0 + x1 - cnt2[1];
                const int cap = max(1, (total + kWarps - 1) / kWarps);
                int full2[2], rem2[2], ext2[2];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    full2[h] = cnt2[h] / cap;
                    rem2[h] = cnt2[h] - full2[h] * cap;
                    ext2[h] = max(full2[h] + (rem2[h] > 0) - 1, 0);   // slices beyond the first
                }
                // exclusive scans of full slices and extra slices over s = 0..63
                int f0 = full2[0], f1 = full2[1], e0 = ext2[0], e1 = ext2[1];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int a0 = __shfl_up_sync(0xffffffffu, f0, o), a1 = __shfl_up_sync(0xffffffffu, f1, o);
                    const int b0 = __shfl_up_sync(0xffffffffu, e0, o), b1 = __shfl_up_sync(0xffffffffu, e1, o);
                    if (lane >= o) { f0 += a0; f1 += a1; e0 += b0; e1 += b1; }
                }
                const int ftot0 = __shfl_sync(0xffffffffu, f0, 31), etot0 = __shfl_sync(0xffffffffu, e0, 31);
                const int n_full = ftot0 + __shfl_sync(0xffffffffu, f1, 31);
                const int n_extra = etot0 + __shfl_sync(0xffffffffu, e1, 31);
                const int fpre[2] = {f0 - full2[0], ftot0 + f1 - full2[1]};
                const int epre[2] = {e0 - ext2[0], etot0 + e1 - ext2[1]};
                // remainder slices: those of at least half a slice first, then the smaller
                // ones, each class in s order (ballot ranks: no serial loop)
                const int half = (cap + 1) / 2;
                const bool v0 = lane < nsub, v1 = lane + 32 < nsub;
                const unsigned a0 = __ballot_sync(0xffffffffu, v0 && rem2[0] >= half);
                const unsigned a1 = __ballot_sync(0xffffffffu, v1 && rem2[1] >= half);
                const unsigned b0 = __ballot_sync(0xffffffffu, v0 && rem2[0] > 0 && rem2[0] < half);
                const unsigned b1 = __ballot_sync(0xffffffffu, v1 && rem2[1] > 0 && rem2[1] < half);
                const int n_a = __popc(a0) + __popc(a1);
                const int n_rem = n_a + __popc(b0) + __popc(b1);
                int rk[2];
                rk[0] = rem2[0] >= half ? __popc(a0 & lt_mask) : n_a + __popc(b0 & lt_mask);
                rk[1] = rem2[1] >= half ? __popc(a0) + __popc(a1 & lt_mask)
                                        : n_a + __popc(b0) + __popc(b1 & lt_mask);
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int s = lane + 32 * h;
                    if (s < nsub) {
                        sub_start[s] = st2[h];
                        sub_cnt[s] = cnt2[h];
                        pool_base[s] = epre[h];
                        for (int k = 0; k < full2[h]; k++) order[fpre[h] + k] = s | (k << 8);
                        if (rem2[h] > 0) order[n_full + rk[h]] = s | (full2[h] << 8);
                        for (int k = 0; k < ext2[h]; k++) slot_sub[epre[h] + k] = s;
                    }
                }
                if (lane == 0) {
                    ctl[1] = 0;
                    ctl[2] = n_full + n_rem;
                    ctl[3] = n_extra;
                    ctl[4] = cap;
                }
            }
            __syncthreads();
            // ---- pass 2: stable permutation into sub-range order, in place: each thread
            //      holds its images' records in registers across a barrier, then stores
            //      them at their sorted positions (pass 3 reads them in order)
            {
                float4 rv[kRounds];
                short nv[kRounds];
                int dst[kRounds];
#pragma unroll
                for (int r = 0; r < kRounds; r++) {
                    const int local = warp * kPerWarp + r * 32 + lane;
                    const int rel = rec_n0[local];
                    rv[r] = rec[local];
                    nv[r] = (short)rel;
                    dst[r] = -1;
                    if (rel != kNoImage) {   // the sub-range as pass 1 derived it from rel
                        const int sub = rel < 0 ? 0 : min(rel / SUB, nsub - 1);
                        // sub-range start + this warp's offset in it + rank among its images
                        dst[r] = sub_start[sub] + my_hist[sub] + rec_rank[local];
                    }
                }
                __syncthreads();
#pragma unroll
                for (int r = 0; r < kRounds; r++)
                    if (dst[r] >= 0) {
                        rec[dst[r]] = rv[r];
                        rec_n0[dst[r]] = nv[r];
                    }
            }
            __syncthreads();
            // ---- pass 3: warps pull slices, scatter taps into private buffers
            {
                const int n_q = ctl[2], cap = ctl[4];
                for (;;) {
                    int q = 0;
                    if (lane == 0) q = atomicAdd(&ctl[1], 1);
                    q = __shfl_sync(0xffffffffu, q, 0);
                    if (q >= n_q) break;
                    const int item = order[q];
                    const int s = item & 255, k = item >> 8;
                    const int j0 = sub_start[s] + k * cap;
                    const int j1 = min(j0 + cap, sub_start[s] + sub_cnt[s]);
                    float *bs = (k == 0 ? buf + s * BUF : pool + (pool_base[s] + k - 1) * slot_words) +
                                P.em + lane;
                    const int origin = s * SUB;   // record n0 is relative to t_lo
                    if (MODE == kModeLUT && P.clamp)   // table values carry their sign: no lane sign
                        scatter_list<TPL, true, MODE>(bs, origin, rec, rec_n0, j0, j1, kf, ck, sk, 1.0f,
                                                      h_lut, lut, lut_cols);
                    else if (MODE == kModeLUT)
                        scatter_list<TPL, false, MODE>(bs, origin, rec, rec_n0, j0, j1, kf, ck, sk, 1.0f,
                                                       h_lut, lut, lut_cols);
                    else if (P.clamp)
                        scatter_list<TPL, true, MODE>(bs, origin, rec, rec_n0, j0, j1, kf, ck, sk,
                                                      lane_sign, H, lut, lut_cols);
                    else
                        scatter_list<TPL, false, MODE>(bs, origin, rec, rec_n0, j0, j1, kf, ck, sk,
                                                       lane_sign, H, lut, lut_cols);
                }
            }
            __syncthreads();
            // ---- merge the extra slices into their sub-range, in slice order (deterministic)
            //      (slots of one sub-range are consecutive: a register sum per run of slots,
            //      added in the same order as one slot at a time)
            {
                const int n_extra = ctl[3];
                if (n_extra > 0)
                    for (int w = tid; w < BUF; w += kThreads) {
                        int cur = slot_sub[0];
                        float acc = buf[P.em + cur * BUF + w];
                        for (int slot = 0; slot < n_extra; slot++) {
                            const int s = slot_sub[slot];
                            if (s != cur) {
                                buf[P.em + cur * BUF + w] = acc;
                                cur = s;
                                acc = buf[P.em + cur * BUF + w];
                            }
                            float *src = pool + slot * slot_words + P.em + w;
                            acc += *src;
                            *src = 0.0f;
                        }
                        buf[P.em + cur * BUF + w] = acc;
                    }
            }
            __syncthreads();
            if (COMP) {
                // this chunk's sums into the running (hi, lo) pairs; only the sub-ranges that
                // received images (their buffers hold every tap of them) are touched
                for (int i = tid; i < nsub * BUF; i += kThreads) {
                    if (sub_cnt[i / BUF] == 0) continue;
                    const float x = buf[P.em + i];
                    if (x == 0.0f) continue;
                    const ff t = ff_two_sum(hi[P.em + i], x);
                    hi[P.em + i] = t.hi;
                    lo[P.em + i] += t.lo;
                    buf[P.em + i] = 0.0f;
                }
                __syncthreads();
            }
        }
        // ---- output: sum of the covering sub-range buffers, ascending s.  An item that
        //      holds a whole early part also predicts the envelope from it and writes the
        //      diffuse tail (unless written above), so those stores overlap other blocks'
        //      tap work.
        // four consecutive samples per thread (t_lo is a multiple of 4): 16-byte stores
        // where the row allows, which also suits stores into host memory
        float pw = 0.0f;
        const bool vec_out = (reinterpret_cast<uintptr_t>(orow + t_lo) & 15) == 0;
        for (int t0 = t_lo + 4 * tid; t0 < t_hi; t0 += 4 * kThreads) {
            float v[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int rel = t0 + e - t_lo;
                int s_max = (rel - k_lo) / SUB;
                if (s_max > nsub - 1) s_max = nsub - 1;
                int num = rel - k_lo - BUF + 1;   // buffer s covers rel in [s*SUB + k_lo, s*SUB + k_lo + BUF)
                int s_min = num <= 0 ? 0 : (num + SUB - 1) / SUB;
                float acc = 0.0f;
                for (int s = s_min; s <= s_max; s++) {
                    const int w = P.em + s * BUF + rel - s * SUB - k_lo;
                    acc += COMP ? hi[w] + lo[w] : buf[w];
                }
                v[e] = acc;
            }
            if (vec_out && t0 + 3 < t_hi) {
                *reinterpret_cast<float4 *>(orow + t0) = make_float4(v[0], v[1], v[2], v[3]);
            } else {
#pragma unroll
                for (int e = 0; e < 4; e++)
                    if (t0 + e < t_hi) orow[t0 + e] = v[e];
            }
#pragma unroll
            for (int e = 0; e < 4; e++)
                if (t0 + e >= w_start && t0 + e < t_hi) pw = fmaf(v[e], v[e], pw);
        }
        if (fuse && !tail_written) {
            float *red = reinterpret_cast<float *>(hist);   // free until the next item
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) pw += __shfl_xor_sync(0xffffffffu, pw, o);
            if (lane == 0) red[warp] = pw;
            __syncthreads();
            if (tid == 0) {
                float tot = 0.0f;
                for (int w = 0; w < kWarps; w++) tot += red[w];
                const TailEnv e = tail_envelope(R, tot, w_start, tau_dp);
                red[kWarps] = e.ea;
                red[kWarps + 1] = e.eb;
                if (P.env_out) {
                    P.env_out[3 * it.rir] = e.A;
                    P.env_out[3 * it.rir + 1] = e.alpha;
                    P.env_out[3 * it.rir + 2] = tau_dp;
                }
            }
            __syncthreads();
            const uint64_t offset = P.offset_ptr ? *P.offset_ptr : P.offset;
            tail_fill(orow + R.n_ism, R.n_total - R.n_ism, 0, R.n_total - R.n_ism, tid, kThreads,
                      red[kWarps], red[kWarps + 1], P.seed, offset, (uint32_t)it.rir, P.noise_kind);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
size_t ism_forward_smem_bytes(int tpl, int em, int max_nsub, int mode, int tw) {
    const int ks = 32 * tpl;
    const size_t comp = (mode & kModeComp) ? 2 * (size_t)(2 * em + max_nsub * 2 * ks) : 0;
    size_t words = (size_t)(2 * em + max_nsub * 2 * ks) + (size_t)kPool * (2 * em + 2 * ks) + comp;
    size_t fixed = kChunk * (sizeof(float4) + sizeof(short) + 1) +
                   (kWarps * kMaxSub + 3 * kMaxSub + kMaxItems + kPool + 8) * sizeof(int);
    size_t lut = (mode & 3) == kModeLUT ? (size_t)kLutOversamp * (tw + 1) * sizeof(float2) + sizeof(float) : 0;
    return fixed + words * sizeof(float) + lut;
}

int ism_forward_max_nsub(int tpl, int em, size_t smem_budget, int mode, int tw) {
    const int ks = 32 * tpl;
    size_t fixed = ism_forward_smem_bytes(tpl, em, 0, mode, tw);
    if (smem_budget <= fixed) return 0;
    const size_t per_sub = sizeof(float) * 2 * ks * ((mode & kModeComp) ? 3 : 1);
    long n = (long)((smem_budget - fixed) / per_sub);
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

template <int TPL, int MODE>
static cudaError_t launch_tpl(const IsmLaunch &p, int grid, size_t smem, cudaStream_t st) {
    static bool attr_set = false;   // per process; the attribute is per function
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(ism_forward_kernel<TPL, MODE>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    ism_forward_kernel<TPL, MODE><<<grid, kThreads, smem, st>>>(p);
    return cudaGetLastError();
}

template <int MODE>
static int occupancy_query(int tpl, size_t smem) {
    int n = 0;
    switch (tpl) {
#define OCC(T) case T: cudaFuncSetAttribute(ism_forward_kernel<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024); \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ism_forward_kernel<T, MODE>, kThreads, smem); break;
        OCC(2) OCC(4) OCC(8) OCC(12) OCC(16) OCC(24)
#undef OCC
    default: return 0;
    }
    return n;
}

// Occupancy per (mode, taps per lane, shared memory), queried once: the queries cost
// tens of microseconds, which small launches would pay on every call.
template <int MODE>
static int occupancy(int tpl, size_t smem) {
    static std::mutex mu;
    static std::map<std::pair<int, size_t>, int> known;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(tpl, smem);
    auto it = known.find(key);
    if (it != known.end()) return it->second;
    const int n = occupancy_query<MODE>(tpl, smem);
    known[key] = n;
    return n;
}

int ism_forward_blocks_per_sm(int tpl, size_t smem, int mode) {
    switch (mode) {
    case kModeF32: return occupancy<kModeF32>(tpl, smem);
    case kModeMP: return occupancy<kModeMP>(tpl, smem);
    case kModeLUT: return occupancy<kModeLUT>(tpl, smem);
    case kModeMP | kModeComp: return occupancy<kModeMP | kModeComp>(tpl, smem);
    case kModeLUT | kModeComp: return occupancy<kModeLUT | kModeComp>(tpl, smem);
    default: return 0;
    }
}

template <int MODE>
static cudaError_t launch_mode(int tpl, const IsmLaunch &p, int grid, size_t smem, cudaStream_t st) {
    switch (tpl) {
    case 2: return launch_tpl<2, MODE>(p, grid, smem, st);
    case 4: return launch_tpl<4, MODE>(p, grid, smem, st);
    case 8: return launch_tpl<8, MODE>(p, grid, smem, st);
    case 12: return launch_tpl<12, MODE>(p, grid, smem, st);
    case 16: return launch_tpl<16, MODE>(p, grid, smem, st);
    case 24: return launch_tpl<24, MODE>(p, grid, smem, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t ism_forward_launch(int tpl, const RoomDesc *rooms, const IsmItem *items, int n_items,
                               const float *pos_src, const float *pos_rcv, const float *orv_src,
                               const float *orv_rcv, float *out, int *work_counter, int *status,
                               int em, int max_nsub, int clamp, int grid, cudaStream_t st, int mode,
                               int tw, const TailArgs *tail, float4 *axis_tab, int axis_cap,
                               float *partial, const unsigned char *skip) {
    IsmLaunch p;
    p.skip = skip;
    p.axis_tab = axis_tab;
    p.axis_cap = axis_cap;
    p.partial = partial;
    p.seed = tail ? tail->seed : 0;
    p.offset = tail ? tail->offset : 0;
    p.offset_ptr = tail ? tail->offset_ptr : nullptr;
    p.noise_kind = tail ? tail->noise_kind : 0;
    p.env_out = tail ? tail->env_out : nullptr;
    p.fuse_tail = tail ? tail->fuse : 0;
    p.tail_pre = tail ? tail->pre : nullptr;
    p.rooms = rooms; p.items = items; p.n_items = n_items;
    p.pos_src = pos_src; p.pos_rcv = pos_rcv; p.orv_src = orv_src; p.orv_rcv = orv_rcv;
    p.out = out; p.work_counter = work_counter; p.status = status;
    p.em = em; p.max_nsub = max_nsub; p.clamp = clamp; p.tw = tw;
    size_t smem = ism_forward_smem_bytes(tpl, em, max_nsub, mode, tw);
    cudaError_t e = cudaMemsetAsync(work_counter, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    switch (mode) {
    case kModeF32: return launch_mode<kModeF32>(tpl, p, grid, smem, st);
    case kModeMP: return launch_mode<kModeMP>(tpl, p, grid, smem, st);
    case kModeLUT: return launch_mode<kModeLUT>(tpl, p, grid, smem, st);
    case kModeMP | kModeComp: return launch_mode<kModeMP | kModeComp>(tpl, p, grid, smem, st);
    case kModeLUT | kModeComp: return launch_mode<kModeLUT | kModeComp>(tpl, p, grid, smem, st);
    default: return cudaErrorInvalidValue;
    }
}

// Per item: 1 when no image of its (source, receiver) pair can reach its segment,
// from the per-axis extremes of the image coordinates at the current positions.
// First segments are not tested (they hold the direct path).
__global__ void item_skip_kernel(const RoomDesc *rooms, const IsmItem *items, int n_items, const float *pos_src,
                                 const float *pos_rcv, unsigned char *skip) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_items) return;
    const IsmItem it = items[k];
    unsigned char m = 0;
    if (it.t_lo > 0) {
        const RoomDesc &R = rooms[it.room];
        const float s3[3] = {pos_src[3 * it.src], pos_src[3 * it.src + 1], pos_src[3 * it.src + 2]};
        const float r3[3] = {pos_rcv[3 * it.rcv], pos_rcv[3 * it.rcv + 1], pos_rcv[3 * it.rcv + 2]};
        m = images_miss_segment(R.L, R.nb, s3, r3, R.kh, R.H, it.t_lo, it.t_hi) ? 1 : 0;
    }
    skip[k] = m;
}

cudaError_t item_skip_launch(const RoomDesc *rooms, const IsmItem *items, int n_items, const float *pos_src,
                             const float *pos_rcv, unsigned char *skip, cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    item_skip_kernel<<<(n_items + 255) / 256, 256, 0, st>>>(rooms, items, n_items, pos_src, pos_rcv, skip);
    return cudaGetLastError();
}

// Sum of the partial segments of each group, parts in increasing order (the result
// does not depend on which block computed which part).
__global__ void partial_reduce_kernel(const PartGroup *groups, int n_groups, const float *part, float *out) {
    const int g = blockIdx.y;
    if (g >= n_groups) return;
    const PartGroup G = groups[g];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= G.len) return;
    const float *p = part + G.base + t;
    float acc = 0.0f;
    for (int k = 0; k < G.n_part; k++) acc += p[(long long)k * G.len];
    out[G.out + t] = acc;
}

cudaError_t partial_reduce_launch(const PartGroup *groups, int n_groups, int max_len, const float *part,
                                  float *out, cudaStream_t st) {
    if (n_groups <= 0 || max_len <= 0) return cudaSuccess;
    if (n_groups > 65535) return cudaErrorInvalidValue;
    dim3 grid((unsigned)((max_len + 255) / 256), (unsigned)n_groups);
    partial_reduce_kernel<<<grid, 256, 0, st>>>(groups, n_groups, part, out);
    return cudaGetLastError();
}

}  // namespace gpurir
