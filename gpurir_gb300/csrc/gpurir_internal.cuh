// gpurir_internal.cuh -- shared device helpers and launch descriptors of the
// gpurir_gb300 image-source-method (ISM) engine for sm_103a.
//
// Reference behaviour restated here comes from src/gpuRIR_cuda.cu of gpuRIR
// (file:line citations at each helper).  Nothing in this file is a copy of it.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gpurir {

// Polar patterns, numbering of src/gpuRIR_cuda.h:2-8.
enum Pattern { P_OMNI = 0, P_HOMNI = 1, P_CARD = 2, P_HYPCARD = 3, P_SUBCARD = 4, P_BIDIR = 5 };

// Maximum exponent + 1 of the per-wall reflection power tables.
constexpr int kPowMax = 96;

// One room of a launch.  Device-resident; the host fills it (ism_host.cu).
struct RoomDesc {
    float L[3];            // room size [m]
    int nb[3];             // images per axis
    int n_img;             // nb[0]*nb[1]*nb[2]
    int n_ism;             // samples of the early (ISM) part
    int n_total;           // samples per RIR row
    int n_src, n_rcv;      // sources / receivers of this room
    int src_off, rcv_off;  // first row of this room in the position arrays
    int rir_off;           // global index of the room's first RIR (src-major)
    int spkr, mic;         // polar patterns
    float kh, kl;          // Fs / c as a float-float pair (samples per metre)
    float H;               // half window Tw/2 [samples]
    float H2;              // H*H
    float wc[4];           // window polynomial in x^2: cos(pi x/Tw) = (H2 - x^2) * poly(x^2)
    float T60;             // Sabine T60 of the walls (tail)
    float fs;              // sampling rate
    float beta[6];         // wall reflection coefficients (tail / adjoint)
    long long out_off;     // element offset of the room's first RIR row in the output
    int pow_n;             // valid entries per wall in the power table
    float c;               // speed of sound [m/s] as the caller gave it
    int ref_delay;         // 1: delays in the reference's float32 arithmetic (ref_tau)
    int pad_;
    float pw[6][kPowMax];  // pw[w][k] = (-beta[w])^k, rounded from FP64
};

// One work item of the persistent ISM kernel: one RIR, one segment of samples, one
// range of its images.  An item holding all the images writes the segment into the
// output; an item holding a part of them writes a partial segment (part_off >= 0)
// that a reduction adds up with the RIR's other parts in a fixed order.
struct IsmItem {
    int room;       // index into the RoomDesc table
    int src, rcv;   // rows of the position arrays (global)
    int t_lo, t_hi; // output samples [t_lo, t_hi) of the early part
    int rir;        // global RIR index
    long long out_row;   // element offset of sample 0 of this RIR in the output
    int i_lo, i_hi;      // images [i_lo, i_hi) of the room's image grid
    long long part_off;  // -1, or the offset of this item's partial segment
};

// A set of partial segments to add up: out[out + t] = sum_p part[base + p len + t].
struct PartGroup {
    long long out;    // element offset of the segment's first sample in the output
    long long base;   // offset of the first partial segment
    int len, n_part;
};

// ---------------------------------------------------------------------------
// Float-float ("double-float") arithmetic from error-free transformations
// (Dekker 1971; Knuth TAOCP vol. 2, 4.2.2).  Used for image geometry so that
// delays keep ~1e-10 absolute precision in samples with FP32 hardware only:
// GB300's FP64 rate is ~1/64 of its FP32 rate.
// ---------------------------------------------------------------------------
struct ff { float hi, lo; };

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {  // |a| >= |b|
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}
__device__ __forceinline__ ff ff_two_prod(float a, float b) {
    float p = __fmul_rn(a, b);
    float e = __fmaf_rn(a, b, -p);
    return {p, e};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = ff_two_sum(a.hi, b.hi);
    float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return ff_fast_two_sum(s.hi, e);
}
__device__ __forceinline__ ff ff_sqr(ff a) {
    ff p = ff_two_prod(a.hi, a.hi);
    float e = __fmaf_rn(2.0f * a.hi, a.lo, p.lo);
    return ff_fast_two_sum(p.hi, e);
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    ff p = ff_two_prod(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
    return ff_fast_two_sum(p.hi, e);
}
__device__ __forceinline__ ff ff_sqrt(ff a) {
    float s = __fsqrt_rn(a.hi);
    ff p = ff_two_prod(s, s);
    float r = __fdiv_rn(__fadd_rn(__fsub_rn(__fsub_rn(a.hi, p.hi), p.lo), a.lo), 2.0f * s);
    return ff_fast_two_sum(s, r);
}

// ---------------------------------------------------------------------------
// Series evaluations and integer splits shared by the ISM kernels.
// ---------------------------------------------------------------------------
// sin(pi f) for 0 <= f <= 1: reflected to g = min(f, 1 - f) <= 1/2 (1 - f is exact
// there), then the Taylor series of sin(pi g) = g * sum_k (-1)^k pi^(2k+1) g^(2k) / (2k+1)!
// through k = 7 (remainder < 1e-9 relative), Horner in g^2.
__device__ __forceinline__ float sinpi_unit(float f) {
    const float g = fminf(f, 1.0f - f);
    const float y = g * g;
    float p = -2.1915353447830215827e-05f;
    p = fmaf(p, y, 4.6630280576761256442e-04f);
    p = fmaf(p, y, -7.3704309457143507773e-03f);
    p = fmaf(p, y, 8.2145886611128228799e-02f);
    p = fmaf(p, y, -5.9926452932079207689e-01f);
    p = fmaf(p, y, 2.5501640398773454439f);
    p = fmaf(p, y, -5.1677127800499700292f);
    p = fmaf(p, y, 3.1415926535897932385f);
    return g * p;
}

// sin(pi u), cos(pi u) for 0 <= u <= 1/16 by their Taylor series (remainders below
// 1e-12 absolute): the per-image window angle, u = f / H.
__device__ __forceinline__ void sincospi_small(float u, float &sn, float &cs) {
    const float y = u * u;
    float ps = -5.9926452932079207689e-01f;
    ps = fmaf(ps, y, 2.5501640398773454439f);
    ps = fmaf(ps, y, -5.1677127800499700292f);
    ps = fmaf(ps, y, 3.1415926535897932385f);
    sn = u * ps;
    float pc = 2.3533063035889320454e-01f;
    pc = fmaf(pc, y, -1.3352627688545894959f);
    pc = fmaf(pc, y, 4.0587121264167682182f);
    pc = fmaf(pc, y, -4.9348022005446793094f);
    cs = fmaf(pc, y, 1.0f);
}

// q = n / d, r = n - q d for 0 <= n < 2^24, 1 <= d: float reciprocal, then an exact
// fix-up of the (at most a few units) rounding error.
__device__ __forceinline__ void divmod_small(int n, int d, float rd, int &q, int &r) {
    q = (int)((float)n * rd);
    r = n - q * d;
    while (r < 0) { q -= 1; r += d; }
    while (r >= d) { q += 1; r -= d; }
}

// sin(pi f), cos(pi f) for 0 <= f <= 1: sin as sinpi_unit, cos(pi f) = +-cos(pi g) by
// the Taylor series of cos(pi g) through g^16 (remainder < 1e-12), g = min(f, 1 - f).
__device__ __forceinline__ void sincospi_unit(float f, float &sn, float &cs) {
    const bool upper = f > 0.5f;
    const float g = upper ? 1.0f - f : f;
    const float y = g * g;
    float ps = -2.1915353447830215827e-05f;
    ps = fmaf(ps, y, 4.6630280576761256442e-04f);
    ps = fmaf(ps, y, -7.3704309457143507773e-03f);
    ps = fmaf(ps, y, 8.2145886611128228799e-02f);
    ps = fmaf(ps, y, -5.9926452932079207689e-01f);
    ps = fmaf(ps, y, 2.5501640398773454439f);
    ps = fmaf(ps, y, -5.1677127800499700292f);
    ps = fmaf(ps, y, 3.1415926535897932385f);
    sn = g * ps;
    float pc = 4.3030695870329470073e-06f;
    pc = fmaf(pc, y, -1.0463810492484570712e-04f);
    pc = fmaf(pc, y, 1.9295743094039230479e-03f);
    pc = fmaf(pc, y, -2.5806891390014060013e-02f);
    pc = fmaf(pc, y, 2.3533063035889320454e-01f);
    pc = fmaf(pc, y, -1.3352627688545894959f);
    pc = fmaf(pc, y, 4.0587121264167682182f);
    pc = fmaf(pc, y, -4.9348022005446793094f);
    pc = fmaf(pc, y, 1.0f);
    cs = upper ? -pc : pc;
}

// Distance from a float-float squared distance: an approximate square root s0
// (rsqrt) and one Newton step s0 + (d2 - s0^2) / (2 s0), the residual by FMA exact to
// ~1e-14 of d2.  inv_d is 1/distance to ~1e-7 (one Newton step on rsqrt).
__device__ __forceinline__ ff ff_dist_newton(ff d2, float rs0, float s0, float &inv_d) {
    const float rs = rs0 * fmaf(-0.5f * d2.hi * rs0, rs0, 1.5f);
    const float res = fmaf(-s0, s0, d2.hi) + d2.lo;
    inv_d = rs;
    return ff_fast_two_sum(s0, 0.5f * res * rs);
}

// ---------------------------------------------------------------------------
// Image bookkeeping of src/gpuRIR_cuda.cu:336-342: k = n - N/2,
// clust = ceil(k/2), refl = |k mod 2|; coordinate 2*clust*L + (1-2 refl)*src.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void image_axis(int n, int N, int &clust, int &refl) {
    int k = n - N / 2;
    clust = (k + 1) >> 1;   // arithmetic shift: ceil(k/2) for every sign of k
    refl = k & 1;           // |k % 2| in two's complement
}

// Range of the squared receiver->image component along one axis over all N images
// of that axis, for any source and receiver coordinates.  The image coordinate is
// k L + s for even k and (k + 1) L - s for odd k: each parity is increasing in k, so
// its extremes are at its first and last index and it crosses zero at most once.
// Plain FP32 (a bound to a few 1e-6 relative; callers leave a margin).
__host__ __device__ __forceinline__ void axis_extent(int N, float L, float s, float r, float &v2min,
                                                    float &v2max) {
    const int k_min = -(N / 2), k_max = N - 1 - N / 2;
    v2min = 3.0e38f;
    v2max = 0.0f;
#pragma unroll
    for (int par = 0; par < 2; par++) {
        const int lo = (k_min & 1) == par ? k_min : k_min + 1;
        const int hi = (k_max & 1) == par ? k_max : k_max - 1;
        if (lo > hi) continue;
        const float a = par ? (float)(lo + 1) * L - s - r : (float)lo * L + s - r;
        const float b = par ? (float)(hi + 1) * L - s - r : (float)hi * L + s - r;
        v2max = fmaxf(v2max, fmaxf(a * a, b * b));
        v2min = fminf(v2min, (a <= 0.0f && b >= 0.0f) ? 0.0f : fminf(a * a, b * b));
    }
}

// True when no image of the pair (src, rcv) has a delay within reach of the samples
// [t_lo, t_hi): every delay lies below t_lo - H - margin or above t_hi + H + margin.
// fs_c = Fs / c in samples per metre.
__host__ __device__ __forceinline__ bool images_miss_segment(const float L[3], const int nb[3],
                                                             const float s[3], const float r[3], float fs_c,
                                                             float H, int t_lo, int t_hi) {
    float lo2 = 0.0f, hi2 = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float mn, mx;
        axis_extent(nb[a], L[a], s[a], r[a], mn, mx);
        lo2 += mn;
        hi2 += mx;
    }
    const float tau_lo = sqrtf(lo2) * fs_c, tau_hi = sqrtf(hi2) * fs_c;
    const float margin = 2.0f + 1e-5f * tau_hi;
    return tau_hi < (float)t_lo - H - margin || tau_lo > (float)t_hi + H + margin;
}

// ---------------------------------------------------------------------------
// Reference-delay model: the image delay exactly as gpuRIR's calcAmpTau_kernel
// rounds it in float32 (src/gpuRIR_cuda.cu:336-367), for callers that want the
// reference's output rather than the exact sum.  Each step is an explicit
// round-to-nearest intrinsic so that no contraction of ours can change it.
// ---------------------------------------------------------------------------
// One component of the receiver -> image vector (:337, :353): the cluster offset
// (2 clust) L rounded, plus or minus the source coordinate rounded, minus the
// receiver coordinate rounded.
__device__ __forceinline__ float ref_axis_component(int clust, int refl, float L, float s, float r) {
    const float cp = __fmul_rn((float)(2 * clust), L);
    return __fsub_rn(__fadd_rn(cp, refl ? -s : s), r);
}

// Squared distance from the three components as the reference build forms it.
// The reference's loop `dist += vec[d] * vec[d]` (:354) is contracted by the
// compiler in two ways, depending on which version of its loop runs: with both
// patterns omni, one FMA per component in axis order; with a directional source
// or receiver, x^2 + y^2 rounded separately and then one FMA for z.  Both were
// identified bit for bit against the delays the reference's own kernel wrote.
__device__ __forceinline__ float ref_dist2(float v0, float v1, float v2, bool directional) {
    if (directional) return __fmaf_rn(v2, v2, __fadd_rn(__fmul_rn(v0, v0), __fmul_rn(v1, v1)));
    return __fmaf_rn(v2, v2, __fmaf_rn(v1, v1, __fmul_rn(v0, v0)));
}

// Delay in samples from the squared distance: sqrtf, then `dist / c * Fs` (:366)
// with IEEE division and multiplication.
__device__ __forceinline__ float ref_tau(float d2, float c, float fs) {
    return __fmul_rn(__fdiv_rn(__fsqrt_rn(d2), c), fs);
}

// Directivity gain, src/gpuRIR_cuda.cu:132-147, with the cosine already formed.
__device__ __forceinline__ float pattern_gain(float cos_t, int pattern) {
    switch (pattern) {
    case P_HOMNI:   return cos_t > 0.0f ? 1.0f : 0.0f;
    case P_CARD:    return 0.5f + 0.5f * cos_t;
    case P_HYPCARD: return 0.25f + 0.75f * cos_t;
    case P_SUBCARD: return 0.75f + 0.25f * cos_t;
    case P_BIDIR:   return cos_t;
    default:        return 1.0f;
    }
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11), the counter-based generator of the
// diffuse tail.  Bit-exact with oracle/ism_oracle.c:orc_philox4x32_10.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// Uniform in (0, 1) from the top 23 bits: (m + 0.5) * 2^-23, exact in float32.
__device__ __forceinline__ float u01(uint32_t x) {
    return ((float)(x >> 9) + 0.5f) * 1.1920928955078125e-07f;
}

// Diffuse-tail parameters passed to the ISM kernel, whose epilogue writes the
// tail of every RIR that is a single work item.
struct TailArgs {
    uint64_t seed, offset;
    const uint64_t *offset_ptr;   // if set, the call offset is read there (captured graphs)
    int noise_kind;
    float *env_out;               // optional [rir][3]: A, alpha, tau_dp
    int fuse;
    // optional [rir]: 1 = the RIR's tail is silent and written by someone else (a copy
    // engine streaming zeros into host memory); the kernel writes only its envelope
    const unsigned char *pre = nullptr;
};

// Error codes shared by kernels and host (written to a device status word).
enum DevError : int { DEV_OK = 0, DEV_BAD_ITEM = 1, DEV_BAD_ROOM = 2 };

}  // namespace gpurir
