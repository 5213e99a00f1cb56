// ism_backward.cu -- adjoint of the image-source early part for sm_103a.
//
// gpuRIR has no gradients.  For a loss L of the RIRs, with g[t] = dL/dh[t] over
// the early part, each image n contributes
//   dL/damp_n = sum_t g[t] W(t - tau_n)            (A)
//   dL/dtau_n = -amp_n sum_t g[t] W'(t - tau_n)    (-amp B)
// with W = Hann window x sinc, the tap of image_sample (src/gpuRIR_cuda.cu:116-121).
// Amplitudes and delays are recomputed from the geometry (as the forward kernel
// does), then the chain rule gives per-image contributions to
//   beta (6 walls), source and receiver positions, source and receiver
//   orientations,
// summed per work item into 18 partials.  A second kernel sums the partials of
// each room / source / receiver over a fixed item order: results are
// deterministic (no floating-point atomics).
//
// Tap arithmetic (x = k - f, tau = n0 + f, per-lane constants ck, sk for the
// window as in the forward kernel, sigma = -sin(pi f)/pi, gamma = cos(pi f)):
//   s  = (-1)^k sigma / x,         s' = ((-1)^k gamma - s) / x
//   w  = 0.5 + ck cos(phi) + sk sin(phi),   w' = (2 pi/Tw)(ck sin(phi) - sk cos(phi))
//   W  = w s,   W' = w' s + w s'.
#include "gpurir_internal.cuh"

namespace gpurir {

constexpr int kBThreads = 256;   // three blocks per SM (registers)
constexpr int kBWarps = kBThreads / 32;
constexpr int kGrad = 18;                       // beta[6], src[3], rcv[3], orv_src[3], orv_rcv[3]

struct BwdLaunch {
    const RoomDesc *rooms;
    const IsmItem *items;
    int n_items;
    const float *pos_src, *pos_rcv, *orv_src, *orv_rcv;
    const float *grad;        // dL/dh, same layout as the forward output
    float *item_grad;         // [n_items][kGrad]
    int *work_counter;
    int *status;
    int max_tseg;
    int pad;                  // g staging margin (>= taps reach)
    int axis_cap;             // per-axis table entries (max over rooms of N0 + N1 + N2)
};

__device__ __forceinline__ float rcp_approx_b(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Asynchronous 4-byte copy global -> shared; src_bytes = 0 writes a zero instead of
// reading (PTX cp.async with a source size).
__device__ __forceinline__ void cp_async4(float *dst, const float *src, int src_bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Derivative of the polar-pattern gain with respect to cos(theta)
// (src/gpuRIR_cuda.cu:140-145; homni is flat almost everywhere).
__device__ __forceinline__ float pattern_slope(int pattern) {
    switch (pattern) {
    case P_CARD: return 0.5f;
    case P_HYPCARD: return 0.75f;
    case P_SUBCARD: return 0.25f;
    case P_BIDIR: return 1.0f;
    default: return 0.0f;
    }
}

template <int TPL, bool CLAMP>
__global__ void __launch_bounds__(kBThreads, 3) ism_backward_kernel(BwdLaunch P) {
    // per-warp scratch of 32 kept images: records, then A and B of each
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // records of the kept images: (sigma, f, cos phi, sin phi) and
    // (2 pi/Tw cos phi, 2 pi/Tw sin phi, cos(pi f), floor(tau) - t_lo as int bits)
    float4 *rec = reinterpret_cast<float4 *>(smem_raw);
    float4 *rec2 = rec + kBThreads;
    float *ga = reinterpret_cast<float *>(rec2 + kBThreads);         // A per kept image
    float *gb = ga + kBThreads;                                      // B per kept image
    int *ctl = reinterpret_cast<int *>(gb + kBThreads);              // [0] item
    float *red = reinterpret_cast<float *>(ctl + 4);                 // [kBWarps][kGrad]
    // then [kGrad][kBThreads] per-thread gradient partials
    float *gs = red + (kBWarps + kBThreads) * kGrad;                 // staged dL/dh
    // per-axis image terms of the current item (m < N0, then N1, then N2 entries):
    //   tab[e]  = {v^2 hi, v^2 lo, v hi, (-b_lo)^e_lo (-b_hi)^e_hi}, as the forward kernel
    //   tabd[e] = {(-b_lo)^e_lo, (-b_hi)^e_hi, e_lo (-b_lo)^(e_lo-1), e_hi (-b_hi)^(e_hi-1)}
    // with e_lo = |c - r|, e_hi = |c| and b_lo, b_hi the axis' two walls
    float4 *tab = reinterpret_cast<float4 *>(gs + ((P.max_tseg + 2 * P.pad + 3) & ~3));
    float4 *tabd = tab + P.axis_cap;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // per-lane tap constants; one Fs per launch, so one window for every room: computed
    // once per block
    float kf[TPL], ck[TPL], sk[TPL];
    {
        const float H0 = P.rooms[0].H, inv_h0 = 1.0f / H0;
        const int k_lo0 = (int)floorf(-H0) + 1;
#pragma unroll
        for (int i = 0; i < TPL; i++) {
            kf[i] = (float)(k_lo0 + lane + 32 * i);
            float sn, cs;
            sincospif(kf[i] * inv_h0, &sn, &cs);
            // the lane's sign (-1)^k goes into the window constants
            const float ls = ((k_lo0 + lane) & 1) ? -0.5f : 0.5f;
            ck[i] = ls * cs;
            sk[i] = ls * sn;
        }
    }
    for (;;) {
        if (tid == 0) ctl[0] = atomicAdd(P.work_counter, 1);
        __syncthreads();
        const int item_id = ctl[0];
        if (item_id >= P.n_items) break;
        const IsmItem it = P.items[item_id];
        const RoomDesc &R = P.rooms[it.room];
        const int t_lo = it.t_lo, t_hi = it.t_hi;
        if (t_hi - t_lo > P.max_tseg || t_hi <= t_lo) {
            if (tid == 0) atomicExch(P.status, DEV_BAD_ITEM);
            __syncthreads();
            continue;
        }
        const float L0 = R.L[0], L1 = R.L[1], L2 = R.L[2];
        const int N0 = R.nb[0], N1 = R.nb[1], N2 = R.nb[2];
        const int n_img = R.n_img;
        const float H = R.H, inv_h = 1.0f / H;
        const float rN1 = 1.0f / (float)N1, rN2 = 1.0f / (float)N2;
        const bool small_phi = inv_h <= 0.0625f;   // window angle f / H <= 1/16: series
        const int k_lo = (int)floorf(-H) + 1;
        const int spkr = R.spkr, mic = R.mic;
        const ff kfs = {R.kh, R.kl};
        const float sx = P.pos_src[3 * it.src], sy = P.pos_src[3 * it.src + 1], sz = P.pos_src[3 * it.src + 2];
        const float rx = P.pos_rcv[3 * it.rcv], ry = P.pos_rcv[3 * it.rcv + 1], rz = P.pos_rcv[3 * it.rcv + 2];
        float os[3] = {0.f, 0.f, 0.f}, orr[3] = {0.f, 0.f, 0.f}, inv_os = 0.f, inv_or = 0.f;
        if (spkr != P_OMNI) {
            for (int d = 0; d < 3; d++) os[d] = P.orv_src[3 * it.src + d];
            inv_os = rsqrtf(os[0] * os[0] + os[1] * os[1] + os[2] * os[2]);
        }
        if (mic != P_OMNI) {
            for (int d = 0; d < 3; d++) orr[d] = P.orv_rcv[3 * it.rcv + d];
            inv_or = rsqrtf(orr[0] * orr[0] + orr[1] * orr[1] + orr[2] * orr[2]);
        }
        const float keep_lo = (float)t_lo - H, keep_hi = (float)t_hi + H;
        const float fs_c = R.kh + R.kl;   // Fs / c
        // an item whose segment no image reaches contributes nothing: no staging, no chunks
        // (tested on later segments; a first segment holds the direct path)
        bool miss = false;
        if (t_lo > 0) {
            const float Lr[3] = {L0, L1, L2}, s3[3] = {sx, sy, sz}, r3[3] = {rx, ry, rz};
            miss = images_miss_segment(Lr, R.nb, s3, r3, R.kh, H, t_lo, t_hi);
        }
        if (miss) {   // zero partials, nothing else
            if (tid < kGrad) P.item_grad[(long)item_id * kGrad + tid] = 0.0f;
            __syncthreads();
            continue;
        }
        // per-axis tables of this item (an image's squared distance is then two float-float
        // additions, the same operations in the same order as in the forward kernel)
        for (int e = tid; e < N0 + N1 + N2; e += kBThreads) {
            const int a = e < N0 ? 0 : (e < N0 + N1 ? 1 : 2);
            const int m = e - (a == 0 ? 0 : (a == 1 ? N0 : N0 + N1));
            const int Na = a == 0 ? N0 : (a == 1 ? N1 : N2);
            const float La = a == 0 ? L0 : (a == 1 ? L1 : L2);
            const float sa = a == 0 ? sx : (a == 1 ? sy : sz), ra = a == 0 ? rx : (a == 1 ? ry : rz);
            int ca, fa;
            image_axis(m, Na, ca, fa);
            const ff v = ff_add(ff_two_prod((float)(2 * ca), La), ff_two_sum(fa ? -sa : sa, -ra));
            const ff sq = ff_sqr(v);
            const int elo = abs(ca - fa), ehi = abs(ca);
            const float plo = R.pw[2 * a][elo], phi = R.pw[2 * a + 1][ehi];
            tab[e] = make_float4(sq.hi, sq.lo, v.hi, plo * phi);
            tabd[e] = make_float4(plo, phi, elo > 0 ? (float)elo * R.pw[2 * a][elo - 1] : 0.0f,
                                  ehi > 0 ? (float)ehi * R.pw[2 * a + 1][ehi - 1] : 0.0f);
        }
        __syncthreads();
        // Stage g over [t_lo - pad, t_hi + pad), zero outside this item's segment: copies
        // in flight while the first images' geometry is computed
        {
            const int g_len = t_hi - t_lo + 2 * P.pad;
            const float *grow = P.grad + it.out_row;
            for (int i = tid; i < g_len; i += kBThreads) {
                const int t = t_lo - P.pad + i;
                const bool in = t >= t_lo && t < t_hi;
                cp_async4(gs + i, grow + (in ? t : t_lo), in ? 4 : 0);
            }
        }
        const float dws = 3.14159265358979323846f * inv_h;   // 2 pi / Tw
        const float half_sign = ((k_lo + lane) & 1) ? -0.5f : 0.5f;   // (-1)^k / 2
        // this thread's gradient partials of the item, in shared memory (registers go to
        // the taps): acc(q) = accs[q * kBThreads + tid]
        float *accs = red + kBWarps * kGrad;
#define acc(q) accs[(q) * kBThreads + tid]
#pragma unroll
        for (int q = 0; q < kGrad; q++) acc(q) = 0.0f;

        const int i_end = min(it.i_hi, n_img);   // this item's images: [i_lo, i_end)
        // Each warp walks its own groups of 32 consecutive images (group g of the item goes
        // to warp g mod kBWarps): geometry one image per lane, the kept images' records
        // packed in the warp's scratch, their taps four images at a time over the lanes,
        // then the chain rule one image per lane.  No block barrier inside an item.
        float4 *wrec = rec + warp * 32, *wrec2 = rec2 + warp * 32;
        float *wga = ga + warp * 32, *wgb = gb + warp * 32;
        bool keep = false;
        float4 r4 = make_float4(0.f, 0.f, 1.f, 0.f);
        float rg = 1.f;
        int rn0 = 0;
        // geometry of image ii: keep, (sigma, f, cos phi, sin phi), cos(pi f), n0 - t_lo
        auto geometry = [&](const int ii) {
            keep = false;
            r4 = make_float4(0.f, 0.f, 1.f, 0.f);
            rg = 1.f;
            rn0 = 0;
            if (ii < i_end) {
                int q, m2, m0, m1;
                divmod_small(ii, N2, rN2, q, m2);
                divmod_small(q, N1, rN1, m0, m1);
                const float4 t0 = tab[m0], t1 = tab[N0 + m1], t2 = tab[N0 + N1 + m2];
                const ff d2 = ff_add(ff_add(ff{t0.x, t0.y}, ff{t1.x, t1.y}), ff{t2.x, t2.y});
                // approximate distance first: far images stop here
                const float rs0 = rsqrtf(d2.hi);
                const float s0 = d2.hi * rs0;
                const float tau_est = s0 * kfs.hi;
                ff tau = {-1e30f, 0.0f};   // culled: fails the keep test below
                if (tau_est > keep_lo - 1.0f && tau_est < keep_hi + 1.0f) {
                    float inv_d;
                    tau = ff_mul(ff_dist_newton(d2, rs0, s0, inv_d), kfs);
                }
                if (tau.hi > keep_lo && tau.hi < keep_hi) {
                    float fl = floorf(tau.hi);
                    int n0 = (int)fl;
                    float f = __fadd_rn(__fsub_rn(tau.hi, fl), tau.lo);
                    if (f < 0.0f) { n0 -= 1; f += 1.0f; }
                    if (f >= 1.0f) { n0 += 1; f -= 1.0f; }
                    f = fmaxf(f, 9.094947017729282e-13f);
                    float sp, cp, sphi, cphi;
                    sincospi_unit(f, sp, cp);
                    if (small_phi) sincospi_small(f * inv_h, sphi, cphi);
                    else sincospif(f * inv_h, &sphi, &cphi);
                    r4 = make_float4(-sp * 0.318309886183790672f, f, cphi, sphi);
                    rg = cp;
                    rn0 = n0 - t_lo;
                    keep = true;
                }
            }
        };
        int gbase = it.i_lo + warp * 32;
        geometry(gbase + lane);
        cp_async_wait_all();
        __syncthreads();   // g staged
        for (; gbase < i_end; gbase += kBThreads) {
            const int i = gbase + lane;
            const unsigned kmask = __ballot_sync(0xffffffffu, keep);
            const int n_k = __popc(kmask);
            const int slot = __popc(kmask & ((1u << lane) - 1u));
            if (keep) {
                wrec[slot] = r4;
                wrec2[slot] = make_float4(dws * r4.z, dws * r4.w, rg, __int_as_float(rn0));
            }
            __syncwarp();
            // per kept image, A and B over its taps, four images per trip
            const float *gl = gs + P.pad + lane;
            for (int j = 0; j < n_k; j += 4) {
                float v[8];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int jj = min(j + u, n_k - 1);
                    const float4 c = wrec[jj], c2 = wrec2[jj];
                    const float sig = c.x, f = c.y, cphi = c.z, sphi = c.w;
                    const float cphd = c2.x, sphd = c2.y, gam = c2.z;   // w' = ck sphd - sk cphd
                    const float *gp = gl + __float_as_int(c2.w) + k_lo;
                    // sigma and gamma are constant over the image: with q = g / x and the
                    // lane's sign (-1)^k inside w and w',
                    //   sum g W  = sigma S,   S = sum q w
                    //   sum g W' = sigma T + gamma S,   T = sum q (w' - w / x)
                    float s1 = 0.0f, t1 = 0.0f;
                    if constexpr ((TPL % 2) == 0 && TPL <= 12) {
                        // taps k and k + 1 in packed FP32 (two-wide FADD/FMUL/FFMA); the two
                        // halves of S and T are added at the end
                        const float2 f2 = make_float2(-f, -f), cp2 = make_float2(cphi, cphi);
                        const float2 sp2 = make_float2(sphi, sphi), hs2 = make_float2(half_sign, half_sign);
                        const float2 sd2 = make_float2(sphd, sphd), cd2 = make_float2(-cphd, -cphd);
                        float2 s2 = make_float2(0.0f, 0.0f), t2 = make_float2(0.0f, 0.0f);
#pragma unroll
                        for (int k = 0; k < TPL; k += 2) {
                            const float2 x = __fadd2_rn(make_float2(kf[k], kf[k + 1]), f2);
                            const float2 rx_ = make_float2(rcp_approx_b(x.x), rcp_approx_b(x.y));
                            const float2 ck2 = make_float2(ck[k], ck[k + 1]), sk2 = make_float2(sk[k], sk[k + 1]);
                            const float2 w = __ffma2_rn(ck2, cp2, __ffma2_rn(sk2, sp2, hs2));
                            const float2 wd = __ffma2_rn(ck2, sd2, __fmul2_rn(sk2, cd2));
                            float2 q = __fmul2_rn(make_float2(gp[32 * k], gp[32 * (k + 1)]), rx_);
                            if (CLAMP) {
                                if (fabsf(x.x) >= H) q.x = 0.0f;
                                if (fabsf(x.y) >= H) q.y = 0.0f;
                            }
                            s2 = __ffma2_rn(q, w, s2);
                            t2 = __ffma2_rn(q, __ffma2_rn(make_float2(-w.x, -w.y), rx_, wd), t2);
                        }
                        s1 = s2.x + s2.y;
                        t1 = t2.x + t2.y;
                    } else {
#pragma unroll
                        for (int k = 0; k < TPL; k++) {
                            const float x = kf[k] - f;
                            const float rx_ = rcp_approx_b(x);
                            const float w = fmaf(ck[k], cphi, fmaf(sk[k], sphi, half_sign));
                            const float wd = fmaf(ck[k], sphd, -sk[k] * cphd);
                            float q = gp[32 * k] * rx_;
                            if (CLAMP && fabsf(x) >= H) q = 0.0f;
                            s1 = fmaf(q, w, s1);
                            t1 = fmaf(q, fmaf(-w, rx_, wd), t1);
                        }
                    }
                    v[2 * u] = sig * s1;
                    v[2 * u + 1] = fmaf(sig, t1, gam * s1);
                }
                // reduce the 8 values over the warp with 9 shuffles: afterwards lanes 4m..4m+3
                // hold value m = 2 u + (0: A, 1: B) of image j + u
                const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
                float w4[4], w2[2];
#pragma unroll
                for (int e = 0; e < 4; e++)
                    w4[e] = (b4 ? v[4 + e] : v[e]) + __shfl_xor_sync(0xffffffffu, b4 ? v[e] : v[4 + e], 16);
#pragma unroll
                for (int e = 0; e < 2; e++)
                    w2[e] = (b3 ? w4[2 + e] : w4[e]) + __shfl_xor_sync(0xffffffffu, b3 ? w4[e] : w4[2 + e], 8);
                float y = (b2 ? w2[1] : w2[0]) + __shfl_xor_sync(0xffffffffu, b2 ? w2[0] : w2[1], 4);
                y += __shfl_xor_sync(0xffffffffu, y, 2);
                y += __shfl_xor_sync(0xffffffffu, y, 1);
                const int m = lane >> 2, u = m >> 1;
                if ((lane & 3) == 0 && j + u < n_k) (m & 1 ? wgb : wga)[j + u] = y;
            }
            __syncwarp();
            // chain rule, one kept image per lane
            if (keep) {
                const int j = slot;
                int q, m2, m0, m1;
                divmod_small(i, N2, rN2, q, m2);
                divmod_small(q, N1, rN1, m0, m1);
                const int mi[3] = {m0, N0 + m1, N0 + N1 + m2};
                const int rr[3] = {(m0 - N0 / 2) & 1, (m1 - N1 / 2) & 1, (m2 - N2 / 2) & 1};
                float v[3], A[3];
                float4 dp[3];
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const float4 t = tab[mi[d]];
                    v[d] = t.z;
                    A[d] = t.w;
                    dp[d] = tabd[mi[d]];
                }
                const float d2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
                const float inv_d = rsqrtf(d2);
                const float att = A[0] * A[1] * A[2];
                float Ds = 1.f, Dm = 1.f, cs_ = 0.f, cm = 0.f;
                float ms[3] = {0.f, 0.f, 0.f};   // mirrored source axis
                if (spkr != P_OMNI) {
#pragma unroll
                    for (int d = 0; d < 3; d++) ms[d] = (rr[d] ? -os[d] : os[d]);
                    cs_ = -(ms[0] * v[0] + ms[1] * v[1] + ms[2] * v[2]) * inv_d * inv_os;
                    Ds = pattern_gain(cs_, spkr);
                }
                if (mic != P_OMNI) {
                    cm = (orr[0] * v[0] + orr[1] * v[1] + orr[2] * v[2]) * inv_d * inv_or;
                    Dm = pattern_gain(cm, mic);
                }
                const float g0 = 0.0795774715459476679f * inv_d;   // 1 / (4 pi d)
                const float amp = att * Ds * Dm * g0;
                const float GA = wga[j];
                const float GT = -amp * wgb[j];                      // dL/dtau
                // beta: d att / d beta_w = -e_w (-beta_w)^(e_w - 1) * (the other five factors);
                // per axis the walls' factors are (-b_lo)^e_lo and (-b_hi)^e_hi
                const float dA = GA * Ds * Dm * g0;   // dL / d att
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const float rest = dA * A[(d + 1) % 3] * A[(d + 2) % 3];
                    acc(2 * d) = fmaf(-rest * dp[d].y, dp[d].z, acc(2 * d));
                    acc(2 * d + 1) = fmaf(-rest * dp[d].x, dp[d].w, acc(2 * d + 1));
                }
                // d amp / d v and d tau / d v
                const float ds = pattern_slope(spkr), dm = pattern_slope(mic);
                float dv[3];
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const float u = v[d] * inv_d;
                    float damp = -amp * u * inv_d;                          // 1/d term
                    if (spkr != P_OMNI)   // d cos_s / d v = (-ms/|o| - cos_s u) / d
                        damp += att * g0 * Dm * ds * (-ms[d] * inv_os - cs_ * u) * inv_d;
                    if (mic != P_OMNI)    // d cos_m / d v = (o/|o| - cos_m u) / d
                        damp += att * g0 * Ds * dm * (orr[d] * inv_or - cm * u) * inv_d;
                    dv[d] = GA * damp + GT * fs_c * u;
                }
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    acc(6 + d) += rr[d] ? -dv[d] : dv[d];   // source: image coordinate (1 - 2 refl) src
                    acc(9 + d) -= dv[d];                    // receiver
                }
                if (spkr != P_OMNI) {   // d cos_s / d o = (-(1-2r) v / d - cos_s o / |o|) / |o|
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        const float dcs = (-(rr[d] ? -v[d] : v[d]) * inv_d - cs_ * os[d] * inv_os) * inv_os;
                        acc(12 + d) = fmaf(GA * att * g0 * Dm * ds, dcs, acc(12 + d));
                    }
                }
                if (mic != P_OMNI) {    // d cos_m / d o = (v / d - cos_m o / |o|) / |o|
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        const float dcm = (v[d] * inv_d - cm * orr[d] * inv_or) * inv_or;
                        acc(15 + d) = fmaf(GA * att * g0 * Ds * dm, dcm, acc(15 + d));
                    }
                }
            }
            __syncwarp();   // the scratch is rewritten by the next group
            if (gbase + kBThreads < i_end) geometry(gbase + kBThreads + lane);
        }
        // ---- item partials: warp sums, then warps in order
#pragma unroll
        for (int q = 0; q < kGrad; q++) {
            float v = acc(q);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) red[warp * kGrad + q] = v;
        }
        __syncthreads();
        if (tid < kGrad) {
            float s = 0.0f;
            for (int w = 0; w < kBWarps; w++) s += red[w * kGrad + tid];
            P.item_grad[(long)item_id * kGrad + tid] = s;
        }
        __syncthreads();
    }
#undef acc
}

// Sum of item partials per target of the five sets (rooms: beta; sources: position,
// orientation; receivers: position, orientation).  Target t of a set sums components
// [comp_lo, comp_lo + n_comp) of the items list[ptr[t]..ptr[t+1]) into
// out[t * n_comp + c].  A set with out == nullptr has no targets.
struct GradSet {
    const int *ptr, *list;
    int n_target, comp_lo, n_comp;
    float *out;
};
struct GradSets {
    GradSet s[5];
};

// One block per target: its threads take the target's items in a fixed stride, then
// a fixed xor tree per warp and the warp sums in order -- deterministic, and a target
// with thousands of items (one room of a long trajectory) is summed by the whole
// block instead of one warp.
constexpr int kRedThreads = 128;

__global__ void __launch_bounds__(kRedThreads) grad_reduce_kernel(const float *item_grad, GradSets G) {
    __shared__ float red[kRedThreads / 32][6];
    int t = blockIdx.x, k = 0;
    while (k < 5 && t >= G.s[k].n_target) t -= G.s[k++].n_target;
    if (k == 5) return;
    const GradSet S = G.s[k];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int p = S.ptr[t] + threadIdx.x; p < S.ptr[t + 1]; p += kRedThreads) {
        const float *row = item_grad + (long)S.list[p] * kGrad + S.comp_lo;
#pragma unroll
        for (int c = 0; c < 6; c++)
            if (c < S.n_comp) v[c] += row[c];
    }
#pragma unroll
    for (int c = 0; c < 6; c++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
        if (lane == 0) red[warp][c] = v[c];
    }
    __syncthreads();
    if (threadIdx.x < S.n_comp) {
        float sum = 0.0f;
#pragma unroll
        for (int w = 0; w < kRedThreads / 32; w++) sum += red[w][threadIdx.x];
        S.out[t * S.n_comp + threadIdx.x] = sum;
    }
}

size_t ism_backward_smem_bytes(int tpl, int max_tseg, int pad, int axis_cap) {
    (void)tpl;
    return kBThreads * (2 * sizeof(float4) + 2 * sizeof(float)) + 4 * sizeof(int) +
           (kBWarps + kBThreads) * kGrad * sizeof(float) +
           (size_t)((max_tseg + 2 * pad + 3) & ~3) * sizeof(float) + (size_t)axis_cap * 2 * sizeof(float4);
}

template <int TPL, bool CLAMP>
static cudaError_t bwd_tpl(const BwdLaunch &p, int grid, size_t smem, cudaStream_t st) {
    static bool attr_set = false;   // per process; the attribute is per function
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(ism_backward_kernel<TPL, CLAMP>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    ism_backward_kernel<TPL, CLAMP><<<grid, kBThreads, smem, st>>>(p);
    return cudaGetLastError();
}

cudaError_t ism_backward_launch(int tpl, const RoomDesc *rooms, const IsmItem *items, int n_items,
                                const float *pos_src, const float *pos_rcv, const float *orv_src,
                                const float *orv_rcv, const float *grad, float *item_grad,
                                int *work_counter, int *status, int max_tseg, int axis_cap, int grid,
                                int clamp, cudaStream_t st) {
    BwdLaunch p;
    p.axis_cap = axis_cap;
    p.rooms = rooms; p.items = items; p.n_items = n_items;
    p.pos_src = pos_src; p.pos_rcv = pos_rcv; p.orv_src = orv_src; p.orv_rcv = orv_rcv;
    p.grad = grad; p.item_grad = item_grad; p.work_counter = work_counter; p.status = status;
    p.max_tseg = max_tseg;
    p.pad = 64 * tpl;   // >= 2 * 32 * TPL reach of the taps on either side
    size_t smem = ism_backward_smem_bytes(tpl, max_tseg, p.pad, axis_cap);
    cudaError_t e = cudaMemsetAsync(work_counter, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    // taps beyond |x| < Tw/2 exist only when the window does not fill the lanes exactly
    switch (tpl * 2 + (clamp ? 1 : 0)) {
    case 4: return bwd_tpl<2, false>(p, grid, smem, st);
    case 5: return bwd_tpl<2, true>(p, grid, smem, st);
    case 8: return bwd_tpl<4, false>(p, grid, smem, st);
    case 9: return bwd_tpl<4, true>(p, grid, smem, st);
    case 16: return bwd_tpl<8, false>(p, grid, smem, st);
    case 17: return bwd_tpl<8, true>(p, grid, smem, st);
    case 24: return bwd_tpl<12, false>(p, grid, smem, st);
    case 25: return bwd_tpl<12, true>(p, grid, smem, st);
    case 32: return bwd_tpl<16, false>(p, grid, smem, st);
    case 33: return bwd_tpl<16, true>(p, grid, smem, st);
    case 48: return bwd_tpl<24, false>(p, grid, smem, st);
    case 49: return bwd_tpl<24, true>(p, grid, smem, st);
    default: return cudaErrorInvalidValue;
    }
}

// One launch for every requested gradient.  csr[0..5] = room ptr/list, source
// ptr/list, receiver ptr/list; out[0..4] = beta, source position, receiver position,
// source orientation, receiver orientation (nullptr: not requested).
cudaError_t grad_reduce_launch(const float *item_grad, const int *const csr[6], int n_rooms, int n_src,
                               int n_rcv, float *const out[5], cudaStream_t st) {
    GradSets G;
    const int n_t[5] = {n_rooms, n_src, n_rcv, n_src, n_rcv};
    const int which[5] = {0, 1, 2, 1, 2}, lo[5] = {0, 6, 9, 12, 15}, nc[5] = {6, 3, 3, 3, 3};
    long targets = 0;
    for (int k = 0; k < 5; k++) {
        G.s[k] = GradSet{csr[2 * which[k]], csr[2 * which[k] + 1], out[k] ? n_t[k] : 0, lo[k], nc[k], out[k]};
        targets += G.s[k].n_target;
    }
    if (targets <= 0) return cudaSuccess;
    if (targets > 0x7fffffffL) return cudaErrorInvalidValue;
    grad_reduce_kernel<<<(unsigned)targets, kRedThreads, 0, st>>>(item_grad, G);
    return cudaGetLastError();
}

// Resident blocks per SM of the adjoint kernel with `smem` bytes of shared memory.
int ism_backward_blocks_per_sm(int tpl, int clamp, size_t smem) {
    int n = 0;
    switch (tpl * 2 + (clamp ? 1 : 0)) {
#define OCC(T, C) case 2 * T + C: cudaFuncSetAttribute(ism_backward_kernel<T, (bool)C>, \
        cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024); \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ism_backward_kernel<T, (bool)C>, kBThreads, smem); break;
        OCC(2, 0) OCC(2, 1) OCC(4, 0) OCC(4, 1) OCC(8, 0) OCC(8, 1)
        OCC(12, 0) OCC(12, 1) OCC(16, 0) OCC(16, 1) OCC(24, 0) OCC(24, 1)
#undef OCC
    default: return 0;
    }
    return n;
}

}  // namespace gpurir
