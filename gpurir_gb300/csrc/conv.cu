// conv.cu -- FFT convolution of trajectory segments with their RIRs, and the
// overlap-add of simulateTrajectory, for sm_103a.
//
// Replaces gpuRIR's cuFFT pipeline (src/gpuRIR_cuda.cu:933-1023: R2C of the
// segments and the RIRs, complexPointwiseMulAndScale :463-482, C2R) and the
// float64 Python overlap-add loop (gpuRIR/__init__.py:215-219).
//
// Real FFTs of size N = 2M are computed as M-point complex FFTs of the packed
// sequence z[n] = x[2n] + i x[2n+1], with the usual split into even/odd
// spectra.  The complex FFT is the self-sorting Stockham formulation
// (radix-4 passes, one radix-2 pass when log2 M is odd) with ping-pong buffers
// in shared memory (M <= 8192) or in a per-block global scratch (larger M).
// Twiddles come from a table W[m] = exp(-2 pi i m / N), m < N, built once per
// size with sincospi.
#include <algorithm>

#include "gpurir_internal.cuh"

namespace gpurir {

constexpr int kFftThreads = 1024;
constexpr int kSmemFftMax = 8192;   // complex points held in shared memory (2 x 64 KB)

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

__global__ void twiddle_kernel(float2 *w, int n) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    double s, c;
    sincospi(-2.0 * (double)m / (double)n, &s, &c);   // FP64 once per size: exact to float rounding
    w[m] = make_float2((float)c, (float)s);
}

// In-block complex FFT of M points (power of two) from buf0; returns the buffer
// that holds the result.  INV conjugates the twiddles (unnormalised inverse).
// tw[m] = exp(-2 pi i m / M) for m < 3M/4 (shared memory, or the global table
// read with stride 2 when TS = 2: the size-N table holds exp(-2 pi i m/M) at 2m).
template <bool INV, int TS>
__device__ float2 *block_fft(float2 *buf0, float2 *buf1, int M, const float2 *tw) {
    float2 *src = buf0, *dst = buf1;
    int Ns = 1;
    int log2M = 31 - __clz(M);
    if (log2M & 1) {   // one radix-2 pass first
        for (int j = threadIdx.x; j < M / 2; j += blockDim.x) {
            float2 a = src[j], b = src[j + M / 2];
            dst[2 * j] = cadd(a, b);
            dst[2 * j + 1] = csub(a, b);
        }
        __syncthreads();
        float2 *t = src; src = dst; dst = t;
        Ns = 2;
    }
    for (; Ns < M; Ns *= 4) {
        const int q = M / 4;
        const int tstep = M / (Ns * 4);   // twiddle index stride in the M-point table
        for (int j = threadIdx.x; j < q; j += blockDim.x) {
            const int k = j & (Ns - 1);
            float2 v0 = src[j], v1 = src[j + q], v2 = src[j + 2 * q], v3 = src[j + 3 * q];
            if (Ns > 1) {
                float2 w1 = tw[TS * (k * tstep)];
                float2 w2 = tw[TS * (2 * k * tstep)];
                float2 w3 = tw[TS * (3 * k * tstep)];
                if (INV) { w1 = cconj(w1); w2 = cconj(w2); w3 = cconj(w3); }
                v1 = cmul(v1, w1);
                v2 = cmul(v2, w2);
                v3 = cmul(v3, w3);
            }
            const float2 t0 = cadd(v0, v2), t1 = csub(v0, v2), t2 = cadd(v1, v3);
            float2 t3 = csub(v1, v3);
            t3 = INV ? make_float2(-t3.y, t3.x) : make_float2(t3.y, -t3.x);   // x (+i) or (-i)
            const int o = (j - k) * 4 + k;
            dst[o] = cadd(t0, t2);
            dst[o + Ns] = cadd(t1, t3);
            dst[o + 2 * Ns] = csub(t0, t2);
            dst[o + 3 * Ns] = csub(t1, t3);
        }
        __syncthreads();
        float2 *t = src; src = dst; dst = t;
    }
    return src;
}

// Twiddles of one block.  In shared memory (M <= kSmemFftMax): twM[m] =
// exp(-2 pi i m/M), m < 3M/4, and twN[k] = exp(-2 pi i k/N), k <= M/2, copied from
// the global size-N table once per block; beyond that the global table is read
// directly (stride 2 for the M-point twiddles).
struct Twiddles {
    const float2 *m;   // M-point twiddles
    int ms;            // index stride into m
    const float2 *n;   // N-point twiddles, k <= M/2
};

__device__ Twiddles load_twiddles(float2 *sm_tw, int M, const float2 *W, bool in_smem) {
    if (!in_smem) return Twiddles{W, 2, W};
    float2 *twm = sm_tw, *twn = sm_tw + 3 * M / 4;
    for (int m = threadIdx.x; m < 3 * M / 4; m += blockDim.x) twm[m] = __ldg(&W[2 * m]);
    for (int k = threadIdx.x; k <= M / 2; k += blockDim.x) twn[k] = __ldg(&W[k]);
    __syncthreads();
    return Twiddles{twm, 1, twn};
}

__device__ __forceinline__ float2 *fft_fwd(float2 *a, float2 *b, int M, const Twiddles &T) {
    return T.ms == 1 ? block_fft<false, 1>(a, b, M, T.m) : block_fft<false, 2>(a, b, M, T.m);
}
__device__ __forceinline__ float2 *fft_inv(float2 *a, float2 *b, int M, const Twiddles &T) {
    return T.ms == 1 ? block_fft<true, 1>(a, b, M, T.m) : block_fft<true, 2>(a, b, M, T.m);
}

// exp(-2 pi i k/N) and exp(-2 pi i (M - k)/N) = -conj(exp(-2 pi i k/N)), 0 <= k <= M/2
__device__ __forceinline__ void twiddle_pair(const Twiddles &T, int k, float2 &wk, float2 &wm) {
    wk = T.n[k];
    wm = make_float2(-wk.x, wk.y);
}

// Forward real FFT of the zero-padded length-`len` row x into X[0..M] (M + 1 bins),
// scaled by `scale`.  z (M complex) is packed from x; work buffers a, b.
__device__ void real_fft_row(const float *x, int len, int M, const Twiddles &T, float2 *a, float2 *b,
                             float2 *X, float scale) {
    for (int n = threadIdx.x; n < M; n += blockDim.x) {
        const int i0 = 2 * n, i1 = 2 * n + 1;
        a[n] = make_float2(i0 < len ? x[i0] : 0.0f, i1 < len ? x[i1] : 0.0f);
    }
    __syncthreads();
    float2 *Z = fft_fwd(a, b, M, T);
    for (int k = threadIdx.x; k <= M / 2; k += blockDim.x) {
        const int km = (M - k) & (M - 1);
        const float2 zk = Z[k], zm = Z[km];
        // k and M - k together
        const float2 ze = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
        const float2 zo = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
        const float2 ze2 = make_float2(ze.x, -ze.y), zo2 = make_float2(zo.x, -zo.y);   // bins M - k
        float2 wk, wm;
        twiddle_pair(T, k, wk, wm);
        const float2 xk = cadd(ze, cmul(wk, zo));
        const float2 xm = cadd(ze2, cmul(wm, zo2));
        X[k] = make_float2(xk.x * scale, xk.y * scale);
        X[M - k] = make_float2(xm.x * scale, xm.y * scale);
    }
    __syncthreads();
}

// Segment spectra: Sg[p][0..M] = FFT_N(segment p) / M (the 1/M of the inverse folded in).
__global__ void __launch_bounds__(kFftThreads) segment_spectra_kernel(
        const float *seg, int P, int S, int M, const float2 *W, float2 *Sg, float2 *scratch) {
    extern __shared__ __align__(16) float2 sm[];
    const bool in_smem = M <= kSmemFftMax;
    float2 *a = in_smem ? sm : scratch + (size_t)blockIdx.x * 2 * M;
    float2 *b = a + M;
    const Twiddles T = load_twiddles(sm + 2 * M, M, W, in_smem);
    for (int p = blockIdx.x; p < P; p += gridDim.x)
        real_fft_row(seg + (size_t)p * S, S, M, T, a, b, Sg + (size_t)p * (M + 1), 1.0f / (float)M);
}

// One block per (point p, receiver r): conv[p][r][0..S+L-1) = segment p * RIR (p, r).
__global__ void __launch_bounds__(kFftThreads) rir_conv_kernel(
        const float *rir, int P, int R, int L, int S, int M, const float2 *W, const float2 *Sg,
        float *out, long out_ld, float2 *scratch) {
    extern __shared__ __align__(16) float2 sm[];
    const bool in_smem = M <= kSmemFftMax;
    float2 *a = in_smem ? sm : scratch + (size_t)blockIdx.x * 2 * M;
    float2 *b = a + M;
    const Twiddles T = load_twiddles(sm + 2 * M, M, W, in_smem);
    const int n_out = S + L - 1;
    for (int pr = blockIdx.x; pr < P * R; pr += gridDim.x) {
        const int p = pr / R;
        const float *x = rir + (size_t)pr * L;
        for (int n = threadIdx.x; n < M; n += blockDim.x) {
            const int i0 = 2 * n, i1 = 2 * n + 1;
            a[n] = make_float2(i0 < L ? x[i0] : 0.0f, i1 < L ? x[i1] : 0.0f);
        }
        __syncthreads();
        float2 *Z = fft_fwd(a, b, M, T);
        float2 *Y = (Z == a) ? b : a;   // the other buffer receives the inverse input
        const float2 *sp = Sg + (size_t)p * (M + 1);
        for (int k = threadIdx.x; k <= M / 2; k += blockDim.x) {
            const int km = (M - k) & (M - 1);
            const float2 zk = Z[k], zm = Z[km];
            const float2 ze = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
            const float2 zo = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
            const float2 ze2 = make_float2(ze.x, -ze.y), zo2 = make_float2(zo.x, -zo.y);
            float2 wk, wm;
            twiddle_pair(T, k, wk, wm);
            // spectra of the RIR at bins k and M - k, times the segment spectrum
            const float2 yk = cmul(cadd(ze, cmul(wk, zo)), __ldg(&sp[k]));
            const float2 ym = cmul(cadd(ze2, cmul(wm, zo2)), __ldg(&sp[M - k]));
            // inverse packing: Z'[k] = Ye + i Yo, Ye = (Y[k] + conj Y[M-k])/2,
            // Yo = (Y[k] - conj Y[M-k]) conj(W[k]) / 2   (and the same at M - k)
            const float2 yec = make_float2(0.5f * (yk.x + ym.x), 0.5f * (yk.y - ym.y));
            const float2 yod = cmul(make_float2(0.5f * (yk.x - ym.x), 0.5f * (yk.y + ym.y)), cconj(wk));
            Y[k] = make_float2(yec.x - yod.y, yec.y + yod.x);
            if (k != 0 && km != k) {
                const float2 yec2 = make_float2(0.5f * (ym.x + yk.x), 0.5f * (ym.y - yk.y));
                const float2 yod2 = cmul(make_float2(0.5f * (ym.x - yk.x), 0.5f * (ym.y + yk.y)), cconj(wm));
                Y[km] = make_float2(yec2.x - yod2.y, yec2.y + yod2.x);
            }
        }
        __syncthreads();
        float2 *other = (Y == a) ? b : a;
        float2 *z = fft_inv(Y, other, M, T);
        float *o = out + (size_t)pr * out_ld;
        for (int n = threadIdx.x; n < M; n += blockDim.x) {
            const float2 v = z[n];
            if (2 * n < n_out) o[2 * n] = v.x;
            if (2 * n + 1 < n_out) o[2 * n + 1] = v.y;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Register-resident FFT convolution for M = 1024 .. 8192 (N = 2M <= 16384).
//
// M/16 threads per row; each holds 16 complex values.  A Stockham pass of radix
// 16 (then one of radix M/Ns in {2, 4, 8}) reads its 16 inputs from shared
// memory, applies the twiddles, does the DFT in registers and writes its 16
// outputs back: log16(M) + 1 round trips per FFT instead of log4(M) with two
// buffers.  One buffer per row, padded by one element per 16 so that every
// pass is free of bank conflicts; several rows per SM overlap their loads,
// passes and stores.  The first pass reads the RIR straight from global memory.
// ---------------------------------------------------------------------------
constexpr float kC8 = 0.92387953251128674f;    // cos(pi/8)
constexpr float kS8 = 0.38268343236508977f;    // sin(pi/8)
constexpr float kR2 = 0.70710678118654752f;    // sqrt(2)/2

__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

// rows transformed together per block by rir_conv_reg_kernel
constexpr int kConvRows = 2;

// x * (-i) (forward) or x * (+i) (inverse)
template <bool INV>
__device__ __forceinline__ float2 rot_q(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <bool INV>
__device__ __forceinline__ void dft2(float2 &a, float2 &b) {
    const float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

// in place: a[0..3] -> X[0..3], X[k] = sum_n a[n] w4^(nk), w4 = exp(-+2 pi i/4)
template <bool INV>
__device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2, float2 &a3) {
    const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3);
    const float2 t3 = rot_q<INV>(csub(a1, a3));
    a0 = cadd(t0, t2);
    a1 = cadd(t1, t3);
    a2 = csub(t0, t2);
    a3 = csub(t1, t3);
}

// exp(-+2 pi i m/16) for the twiddles inside a radix-16 DFT
template <bool INV>
__device__ __forceinline__ float2 w16(int m) {
    float c, s;
    switch (m) {
    case 1: c = kC8; s = kS8; break;
    case 2: c = kR2; s = kR2; break;
    case 3: c = kS8; s = kC8; break;
    case 4: c = 0.0f; s = 1.0f; break;
    case 6: c = -kR2; s = kR2; break;
    case 9: c = -kC8; s = -kS8; break;
    default: c = 1.0f; s = 0.0f; break;
    }
    return make_float2(c, INV ? s : -s);
}

// v[n], n = 4 n1 + n2  ->  V[k1 + 4 k2] held in v[4 k1 + k2] (digit-reversed; the
// writer below reads output s from v[dr16(s)])
template <bool INV>
__device__ __forceinline__ void dft16(float2 (&v)[16]) {
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) dft4<INV>(v[n2], v[4 + n2], v[8 + n2], v[12 + n2]);
    // v[4 k1 + n2] now holds Y[k1][n2]; twiddle by w16^(n2 k1)
#pragma unroll
    for (int k1 = 1; k1 < 4; k1++)
#pragma unroll
        for (int n2 = 1; n2 < 4; n2++) v[4 * k1 + n2] = cmul(v[4 * k1 + n2], w16<INV>(n2 * k1));
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) dft4<INV>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
}

__host__ __device__ constexpr int dr16(int s) { return 4 * (s & 3) + (s >> 2); }

// Twiddles w^r, r = 1..15, of one radix-16 pass (w = W[e]): w, w^2, w^4, w^8 from the
// table, the others as products of at most three of them (4 loads instead of 15; error
// within 3 roundings).
__device__ __forceinline__ void twiddle_powers(const float2 *__restrict__ W, int e, float2 (&t)[16]) {
    t[1] = __ldg(&W[e]);
    t[2] = __ldg(&W[2 * e]);
    t[4] = __ldg(&W[4 * e]);
    t[8] = __ldg(&W[8 * e]);
    t[3] = cmul(t[1], t[2]);
    t[5] = cmul(t[1], t[4]);
    t[6] = cmul(t[2], t[4]);
    t[7] = cmul(t[3], t[4]);
    t[9] = cmul(t[1], t[8]);
    t[10] = cmul(t[2], t[8]);
    t[11] = cmul(t[3], t[8]);
    t[12] = cmul(t[4], t[8]);
    t[13] = cmul(t[5], t[8]);
    t[14] = cmul(t[6], t[8]);
    t[15] = cmul(t[7], t[8]);
}

// One radix-16 Stockham pass at stride Ns for the thread's j (= thread index):
// twiddle, DFT, write dst[(j - k) 16 + k + s Ns], k = j mod Ns.
// W: exp(-2 pi i m/N) for m < N = 2M.
template <bool INV, int M>
__device__ __forceinline__ void pass16_compute_write(float2 (&v)[16], float2 *buf, int j, int Ns,
                                                     const float2 *__restrict__ W) {
    const int k = j & (Ns - 1);
    if (Ns > 1) {
        float2 t[16];
        twiddle_powers(W, k * ((2 * M) / (Ns * 16)), t);   // W_{16 Ns}^1 = W_N^step
#pragma unroll
        for (int r = 1; r < 16; r++) v[r] = cmul(v[r], INV ? cconj(t[r]) : t[r]);
    }
    dft16<INV>(v);
    const int base = (j - k) * 16 + k;
#pragma unroll
    for (int s = 0; s < 16; s++) buf[pad16(base + s * Ns)] = v[dr16(s)];
}

// The full M-point FFT of the values in `buf` (natural order, padded), or, for
// the forward transform, of v[] already loaded for pass 1 (LOADED).  Result in
// `buf`, natural order.  Every thread of the block calls it.
template <bool INV, int M, bool LOADED>
__device__ __forceinline__ void reg_fft(float2 (&v)[16], float2 *buf, const float2 *__restrict__ W) {
    constexpr int T = M / 16;
    const int j = threadIdx.x;
    int Ns = 1;
    if (!LOADED) {
#pragma unroll
        for (int r = 0; r < 16; r++) v[r] = buf[pad16(j + r * T)];
        __syncthreads();
    }
    pass16_compute_write<INV, M>(v, buf, j, 1, W);
    __syncthreads();
    Ns = 16;
#pragma unroll 1
    for (; Ns * 16 <= M; Ns *= 16) {
#pragma unroll
        for (int r = 0; r < 16; r++) v[r] = buf[pad16(j + r * T)];
        __syncthreads();
        pass16_compute_write<INV, M>(v, buf, j, Ns, W);
        __syncthreads();
    }
    if (Ns < M) {
        // last pass, radix R = M / Ns in {2, 4, 8}: 16 / R groups per thread, j' = j + T g;
        // each group reads and writes only its own R elements (j' + r M/R = j' + r Ns)
        constexpr int dummy = 0;
        (void)dummy;
        const int R = M / Ns;
        const int step = (2 * M) / M;   // W_M^1 = W_N^2
        for (int g = 0; g < 16 / R; g++) {
            const int jj = j + T * g;   // jj < M / R = Ns, so k = jj
            float2 a[8];
            for (int r = 0; r < R; r++) a[r] = buf[pad16(jj + r * Ns)];
            for (int r = 1; r < R; r++) {
                float2 w = __ldg(&W[r * jj * step]);
                if (INV) w = cconj(w);
                a[r] = cmul(a[r], w);
            }
            if (R == 2) {
                dft2<INV>(a[0], a[1]);
            } else if (R == 4) {
                dft4<INV>(a[0], a[1], a[2], a[3]);
            } else {   // R == 8: two radix-4 over even/odd, then combine
                dft4<INV>(a[0], a[2], a[4], a[6]);
                dft4<INV>(a[1], a[3], a[5], a[7]);
                const float2 w1 = make_float2(kR2, INV ? kR2 : -kR2);
                const float2 w3 = make_float2(-kR2, INV ? kR2 : -kR2);
                const float2 o1 = cmul(a[3], w1), o2 = rot_q<INV>(a[5]), o3 = cmul(a[7], w3);
                const float2 e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6], o0 = a[1];
                a[0] = cadd(e0, o0); a[4] = csub(e0, o0);
                a[1] = cadd(e1, o1); a[5] = csub(e1, o1);
                a[2] = cadd(e2, o2); a[6] = csub(e2, o2);
                a[3] = cadd(e3, o3); a[7] = csub(e3, o3);
            }
            for (int s = 0; s < R; s++) buf[pad16(jj + s * Ns)] = a[s];
        }
    }
    __syncthreads();
}

// ROWS transforms at once (rows q at buf + q * pad16(M)): the same passes, barriers
// and twiddle loads serve every row, and each thread has ROWS independent DFTs in
// flight per pass.
template <bool INV, int M, int ROWS>
__device__ __forceinline__ void pass16_rows(float2 (&v)[ROWS][16], float2 *buf, int j, int Ns,
                                            const float2 *__restrict__ W) {
    constexpr int BS = M + M / 16;
    const int k = j & (Ns - 1);
    if (Ns > 1) {
        float2 t[16];
        twiddle_powers(W, k * ((2 * M) / (Ns * 16)), t);
#pragma unroll
        for (int r = 1; r < 16; r++) {
            const float2 w = INV ? cconj(t[r]) : t[r];
#pragma unroll
            for (int q = 0; q < ROWS; q++) v[q][r] = cmul(v[q][r], w);
        }
    }
#pragma unroll
    for (int q = 0; q < ROWS; q++) dft16<INV>(v[q]);
    const int base = (j - k) * 16 + k;
#pragma unroll
    for (int q = 0; q < ROWS; q++)
#pragma unroll
        for (int s = 0; s < 16; s++) buf[q * BS + pad16(base + s * Ns)] = v[q][dr16(s)];
}

template <bool INV, int M, bool LOADED, int ROWS>
__device__ __forceinline__ void reg_fft_rows(float2 (&v)[ROWS][16], float2 *buf, const float2 *__restrict__ W) {
    constexpr int T = M / 16, BS = M + M / 16;
    const int j = threadIdx.x;
    if (!LOADED) {
#pragma unroll
        for (int q = 0; q < ROWS; q++)
#pragma unroll
            for (int r = 0; r < 16; r++) v[q][r] = buf[q * BS + pad16(j + r * T)];
        __syncthreads();
    }
    pass16_rows<INV, M, ROWS>(v, buf, j, 1, W);
    __syncthreads();
    int Ns = 16;
#pragma unroll 1
    for (; Ns * 16 <= M; Ns *= 16) {
#pragma unroll
        for (int q = 0; q < ROWS; q++)
#pragma unroll
            for (int r = 0; r < 16; r++) v[q][r] = buf[q * BS + pad16(j + r * T)];
        __syncthreads();
        pass16_rows<INV, M, ROWS>(v, buf, j, Ns, W);
        __syncthreads();
    }
    if (Ns < M) {   // last pass, radix R = M / Ns in {2, 4, 8}, as in reg_fft
        const int R = M / Ns;
        for (int g = 0; g < 16 / R; g++) {
            const int jj = j + T * g;
            float2 a[ROWS][8];
#pragma unroll
            for (int q = 0; q < ROWS; q++)
                for (int r = 0; r < R; r++) a[q][r] = buf[q * BS + pad16(jj + r * Ns)];
            for (int r = 1; r < R; r++) {
                float2 w = __ldg(&W[r * jj * 2]);   // W_M^1 = W_N^2
                if (INV) w = cconj(w);
#pragma unroll
                for (int q = 0; q < ROWS; q++) a[q][r] = cmul(a[q][r], w);
            }
#pragma unroll
            for (int q = 0; q < ROWS; q++) {
                if (R == 2) {
                    dft2<INV>(a[q][0], a[q][1]);
                } else if (R == 4) {
                    dft4<INV>(a[q][0], a[q][1], a[q][2], a[q][3]);
                } else {
                    dft4<INV>(a[q][0], a[q][2], a[q][4], a[q][6]);
                    dft4<INV>(a[q][1], a[q][3], a[q][5], a[q][7]);
                    const float2 w1 = make_float2(kR2, INV ? kR2 : -kR2);
                    const float2 w3 = make_float2(-kR2, INV ? kR2 : -kR2);
                    const float2 o1 = cmul(a[q][3], w1), o2 = rot_q<INV>(a[q][5]), o3 = cmul(a[q][7], w3);
                    const float2 e0 = a[q][0], e1 = a[q][2], e2 = a[q][4], e3 = a[q][6], o0 = a[q][1];
                    a[q][0] = cadd(e0, o0); a[q][4] = csub(e0, o0);
                    a[q][1] = cadd(e1, o1); a[q][5] = csub(e1, o1);
                    a[q][2] = cadd(e2, o2); a[q][6] = csub(e2, o2);
                    a[q][3] = cadd(e3, o3); a[q][7] = csub(e3, o3);
                }
                for (int s = 0; s < R; s++) buf[q * BS + pad16(jj + s * Ns)] = a[q][s];
            }
        }
    }
    __syncthreads();
}

// For M = 2 * 16^n the last Stockham pass of reg_fft_rows is a radix-2 pass, one more
// shared-memory round trip and barrier for two additions per element.  The
// convolution folds it into its spectral step instead (and the inverse's first
// radix-2 pass likewise): reg_fft_rows_head stops before that pass, leaving the
// half-size DFTs A = buf[0, M/2) and B = buf[M/2, M) (Z[k] = A[k] + W_M^k B[k],
// Z[k + M/2] = A[k] - W_M^k B[k]); reg_fft_rows_tail runs the radix-16 passes that
// follow an external first radix-2 pass (Ns = 2, 32, 512, ...).
template <bool INV, int M, int ROWS>
__device__ __forceinline__ void reg_fft_rows_head(float2 (&v)[ROWS][16], float2 *buf, const float2 *__restrict__ W) {
    constexpr int T = M / 16, BS = M + M / 16;
    const int j = threadIdx.x;
    pass16_rows<INV, M, ROWS>(v, buf, j, 1, W);   // v loaded by the caller
    __syncthreads();
    int Ns = 16;
#pragma unroll 1
    for (; Ns * 16 <= M; Ns *= 16) {
#pragma unroll
        for (int q = 0; q < ROWS; q++)
#pragma unroll
            for (int r = 0; r < 16; r++) v[q][r] = buf[q * BS + pad16(j + r * T)];
        __syncthreads();
        pass16_rows<INV, M, ROWS>(v, buf, j, Ns, W);
        __syncthreads();
    }
}

template <bool INV, int M, int ROWS>
__device__ __forceinline__ void reg_fft_rows_tail(float2 (&v)[ROWS][16], float2 *buf, const float2 *__restrict__ W) {
    constexpr int T = M / 16, BS = M + M / 16;
    const int j = threadIdx.x;
#pragma unroll 1
    for (int Ns = 2; Ns * 16 <= M; Ns *= 16) {
#pragma unroll
        for (int q = 0; q < ROWS; q++)
#pragma unroll
            for (int r = 0; r < 16; r++) v[q][r] = buf[q * BS + pad16(j + r * T)];
        __syncthreads();
        pass16_rows<INV, M, ROWS>(v, buf, j, Ns, W);
        __syncthreads();
    }
}

// Spectral step of one bin pair (k, M - k) of the convolution: real-FFT bins from the
// packed spectrum values zk = Z[k], zm = Z[(M - k) mod M], times the segment spectrum
// (sk, sm), repacked for the inverse packed FFT: returns Y'[k] and Y'[M - k].
__device__ __forceinline__ void conv_bin_pair(float2 zk, float2 zm, float2 wk, float2 sk, float2 sm, float2 &ok,
                                              float2 &om) {
    const float2 ze = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
    const float2 zo = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
    const float2 ze2 = make_float2(ze.x, -ze.y), zo2 = make_float2(zo.x, -zo.y);
    const float2 wm = make_float2(-wk.x, wk.y);
    const float2 yk = cmul(cadd(ze, cmul(wk, zo)), sk);
    const float2 ym = cmul(cadd(ze2, cmul(wm, zo2)), sm);
    const float2 yec = make_float2(0.5f * (yk.x + ym.x), 0.5f * (yk.y - ym.y));
    const float2 yod = cmul(make_float2(0.5f * (yk.x - ym.x), 0.5f * (yk.y + ym.y)), cconj(wk));
    ok = make_float2(yec.x - yod.y, yec.y + yod.x);
    const float2 yec2 = make_float2(0.5f * (ym.x + yk.x), 0.5f * (ym.y - yk.y));
    const float2 yod2 = cmul(make_float2(0.5f * (ym.x - yk.x), 0.5f * (ym.y + yk.y)), cconj(wm));
    om = make_float2(yec2.x - yod2.y, yec2.y + yod2.x);
}

// Pass-1 inputs of thread j straight from global memory: z[n] = x[2n] + i x[2n+1],
// n = j + r M/16, zero past `len` (8-byte loads when the row allows).
template <int M>
__device__ __forceinline__ void load_packed(const float *__restrict__ x, int len, float2 (&v)[16]) {
    constexpr int T = M / 16;
    const int j = threadIdx.x;
    if ((reinterpret_cast<uintptr_t>(x) & 7) == 0) {
#pragma unroll
        for (int r = 0; r < 16; r++) {
            const int n = j + r * T;
            if (2 * n + 1 < len) v[r] = __ldg(reinterpret_cast<const float2 *>(x) + n);
            else v[r] = make_float2(2 * n < len ? __ldg(&x[2 * n]) : 0.0f, 0.0f);
        }
    } else {
#pragma unroll
        for (int r = 0; r < 16; r++) {
            const int n = j + r * T;
            v[r] = make_float2(2 * n < len ? __ldg(&x[2 * n]) : 0.0f, 2 * n + 1 < len ? __ldg(&x[2 * n + 1]) : 0.0f);
        }
    }
}

// Segment spectra with the register FFT: Sg[p][0..M] = FFT_N(segment p) / M.
template <int M>
__global__ void __launch_bounds__(M / 16, 16384 / M) segment_spectra_reg_kernel(
        const float *__restrict__ seg, int P, int S, const float2 *__restrict__ W, float2 *__restrict__ Sg) {
    constexpr int T = M / 16;
    extern __shared__ __align__(16) float2 sm[];
    float2 *buf = sm;
    const int j = threadIdx.x;
    const float scale = 1.0f / (float)M;
    float2 v[16];
    for (int p = blockIdx.x; p < P; p += gridDim.x) {
        load_packed<M>(seg + (size_t)p * S, S, v);
        reg_fft<false, M, true>(v, buf, W);
        float2 *X = Sg + (size_t)p * (M + 1);
        for (int k = j; k <= M / 2; k += T) {
            const int km = (M - k) & (M - 1);
            const float2 zk = buf[pad16(k)], zm = buf[pad16(km)];
            const float2 ze = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
            const float2 zo = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
            const float2 ze2 = make_float2(ze.x, -ze.y), zo2 = make_float2(zo.x, -zo.y);
            const float2 wk = __ldg(&W[k]);
            const float2 wm = make_float2(-wk.x, wk.y);
            const float2 xk = cadd(ze, cmul(wk, zo));
            const float2 xm = cadd(ze2, cmul(wm, zo2));
            X[k] = make_float2(xk.x * scale, xk.y * scale);
            X[M - k] = make_float2(xm.x * scale, xm.y * scale);
        }
        __syncthreads();
    }
}

// Forward FFT of the rows (v loaded), spectral step and inverse FFT for M = 2 * 16^n, with
// the forward's last radix-2 pass and the inverse's first one folded into the spectral
// step.  Unit u in [0, M/4] takes the bins k = u, M - k, k' = M/2 - u, M - k': it reads
// A[k], B[k], A[k'], B[k'], forms Z[k], Z[k + M/2], Z[k'], Z[k' + M/2] exactly as the
// radix-2 pass would, does the spectral step of the pairs (k, M - k) and (k', M - k'),
// and writes the inverse's first radix-2 outputs 2k, 2k + 1, 2k', 2k' + 1.  All reads
// happen before a barrier and all writes after it (the writes land on other units'
// inputs); the values wait in v, free between the transforms.
template <int M, int ROWS>
__device__ __forceinline__ void conv_spectral_fused(float2 (&v)[ROWS][16], float2 *buf, const float2 *__restrict__ W,
                                                    const float2 *__restrict__ Sg, int pr0, int nq, int R) {
    constexpr int T = M / 16, BS = M + M / 16, H = M / 2, Q = M / 4;
    static_assert(Q == 4 * T, "four units per thread");
    const int j = threadIdx.x;
    reg_fft_rows_head<false, M, ROWS>(v, buf, W);
    float2 e[ROWS][2];   // unit M/4 (thread 0 only): Z[M/4], Z[3M/4]
#pragma unroll
    for (int q = 0; q < ROWS; q++) {
        const float2 *bq = buf + q * BS;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int u = j + i * T;
            if (u == 0) {   // bins 0 and M/2: Z[0] = A[0] + B[0], Z[M/2] = A[0] - B[0]
                float2 a0 = bq[pad16(0)], a1 = cmul(bq[pad16(H)], __ldg(&W[0]));
                v[q][4 * i] = cadd(a0, a1);
                v[q][4 * i + 1] = csub(a0, a1);
            } else {
                const int k = u, kp = H - u;
                const float2 ak = bq[pad16(k)], bk = cmul(bq[pad16(k + H)], __ldg(&W[2 * k]));
                const float2 ap = bq[pad16(kp)], bp = cmul(bq[pad16(kp + H)], __ldg(&W[2 * kp]));
                v[q][4 * i] = cadd(ak, bk);        // Z[k]
                v[q][4 * i + 1] = csub(ak, bk);    // Z[k + M/2] = Z[M - k']
                v[q][4 * i + 2] = cadd(ap, bp);    // Z[k']
                v[q][4 * i + 3] = csub(ap, bp);    // Z[k' + M/2] = Z[M - k]
            }
        }
        if (j == 0) {
            const float2 a = bq[pad16(Q)], b = cmul(bq[pad16(Q + H)], __ldg(&W[2 * Q]));
            e[q][0] = cadd(a, b);
            e[q][1] = csub(a, b);
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < ROWS; q++) {
        if (q >= nq) break;
        float2 *bq = buf + q * BS;
        const float2 *sp = Sg + (size_t)((pr0 + q) / R) * (M + 1);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int u = j + i * T;
            if (u == 0) {
                float2 y0, yM, yh, yh2;
                conv_bin_pair(v[q][0], v[q][0], __ldg(&W[0]), __ldg(&sp[0]), __ldg(&sp[M]), y0, yM);
                conv_bin_pair(v[q][1], v[q][1], __ldg(&W[H]), __ldg(&sp[H]), __ldg(&sp[H]), yh, yh2);
                bq[pad16(0)] = cadd(y0, yh);
                bq[pad16(1)] = csub(y0, yh);
            } else {
                const int k = u, kp = H - u;
                float2 yk, ymk, ykp, ymkp;
                // pair (k, M - k): Z[k], Z[M - k] = Z[k' + M/2]; pair (k', M - k'): Z[k'], Z[k + M/2]
                conv_bin_pair(v[q][4 * i], v[q][4 * i + 3], __ldg(&W[k]), __ldg(&sp[k]), __ldg(&sp[M - k]), yk, ymk);
                conv_bin_pair(v[q][4 * i + 2], v[q][4 * i + 1], __ldg(&W[kp]), __ldg(&sp[kp]), __ldg(&sp[M - kp]),
                              ykp, ymkp);
                // the inverse's first radix-2 pass: out[2j] = Y'[j] + Y'[j + M/2], out[2j + 1] = difference
                bq[pad16(2 * k)] = cadd(yk, ymkp);        // Y'[k + M/2] = Y'[M - k']
                bq[pad16(2 * k + 1)] = csub(yk, ymkp);
                bq[pad16(2 * kp)] = cadd(ykp, ymk);       // Y'[k' + M/2] = Y'[M - k]
                bq[pad16(2 * kp + 1)] = csub(ykp, ymk);
            }
        }
        if (j == 0) {
            float2 yq, y3q;
            conv_bin_pair(e[q][0], e[q][1], __ldg(&W[Q]), __ldg(&sp[Q]), __ldg(&sp[M - Q]), yq, y3q);
            bq[pad16(2 * Q)] = cadd(yq, y3q);
            bq[pad16(2 * Q + 1)] = csub(yq, y3q);
        }
    }
    __syncthreads();
    reg_fft_rows_tail<true, M, ROWS>(v, buf, W);
}

template <int M, int ROWS>
__global__ void __launch_bounds__(M / 16, (16384 / M / ROWS > 0 ? 16384 / M / ROWS : 1)) rir_conv_reg_kernel(
        const float *__restrict__ rir, int P, int R, int L, int S, const float2 *__restrict__ W,
        const float2 *__restrict__ Sg, float *__restrict__ out, long out_ld) {
    constexpr int T = M / 16, BS = M + M / 16;
    extern __shared__ __align__(16) float2 sm[];
    float2 *buf = sm;   // ROWS buffers of pad16(M) elements
    const int j = threadIdx.x;
    const int n_out = S + L - 1;
    float2 v[ROWS][16];
    const bool vec_out = (out_ld & 3) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    const int n_rows = P * R;
    for (int pr0 = blockIdx.x * ROWS; pr0 < n_rows; pr0 += gridDim.x * ROWS) {
        const int nq = min(ROWS, n_rows - pr0);   // rows of this group (uniform over the block)
        if (j == 0 && pr0 + (int)gridDim.x * ROWS < n_rows) {
            // the block's next RIR rows into L2 while these are transformed (whole 16-byte
            // units inside the rows only)
            const int nn = min(ROWS, n_rows - (pr0 + (int)gridDim.x * ROWS));
            const uintptr_t a = reinterpret_cast<uintptr_t>(rir + (size_t)(pr0 + gridDim.x * ROWS) * L);
            const uintptr_t lo = (a + 15) & ~(uintptr_t)15, hi = (a + (size_t)nn * L * sizeof(float)) & ~(uintptr_t)15;
            if (hi > lo)
                asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"((unsigned)(hi - lo))
                             : "memory");
        }
#pragma unroll
        for (int q = 0; q < ROWS; q++) {
            if (q < nq) {
                load_packed<M>(rir + (size_t)(pr0 + q) * L, L, v[q]);
            } else {
#pragma unroll
                for (int r = 0; r < 16; r++) v[q][r] = make_float2(0.0f, 0.0f);
            }
        }
        if constexpr (M == 8192) {
            conv_spectral_fused<M, ROWS>(v, buf, W, Sg, pr0, nq, R);
        } else {
        reg_fft_rows<false, M, true, ROWS>(v, buf, W);
        // spectrum of the RIR at k and M - k, times the segment's spectrum, repacked
        // for the inverse real FFT (same algebra as rir_conv_kernel).  The thread's k are
        // j + i T; their twiddles and segment spectra are loaded four k at a time before
        // any arithmetic (the transform's registers are free here), not one round trip
        // per k.
        for (int q = 0; q < nq; q++) {
            float2 *bq = buf + q * BS;
            const float2 *sp = Sg + (size_t)((pr0 + q) / R) * (M + 1);
            for (int k0 = j; k0 <= M / 2; k0 += 4 * T) {
                float2 wk4[4], sk4[4], sm4[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int k = k0 + i * T;
                    const int kk = min(k, M / 2);   // in bounds; results of k > M / 2 unused
                    wk4[i] = __ldg(&W[kk]);
                    sk4[i] = __ldg(&sp[kk]);
                    sm4[i] = __ldg(&sp[M - kk]);
                }
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int k = k0 + i * T;
                    if (k > M / 2) break;
                    const int km = (M - k) & (M - 1);
                    const float2 zk = bq[pad16(k)], zm = bq[pad16(km)];
                    const float2 ze = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
                    const float2 zo = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
                    const float2 ze2 = make_float2(ze.x, -ze.y), zo2 = make_float2(zo.x, -zo.y);
                    const float2 wk = wk4[i];
                    const float2 wm = make_float2(-wk.x, wk.y);
                    const float2 yk = cmul(cadd(ze, cmul(wk, zo)), sk4[i]);
                    const float2 ym = cmul(cadd(ze2, cmul(wm, zo2)), sm4[i]);
                    const float2 yec = make_float2(0.5f * (yk.x + ym.x), 0.5f * (yk.y - ym.y));
                    const float2 yod = cmul(make_float2(0.5f * (yk.x - ym.x), 0.5f * (yk.y + ym.y)), cconj(wk));
                    bq[pad16(k)] = make_float2(yec.x - yod.y, yec.y + yod.x);
                    if (k != 0 && km != k) {
                        const float2 yec2 = make_float2(0.5f * (ym.x + yk.x), 0.5f * (ym.y - yk.y));
                        const float2 yod2 = cmul(make_float2(0.5f * (ym.x - yk.x), 0.5f * (ym.y + yk.y)), cconj(wm));
                        bq[pad16(km)] = make_float2(yec2.x - yod2.y, yec2.y + yod2.x);
                    }
                }
            }
        }
        __syncthreads();
        reg_fft_rows<true, M, false, ROWS>(v, buf, W);
        }
        for (int q = 0; q < nq; q++) {
            const float2 *bq = buf + q * BS;
            float *o = out + (size_t)(pr0 + q) * out_ld;
            if (vec_out) {   // rows padded to whole float4: the 0..3 floats past n_out land in the padding
                for (int c = j; 4 * c < n_out; c += T) {
                    const float2 z0 = bq[pad16(2 * c)], z1 = bq[pad16(2 * c + 1)];
                    reinterpret_cast<float4 *>(o)[c] = make_float4(z0.x, z0.y, z1.x, z1.y);
                }
            } else {
                for (int i = j; i < n_out; i += T) {
                    const float2 z = bq[pad16(i >> 1)];
                    o[i] = (i & 1) ? z.y : z.x;
                }
            }
        }
        __syncthreads();
    }
}

int tuning(int knob);
constexpr int kTuneConvRowsKnob = 0;   // TuneKnob::kTuneConvRows (tuning.cu)
constexpr int kTuneTrajBlocksKnob = 3; // TuneKnob::kTuneTrajBlocksPerSm

template <int M, int ROWS>
static cudaError_t launch_reg_conv_rows(const float *rir, int P, int R, int L, int S, const float2 *W,
                                        const float2 *Sg, float *out, long out_ld, cudaStream_t st) {
    const size_t smem = (size_t)ROWS * (M + M / 16) * sizeof(float2);
    static int blocks = -1;
    if (blocks < 0) {
        cudaError_t e = cudaFuncSetAttribute(rir_conv_reg_kernel<M, ROWS>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        int per_sm = 0, dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rir_conv_reg_kernel<M, ROWS>, M / 16, smem);
        if (e != cudaSuccess) return e;
        blocks = std::max(1, per_sm) * std::max(1, sms);
    }
    const int grid = std::min((P * R + ROWS - 1) / ROWS, blocks);
    rir_conv_reg_kernel<M, ROWS><<<grid, M / 16, smem, st>>>(rir, P, R, L, S, W, Sg, out, out_ld);
    return cudaGetLastError();
}

// Rows per block from the tuning table (1: more blocks per SM; 2: twiddles and
// barriers shared by a pair of rows).  Each row's arithmetic is the same either way.
template <int M>
static cudaError_t launch_reg_conv(const float *rir, int P, int R, int L, int S, const float2 *W,
                                   const float2 *Sg, float *out, long out_ld, cudaStream_t st) {
    if (tuning(kTuneConvRowsKnob) == 1)
        return launch_reg_conv_rows<M, 1>(rir, P, R, L, S, W, Sg, out, out_ld, st);
    return launch_reg_conv_rows<M, kConvRows>(rir, P, R, L, S, W, Sg, out, out_ld, st);
}

// ---------------------------------------------------------------------------
// Adjoint of simulateTrajectory (no counterpart in the reference, which is not
// differentiable).  The forward pass is, per point p and receiver r,
//   y[w_ini[p] + j][r] += (x_p * h_pr)[j],  0 <= j < w_len[p] + L - 1,
// with x_p the segment of point p and h_pr its RIR.  Given g = dL/dy:
//   dL/dh_pr[k] = sum_t g_pr[t + k] x_p[t]             (correlation with the segment)
//   dL/dx_p[t]  = sum_r sum_k g_pr[t + k] h_pr[k]       (correlation with the RIRs)
// where g_pr[j] = g[w_ini[p] + j][r] on the window the forward pass wrote.  Both
// are computed as spectra: D = G conj(X) and sum_r G conj(H), with the real FFTs
// of the forward kernel (N = 2M >= S + L - 1, so no circular wrap on the kept
// lags).  One block per point walks its receivers: FFT of the gradient window and
// of the RIR, the product with the segment's spectrum inverted to dL/dh, the
// product with the RIR's spectrum added to the point's accumulator (bins owned by
// one thread each: no atomics), and at the end the accumulator inverted to dL/dx.
// ---------------------------------------------------------------------------

// g [n_out][R] float64 -> gt [R][n_out] float32 (rows the FFT kernels read contiguously)
__global__ void grad_transpose_kernel(const double *__restrict__ g, long n_out, int R, float *__restrict__ gt) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_out) return;
    for (int r = 0; r < R; r++) gt[(long)r * n_out + t] = (float)g[t * R + r];
}

// Real-spectrum bins k and M - k of the packed FFT z (natural order in buf).
__device__ __forceinline__ void real_bins(const float2 *buf, int k, int M, float2 wk, float2 &xk, float2 &xm) {
    const int km = (M - k) & (M - 1);
    const float2 zk = buf[pad16(k)], zm = buf[pad16(km)];
    const float2 ze = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
    const float2 zo = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
    const float2 ze2 = make_float2(ze.x, -ze.y), zo2 = make_float2(zo.x, -zo.y);
    const float2 wm = make_float2(-wk.x, wk.y);
    xk = cadd(ze, cmul(wk, zo));
    xm = cadd(ze2, cmul(wm, zo2));
}

// Packs the real spectrum (bins k, M - k) into buf for the inverse packed FFT.
__device__ __forceinline__ void pack_inverse(float2 *buf, int k, int M, float2 wk, float2 yk, float2 ym) {
    const int km = (M - k) & (M - 1);
    const float2 wm = make_float2(-wk.x, wk.y);
    const float2 yec = make_float2(0.5f * (yk.x + ym.x), 0.5f * (yk.y - ym.y));
    const float2 yod = cmul(make_float2(0.5f * (yk.x - ym.x), 0.5f * (yk.y + ym.y)), cconj(wk));
    buf[pad16(k)] = make_float2(yec.x - yod.y, yec.y + yod.x);
    if (k != 0 && km != k) {
        const float2 yec2 = make_float2(0.5f * (ym.x + yk.x), 0.5f * (ym.y - yk.y));
        const float2 yod2 = cmul(make_float2(0.5f * (ym.x - yk.x), 0.5f * (ym.y + yk.y)), cconj(wm));
        buf[pad16(km)] = make_float2(yec2.x - yod2.y, yec2.y + yod2.x);
    }
}

// Stores the first n values of the inverse packed FFT in buf (z[n] = y[2n] + i y[2n+1]).
template <int M>
__device__ __forceinline__ void store_real(const float2 *buf, float *__restrict__ o, int n) {
    constexpr int T = M / 16;
    if ((reinterpret_cast<uintptr_t>(o) & 7) == 0) {
        for (int c = threadIdx.x; 2 * c < n; c += T) {
            const float2 z = buf[pad16(c)];
            if (2 * c + 1 < n) reinterpret_cast<float2 *>(o)[c] = z;
            else o[2 * c] = z.x;
        }
    } else {
        for (int i = threadIdx.x; i < n; i += T) {
            const float2 z = buf[pad16(i >> 1)];
            o[i] = (i & 1) ? z.y : z.x;
        }
    }
}

template <int M>
__global__ void __launch_bounds__(M / 16) traj_adjoint_kernel(
        const float *__restrict__ gt, long n_out, const int *__restrict__ w_ini, const int *__restrict__ w_len,
        const float *__restrict__ rir, int P, int R, int L, const float2 *__restrict__ W,
        const float2 *__restrict__ Sg, float *__restrict__ grad_rir, float *__restrict__ grad_sig,
        float2 *__restrict__ acc_all) {
    constexpr int T = M / 16, BS = M + M / 16;
    extern __shared__ __align__(16) float2 sm[];
    float2 *bg = sm, *bh = sm + BS;   // gradient window, RIR
    const int j = threadIdx.x;
    float2 *acc = acc_all + (size_t)blockIdx.x * (M + 1);
    const float inv_m = 1.0f / (float)M;
    float2 v[16];
    for (int p = blockIdx.x; p < P; p += gridDim.x) {
        const int w0 = w_ini[p], wl = w_len[p];
        const int glen = wl + L - 1;   // gradient entries the forward pass wrote for this point
        const float2 *xs = Sg + (size_t)p * (M + 1);   // segment spectrum / M
        for (int r = 0; r < R; r++) {
            load_packed<M>(gt + (size_t)r * n_out + w0, glen, v);
            reg_fft<false, M, true>(v, bg, W);
            if (grad_sig) {
                load_packed<M>(rir + ((size_t)p * R + r) * L, L, v);
                reg_fft<false, M, true>(v, bh, W);
            }
            for (int k = j; k <= M / 2; k += T) {
                const float2 wk = __ldg(&W[k]);
                float2 gk, gm;
                real_bins(bg, k, M, wk, gk, gm);
                if (grad_sig) {
                    float2 hk, hm;
                    real_bins(bh, k, M, wk, hk, hm);
                    float2 ak = cmul(gk, cconj(hk)), am = cmul(gm, cconj(hm));
                    if (r > 0) {
                        ak = cadd(ak, acc[k]);
                        am = cadd(am, acc[M - k]);
                    }
                    acc[k] = ak;
                    if (M - k != k) acc[M - k] = am;
                }
                if (grad_rir) {
                    const float2 dk = cmul(gk, cconj(__ldg(&xs[k])));
                    const float2 dm = cmul(gm, cconj(__ldg(&xs[M - k])));
                    pack_inverse(bg, k, M, wk, dk, dm);   // (k, M - k) of this thread only
                }
            }
            __syncthreads();
            if (grad_rir) {
                reg_fft<true, M, false>(v, bg, W);
                store_real<M>(bg, grad_rir + ((size_t)p * R + r) * L, L);
                __syncthreads();
            }
        }
        if (grad_sig) {
            for (int k = j; k <= M / 2; k += T) {   // the bins this thread accumulated
                const float2 wk = __ldg(&W[k]);
                const float2 ak = acc[k], am = acc[M - k];
                pack_inverse(bg, k, M, wk, make_float2(ak.x * inv_m, ak.y * inv_m),
                             make_float2(am.x * inv_m, am.y * inv_m));
            }
            __syncthreads();
            reg_fft<true, M, false>(v, bg, W);
            store_real<M>(bg, grad_sig + w0, wl);
            __syncthreads();
        }
    }
}

template <int M>
static cudaError_t launch_traj_adjoint(const float *gt, long n_out, const int *w_ini, const int *w_len,
                                       const float *rir, int P, int R, int L, const float2 *W,
                                       const float2 *Sg, float *grad_rir, float *grad_sig, float2 *acc,
                                       int grid, cudaStream_t st) {
    const size_t smem = (size_t)2 * (M + M / 16) * sizeof(float2);
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(traj_adjoint_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    traj_adjoint_kernel<M><<<grid, M / 16, smem, st>>>(gt, n_out, w_ini, w_len, rir, P, R, L, W, Sg, grad_rir,
                                                       grad_sig, acc);
    return cudaGetLastError();
}

// Blocks of the adjoint kernel for FFT half-size M (one per SM at most: the kernel
// holds two padded rows of shared memory).
int traj_adjoint_grid(int M, int P, int num_sms) {
    const int t = tuning(kTuneTrajBlocksKnob);
    const int per_sm = t > 0 ? t : (M <= 4096 ? 2 : 1);
    return std::max(1, std::min(P, num_sms * per_sm));
}

cudaError_t traj_adjoint_launch(const double *g, long n_out, const int *w_ini, const int *w_len, const float *rir,
                                int P, int R, int L, int M, const float2 *W, const float2 *Sg, float *gt,
                                float *grad_rir, float *grad_sig, float2 *acc, int grid, cudaStream_t st) {
    if (n_out <= 0 || P <= 0 || R <= 0) return cudaSuccess;
    grad_transpose_kernel<<<(unsigned)((n_out + 255) / 256), 256, 0, st>>>(g, n_out, R, gt);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    switch (M) {
    case 1024: return launch_traj_adjoint<1024>(gt, n_out, w_ini, w_len, rir, P, R, L, W, Sg, grad_rir, grad_sig, acc, grid, st);
    case 2048: return launch_traj_adjoint<2048>(gt, n_out, w_ini, w_len, rir, P, R, L, W, Sg, grad_rir, grad_sig, acc, grid, st);
    case 4096: return launch_traj_adjoint<4096>(gt, n_out, w_ini, w_len, rir, P, R, L, W, Sg, grad_rir, grad_sig, acc, grid, st);
    case 8192: return launch_traj_adjoint<8192>(gt, n_out, w_ini, w_len, rir, P, R, L, W, Sg, grad_rir, grad_sig, acc, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

// Overlap-add (gpuRIR/__init__.py:216-219): out[t][r] = sum over points p, in
// increasing p, of conv[p][r][t - w_ini[p]] for 0 <= t - w_ini[p] < w_len[p] + L - 1.
// Compensated FP32 sum (two-sum), written as float64.
__global__ void ola_kernel(const float *conv, long conv_ld, const int *w_ini, const int *w_len, int P,
                           int R, int L, long n_out, int uni_w, double *out) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;   // consecutive t: coalesced reads
    const int r = blockIdx.y;
    if (t >= n_out) return;
    // points whose filtered segment covers t: lo = first p with w_ini[p] + w_len[p] + L - 1 > t,
    // e = first p with w_ini[p] > t (w_ini increasing, w_ini[p] + w_len[p] = w_ini[p + 1])
    int lo, e;
    if (uni_w > 0) {   // w_ini[p] = p W, w_len[p] = W: both bounds by division
        const long a = t - (uni_w + L - 1);   // p W + W + L - 1 > t  <=>  p > a / W
        lo = a < 0 ? 0 : (int)min((long)P, a / uni_w + 1);
        e = (int)min((long)P, t / uni_w + 1);
    } else {
        lo = 0;
        int hi = P;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if ((long)w_ini[mid] + w_len[mid] + L - 1 > t) hi = mid; else lo = mid + 1;
        }
        e = lo;
        int e_hi = P;
        while (e < e_hi) {
            const int mid = (e + e_hi) >> 1;
            if ((long)w_ini[mid] > t) e_hi = mid; else e = mid + 1;
        }
    }
    // every p in [lo, e) contributes conv[p][r][t - w_ini[p]]: independent loads, then the
    // compensated sum in increasing p
    float s = 0.0f, comp = 0.0f;
    const float *col = conv + (long)r * conv_ld + t;
    const long pstride = (long)R * conv_ld;
#pragma unroll 4
    for (int p = lo; p < e; p++) {
        const float v = __ldg(col + p * pstride - w_ini[p]);
        const float y = s + v;                       // two-sum
        const float bb = y - s;
        comp += (s - (y - bb)) + (v - bb);
        s = y;
    }
    out[t * R + r] = (double)s + (double)comp;
}

// data (2 M) + M-point twiddles (3M/4) + N-point twiddles (M/2 + 1)
size_t fft_smem_bytes(int M) {
    return M <= kSmemFftMax ? (2 * (size_t)M + 3 * (size_t)M / 4 + (size_t)M / 2 + 1) * sizeof(float2) : 0;
}
size_t fft_scratch_floats2(int M, int grid) { return M <= kSmemFftMax ? 0 : (size_t)grid * 2 * M; }

cudaError_t twiddle_launch(float2 *w, int n, cudaStream_t st) {
    twiddle_kernel<<<(n + 255) / 256, 256, 0, st>>>(w, n);
    return cudaGetLastError();
}

static cudaError_t set_fft_smem() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(segment_spectra_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)fft_smem_bytes(kSmemFftMax));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(rir_conv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)fft_smem_bytes(kSmemFftMax));
    done = e == cudaSuccess;
    return e;
}

template <int M>
static cudaError_t launch_reg_spectra(const float *seg, int P, int S, const float2 *W, float2 *Sg,
                                     cudaStream_t st) {
    const size_t smem = (size_t)(M + M / 16) * sizeof(float2);
    static int blocks = -1;
    if (blocks < 0) {
        cudaError_t e = cudaFuncSetAttribute(segment_spectra_reg_kernel<M>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        int per_sm = 0, dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, segment_spectra_reg_kernel<M>, M / 16, smem);
        if (e != cudaSuccess) return e;
        blocks = std::max(1, per_sm) * std::max(1, sms);
    }
    segment_spectra_reg_kernel<M><<<std::min(P, blocks), M / 16, smem, st>>>(seg, P, S, W, Sg);
    return cudaGetLastError();
}

cudaError_t segment_spectra_launch(const float *seg, int P, int S, int M, const float2 *W, float2 *Sg,
                                   float2 *scratch, int grid, cudaStream_t st) {
    switch (M) {   // register-resident kernel for the common sizes
    case 1024: return launch_reg_spectra<1024>(seg, P, S, W, Sg, st);
    case 2048: return launch_reg_spectra<2048>(seg, P, S, W, Sg, st);
    case 4096: return launch_reg_spectra<4096>(seg, P, S, W, Sg, st);
    case 8192: return launch_reg_spectra<8192>(seg, P, S, W, Sg, st);
    default: break;
    }
    cudaError_t e = set_fft_smem();
    if (e != cudaSuccess) return e;
    segment_spectra_kernel<<<grid, kFftThreads, fft_smem_bytes(M), st>>>(seg, P, S, M, W, Sg, scratch);
    return cudaGetLastError();
}

cudaError_t rir_conv_launch(const float *rir, int P, int R, int L, int S, int M, const float2 *W,
                            const float2 *Sg, float *out, long out_ld, float2 *scratch, int grid,
                            cudaStream_t st) {
    switch (M) {   // register-resident kernel for the common sizes
    case 1024: return launch_reg_conv<1024>(rir, P, R, L, S, W, Sg, out, out_ld, st);
    case 2048: return launch_reg_conv<2048>(rir, P, R, L, S, W, Sg, out, out_ld, st);
    case 4096: return launch_reg_conv<4096>(rir, P, R, L, S, W, Sg, out, out_ld, st);
    case 8192: return launch_reg_conv<8192>(rir, P, R, L, S, W, Sg, out, out_ld, st);
    default: break;
    }
    cudaError_t e = set_fft_smem();
    if (e != cudaSuccess) return e;
    rir_conv_kernel<<<grid, kFftThreads, fft_smem_bytes(M), st>>>(rir, P, R, L, S, M, W, Sg, out, out_ld,
                                                                 scratch);
    return cudaGetLastError();
}

cudaError_t ola_launch(const float *conv, long conv_ld, const int *w_ini, const int *w_len, int P, int R,
                       int L, long n_out, int uni_w, double *out, cudaStream_t st) {
    if (n_out <= 0 || R <= 0) return cudaSuccess;
    if (R > 65535) return cudaErrorInvalidValue;
    dim3 grid((unsigned)((n_out + 255) / 256), (unsigned)R);
    ola_kernel<<<grid, 256, 0, st>>>(conv, conv_ld, w_ini, w_len, P, R, L, n_out, uni_w, out);
    return cudaGetLastError();
}

}  // namespace gpurir
