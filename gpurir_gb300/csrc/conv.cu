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

// Overlap-add (gpuRIR/__init__.py:216-219): out[t][r] = sum over points p, in
// increasing p, of conv[p][r][t - w_ini[p]] for 0 <= t - w_ini[p] < w_len[p] + L - 1.
// Compensated FP32 sum (two-sum), written as float64.
__global__ void ola_kernel(const float *conv, long conv_ld, const int *w_ini, const int *w_len, int P,
                           int R, int L, long n_out, double *out) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;   // consecutive t: coalesced reads
    const int r = blockIdx.y;
    if (t >= n_out) return;
    // first point whose window may reach t: w_ini[p] + w_len[p] + L - 1 > t; points are sorted by w_ini
    int lo = 0, hi = P;   // smallest p with w_ini[p] + w_len[p] + L - 1 > t
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((long)w_ini[mid] + w_len[mid] + L - 1 > t) hi = mid; else lo = mid + 1;
    }
    float s = 0.0f, comp = 0.0f;
    for (int p = lo; p < P && w_ini[p] <= t; p++) {
        const long k = t - w_ini[p];
        if (k < (long)w_len[p] + L - 1) {
            const float v = conv[((long)p * R + r) * conv_ld + k];
            const float y = s + v;                       // two-sum
            const float bb = y - s;
            comp += (s - (y - bb)) + (v - bb);
            s = y;
        }
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

cudaError_t segment_spectra_launch(const float *seg, int P, int S, int M, const float2 *W, float2 *Sg,
                                   float2 *scratch, int grid, cudaStream_t st) {
    cudaError_t e = set_fft_smem();
    if (e != cudaSuccess) return e;
    segment_spectra_kernel<<<grid, kFftThreads, fft_smem_bytes(M), st>>>(seg, P, S, M, W, Sg, scratch);
    return cudaGetLastError();
}

cudaError_t rir_conv_launch(const float *rir, int P, int R, int L, int S, int M, const float2 *W,
                            const float2 *Sg, float *out, long out_ld, float2 *scratch, int grid,
                            cudaStream_t st) {
    cudaError_t e = set_fft_smem();
    if (e != cudaSuccess) return e;
    rir_conv_kernel<<<grid, kFftThreads, fft_smem_bytes(M), st>>>(rir, P, R, L, S, M, W, Sg, out, out_ld,
                                                                 scratch);
    return cudaGetLastError();
}

cudaError_t ola_launch(const float *conv, long conv_ld, const int *w_ini, const int *w_len, int P, int R,
                       int L, long n_out, double *out, cudaStream_t st) {
    if (n_out <= 0 || R <= 0) return cudaSuccess;
    if (R > 65535) return cudaErrorInvalidValue;
    dim3 grid((unsigned)((n_out + 255) / 256), (unsigned)R);
    ola_kernel<<<grid, 256, 0, st>>>(conv, conv_ld, w_ini, w_len, P, R, L, n_out, out);
    return cudaGetLastError();
}

}  // namespace gpurir
