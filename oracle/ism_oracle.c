/*
 * ism_oracle.c -- CPU restatement of gpuRIR's image-source-method (ISM) pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA path
 * in gpurir_gb300/csrc.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it.  The product never links it or falls back to it.
 *
 * Parity status of this restatement:
 *   - The host-side helpers and the trajectory overlap-add it is used with are
 *     pinned against golden vectors produced by importing the reference's own
 *     Python package (tests/golden/make_golden.py).
 *   - The ISM arithmetic is pinned against the reference's own CUDA kernels:
 *     src/gpuRIR_cuda.cu compiled from the reference sources (oracle/ref_kernels.py)
 *     and run on a GB300 produced tests/golden/reference_kernels.npz.  Fed the
 *     reference's image amplitudes and delays, orc_ism_sum, orc_ism_sum_lut,
 *     orc_env_pred and orc_diffuse_from_uniforms reproduce those kernels to
 *     float32 rounding (tests/test_reference_kernels.py).
 *
 * Every function names the reference lines (path:line inside the gpuRIR
 * project) that it restates.  Arithmetic is FP64 unless the name says f32.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846

/* Polar patterns, src/gpuRIR_cuda.h:2-8. */
enum { P_OMNI = 0, P_HOMNI = 1, P_CARD = 2, P_HYPCARD = 3, P_SUBCARD = 4, P_BIDIR = 5 };

/* ---------------------------------------------------------------------------
 * Lengths.  src/gpuRIR_cuda.cu:831-835 and src/python_bind.cpp:82-83 compute
 * ceil(T*Fs) from float32 operands, then round up to an even count.
 * ------------------------------------------------------------------------- */
int orc_n_samples(float T, float Fs)
{
    float p = T * Fs;               /* float32 product, as in the reference */
    int n = (int)ceilf(p);
    n += n % 2;
    return n;
}

/* Window length in samples: (int)round(8e-3f*Fs), src/gpuRIR_cuda.cu:629. */
int orc_window_len(float Fs)
{
    float p = 8e-3f * Fs;
    return (int)roundf(p);
}

/* src/gpuRIR_cuda.cu:132-147 (directivity), evaluated in FP64. */
static double orc_directivity(const double doa[3], const double orv[3], int pattern)
{
    if (pattern == P_OMNI) return 1.0;
    double c = doa[0] * orv[0] + doa[1] * orv[1] + doa[2] * orv[2];
    c /= sqrt(doa[0] * doa[0] + doa[1] * doa[1] + doa[2] * doa[2]);
    c /= sqrt(orv[0] * orv[0] + orv[1] * orv[1] + orv[2] * orv[2]);
    switch (pattern) {
    case P_HOMNI:   return c > 0.0 ? 1.0 : 0.0;
    case P_CARD:    return 0.5 + 0.5 * c;
    case P_HYPCARD: return 0.25 + 0.75 * c;
    case P_SUBCARD: return 0.75 + 0.25 * c;
    case P_BIDIR:   return c;
    default:        return 0.0;
    }
}

/* Per-axis image bookkeeping of src/gpuRIR_cuda.cu:336-342:
 *   k = n - N/2, clust = ceil(k/2), r = |k mod 2| (C remainder). */
static void orc_axis(int n, int N, int *clust, int *refl)
{
    int k = n - N / 2;
    *clust = (int)ceil(k / 2.0);
    *refl = abs(k % 2);
}

/*
 * Amplitude and delay (in samples) of every image for every (src, rcv) pair.
 * Restates calcAmpTau_kernel, src/gpuRIR_cuda.cu:245-375.
 *   amp, tau : [M_src][M_rcv][N0*N1*N2], image index n0*N1*N2 + n1*N2 + n2
 *   tau_dp   : [M_src][M_rcv], delay of the direct path (all clust = refl = 0)
 */
void orc_amp_tau(const float room[3], const float beta[6],
                 const float *pos_src, int M_src, const float *pos_rcv, int M_rcv,
                 const float *orv_src, const float *orv_rcv, int spkr_pattern, int mic_pattern,
                 const int nb_img[3], float c, float Fs,
                 double *amp, double *tau, double *tau_dp)
{
    const int N0 = nb_img[0], N1 = nb_img[1], N2 = nb_img[2];
    const long NN = (long)N0 * N1 * N2;
    for (int n0 = 0; n0 < N0; n0++)
    for (int n1 = 0; n1 < N1; n1++)
    for (int n2 = 0; n2 < N2; n2++) {
        int n[3] = {n0, n1, n2}, N[3] = {N0, N1, N2};
        int clust[3], refl[3];
        double att = 1.0;
        int direct = 1;
        for (int d = 0; d < 3; d++) {
            orc_axis(n[d], N[d], &clust[d], &refl[d]);
            /* beta is negated before the powers, src/gpuRIR_cuda.cu:272-277, 340 */
            att *= pow(-(double)beta[2 * d], abs(clust[d] - refl[d])) *
                   pow(-(double)beta[2 * d + 1], abs(clust[d]));
            direct = direct && clust[d] == 0 && refl[d] == 0;
        }
        long idx = (long)n0 * N1 * N2 + (long)n1 * N2 + n2;
        for (int ms = 0; ms < M_src; ms++)
        for (int mr = 0; mr < M_rcv; mr++) {
            double vec[3], im2rcv[3], osrc[3], dist2 = 0.0;
            for (int d = 0; d < 3; d++) {
                double s = (1 - 2 * refl[d]);
                /* vector from the receiver to the image, src/gpuRIR_cuda.cu:353 */
                vec[d] = clust[d] * 2.0 * (double)room[d] + s * (double)pos_src[ms * 3 + d]
                         - (double)pos_rcv[mr * 3 + d];
                dist2 += vec[d] * vec[d];
                osrc[d] = s * (double)orv_src[ms * 3 + d];   /* mirrored source axis, :357 */
                im2rcv[d] = -vec[d];
            }
            double dist = sqrt(dist2);
            double a = att / (4.0 * ORC_PI * dist);
            if (spkr_pattern != P_OMNI) a *= orc_directivity(im2rcv, osrc, spkr_pattern);
            if (mic_pattern != P_OMNI) {
                double orc[3] = {orv_rcv[mr * 3], orv_rcv[mr * 3 + 1], orv_rcv[mr * 3 + 2]};
                a *= orc_directivity(vec, orc, mic_pattern);
            }
            long o = ((long)ms * M_rcv + mr) * NN + idx;
            amp[o] = a;
            tau[o] = dist / (double)c * (double)Fs;
            if (direct) tau_dp[ms * M_rcv + mr] = tau[o];
        }
    }
}

/*
 * Image delays as the reference build rounds them in float32 (the engine's
 * reference-delay mode).  calcAmpTau_kernel, src/gpuRIR_cuda.cu:336-369:
 * cluster offset (2 clust) * L, plus or minus the source coordinate, minus the
 * receiver coordinate, each rounded; the squared distance as the compiled
 * kernel contracts `dist += vec[d]*vec[d]` (one FMA per axis when both patterns
 * are omni; x^2 + y^2 rounded separately, then an FMA for z, otherwise; matched
 * bit for bit against the delays the reference kernel wrote,
 * tests/golden/reference_kernels.npz); then sqrtf and dist / c * Fs.
 * Compiled without contraction so that only the fmaf calls fuse.
 *   tau    : [M_src][M_rcv][N0*N1*N2] float32
 *   tau_dp : [M_src][M_rcv] float32
 */
__attribute__((optimize("fp-contract=off")))
void orc_tau_ref_f32(const float room[3], const float *pos_src, int M_src, const float *pos_rcv,
                     int M_rcv, int spkr_pattern, int mic_pattern, const int nb_img[3], float c,
                     float Fs, float *tau, float *tau_dp)
{
    const int N0 = nb_img[0], N1 = nb_img[1], N2 = nb_img[2];
    const long NN = (long)N0 * N1 * N2;
    const int directional = spkr_pattern != P_OMNI || mic_pattern != P_OMNI;
    for (int ms = 0; ms < M_src; ms++)
    for (int mr = 0; mr < M_rcv; mr++)
    for (int n0 = 0; n0 < N0; n0++)
    for (int n1 = 0; n1 < N1; n1++)
    for (int n2 = 0; n2 < N2; n2++) {
        int n[3] = {n0, n1, n2}, N[3] = {N0, N1, N2};
        float v[3];
        int direct = 1;
        for (int d = 0; d < 3; d++) {
            int cl, rf;
            orc_axis(n[d], N[d], &cl, &rf);
            volatile float cp = (float)(2 * cl) * room[d];
            volatile float a = cp + (rf ? -pos_src[ms * 3 + d] : pos_src[ms * 3 + d]);
            v[d] = a - pos_rcv[mr * 3 + d];
            direct = direct && cl == 0 && rf == 0;
        }
        float d2;
        if (directional) {
            volatile float xx = v[0] * v[0], yy = v[1] * v[1];
            volatile float s = xx + yy;
            d2 = fmaf(v[2], v[2], s);
        } else {
            volatile float xx = v[0] * v[0];
            d2 = fmaf(v[2], v[2], fmaf(v[1], v[1], xx));
        }
        volatile float dist = sqrtf(d2);
        volatile float q = dist / c;
        float t = q * Fs;
        long o = ((long)ms * M_rcv + mr) * NN + (long)n0 * N1 * N2 + (long)n1 * N2 + n2;
        tau[o] = t;
        if (direct) tau_dp[ms * M_rcv + mr] = t;
    }
}

/*
 * Windowed-sinc accumulation of the early part.  Restates image_sample,
 * hanning_window and sinc (src/gpuRIR_cuda.cu:110-121) summed over images as
 * generateRIR_kernel/reduceRIR_kernel do (:377-413).  Terms outside
 * |t - tau| < Tw/2 are exactly zero in the reference, so visiting only the
 * window gives the same sum.
 *   rir : [M][ld] doubles, columns [0, nISM) written (zeroed first)
 */
void orc_ism_sum(const double *amp, const double *tau, long M, long N, int nISM, float Fs,
                 double *rir, long ld)
{
    const double Tw = (double)orc_window_len(Fs);
    const double H = Tw / 2.0;
    /* RIRs in parallel; each RIR's sum runs in image order on one thread */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (long m = 0; m < M; m++) {
        double *h = rir + m * ld;
        for (int t = 0; t < nISM; t++) h[t] = 0.0;
        for (long i = 0; i < N; i++) {
            double a = amp[m * N + i], ta = tau[m * N + i];
            long t0 = (long)floor(ta - H);
            if (t0 < 0) t0 = 0;
            for (long t = t0; t < nISM && (double)t < ta + H; t++) {
                double x = (double)t - ta;
                if (fabs(x) >= H) continue;
                double w = 0.5 * (1.0 + cos(2.0 * ORC_PI * x / Tw));
                double s = (x == 0.0) ? 1.0 : sin(ORC_PI * x) / (ORC_PI * x);
                h[t] += w * a * s;
            }
        }
    }
}

int orc_lut_len(float Fs) { return orc_window_len(Fs) * 16 + 1; }

/* The Hann x sinc table of create_sinc_texture_lut (src/gpuRIR_cuda.cu:578-592),
 * float arithmetic, symmetric about lut_len/2: T[lut_len/2 +- i] at x = i/16. */
void orc_lut_table(float Fs, float *T)
{
    const int Tw = orc_window_len(Fs);
    const int lut_len = orc_lut_len(Fs), center = lut_len / 2;
    const float PIf = 3.141592654f;
    for (int i = 0; i <= center; i++) {
        float x = (float)i / 16;
        float sc = (x == 0.0f) ? 1.0f : sinf(PIf * x) / (PIf * x);
        float hn = 0.5f * (1.0f + cosf(2.0f * PIf * x / Tw));
        T[center + i] = hn * sc;
        T[center - i] = hn * sc;
    }
}

/* fmaf(a, b, c) rounded toward zero (the __fmaf_rz of image_sample_lut) for a
 * result > 0: the exact value is s + e (TwoSum of a*b, exact in double, and c),
 * and the nearest float is stepped down when it lies above it. */
static float orc_fmaf_rz_pos(float a, float b, float c)
{
    const double p = (double)a * (double)b, q = (double)c;
    const double s = p + q;
    const double bb = s - p;
    const double e = (p - (s - bb)) + (q - bb);
    float f = (float)s;
    if ((double)f - s > e) f = nextafterf(f, 0.0f);
    return f;
}

/*
 * Lookup-table variant of the early part, restating gpuRIR's LUT path in its
 * float arithmetic: the table of create_sinc_texture_lut (src/gpuRIR_cuda.cu:
 * 578-592: Hann x sinc at 16 samples per sample, lut_len = 16 Tw + 1), the fetch
 * of image_sample_lut (:236-239): t_tau = t - tau in float, support
 * |t_tau| < Tw/2 (integer division), coordinate __fmaf_rz(t_tau, 16,
 * lut_len/2 + 0.5), and the linear filter of a float texture: texel position
 * x - 0.5, weight of the upper texel held on 8 fractional bits, rounded half up
 * (measured on GB300 texture units), border texels 0.  tau is taken as the
 * nearest float, as the reference stores it.
 */
void orc_ism_sum_lut(const double *amp, const double *tau, long M, long N, int nISM, float Fs,
                     double *rir, long ld)
{
    const int Tw = orc_window_len(Fs);
    const int lut_len = orc_lut_len(Fs), center = lut_len / 2, H = Tw / 2;
    const float cfetch = (float)center + 0.5f;
    float *T = (float *)malloc(sizeof(float) * (size_t)(lut_len + 1));
    orc_lut_table(Fs, T);
    T[lut_len] = 0.0f;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (long m = 0; m < M; m++) {
        double *h = rir + m * ld;
        for (int t = 0; t < nISM; t++) h[t] = 0.0;
        for (long i = 0; i < N; i++) {
            const double a = amp[m * N + i];
            const float tf = (float)tau[m * N + i];
            long t0 = (long)floor((double)tf - H) - 1;
            if (t0 < 0) t0 = 0;
            for (long t = t0; t < nISM && (double)t < (double)tf + H + 1; t++) {
                const float x = (float)t - tf;
                if (fabsf(x) >= (float)H) continue;
                const float xb = orc_fmaf_rz_pos(x, 16.0f, cfetch) - 0.5f;
                const float jf = floorf(xb);
                long j = (long)jf;
                double al = floor((double)(xb - jf) * 256.0 + 0.5) / 256.0;
                if (al >= 1.0) { j += 1; al = 0.0; }
                double t0v = (j >= 0 && j < lut_len) ? T[j] : 0.0;
                double t1v = (j + 1 >= 0 && j + 1 < lut_len) ? T[j + 1] : 0.0;
                h[t] += a * (t0v + al * (t1v - t0v));
            }
        }
    }
    free(T);
}

/* Sabine reverberation time from the walls, src/gpuRIR_cuda.cu:123-130. */
double orc_sabine_t60(const float room[3], const float beta[6])
{
    double b[6];
    for (int i = 0; i < 6; i++) b[i] = beta[i];
    double Sa = ((1 - b[0] * b[0]) + (1 - b[1] * b[1])) * room[1] * room[2] +
                ((1 - b[2] * b[2]) + (1 - b[3] * b[3])) * room[0] * room[2] +
                ((1 - b[4] * b[4]) + (1 - b[5] * b[5])) * room[0] * room[1];
    double V = (double)room[0] * room[1] * room[2];
    return 0.161 * V / Sa;
}

/*
 * Diffuse-tail envelope, restating envPred_kernel (src/gpuRIR_cuda.cu:415-443):
 * mean power of the last <=10 ms of the early part after the direct path, an
 * exponential decay alpha from the Sabine T60, and the gain A that makes
 * A*exp(alpha*(t - tau_dp)) pass through that power at the window centre.
 * When the window is empty (tau_dp >= nISM) the reference divides by <= 0;
 * here A is set to 0 (no tail), the documented deviation of this engine.
 */
void orc_env_pred(const double *rir, long ld, const double *tau_dp, long M, int nISM, float Fs,
                  const float room[3], const float beta[6], double *A, double *alpha)
{
    double w_sz = (double)(10e-3f * Fs);
    double T60 = orc_sabine_t60(room, beta);
    double al = -13.8155 / (T60 * (double)Fs);
    for (long m = 0; m < M; m++) {
        double lo = (double)nISM - w_sz;
        if (tau_dp[m] > lo) lo = tau_dp[m];
        long ws = (long)ceil(lo);
        alpha[m] = al;
        if (ws >= nISM) { A[m] = 0.0; continue; }
        double wc = ws + (nISM - ws) / 2.0;
        double p = 0.0;
        for (long t = ws; t < nISM; t++) p += rir[m * ld + t] * rir[m * ld + t];
        p /= (double)(nISM - ws);
        A[m] = p / exp(al * (wc - tau_dp[m]));
    }
}

/* ---------------------------------------------------------------------------
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11).  Host replay of the counter-based stream that the tail
 * kernel uses in place of the reference's stateful cuRAND generator
 * (src/gpuRIR_cuda.cu:874, 1046-1047).
 * ------------------------------------------------------------------------- */
void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Raw stream of the tail for one RIR: words [0, n) of the blocks
 * ctr = (j, rir_index, offset_lo, offset_hi), key = (seed_lo, seed_hi). */
void orc_tail_stream(uint64_t seed, uint64_t offset, uint32_t rir_index, long n, uint32_t *out)
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (long j = 0; 4 * j < n; j++) {
        uint32_t ctr[4] = {(uint32_t)j, rir_index, (uint32_t)offset, (uint32_t)(offset >> 32)};
        uint32_t r[4];
        orc_philox4x32_10(ctr, key, r);
        for (int q = 0; q < 4 && 4 * j + q < n; q++) out[4 * j + q] = r[q];
    }
}

/* Uniform in (0, 1) from the top 23 bits of one word: (m + 0.5) * 2^-23, a
 * value that float32 represents exactly. */
static double orc_u01(uint32_t x) { return ((double)(x >> 9) + 0.5) * (1.0 / 8388608.0); }

/* Tail sample s: noise z shaped by sqrt(A*exp(alpha*(nISM + s - tau_dp))) (:457-459). */
static double orc_tail_sample(double A, double alpha, double tau_dp, int nISM, int s, double z)
{
    return sqrt(A * exp(alpha * ((double)nISM + s - tau_dp))) * z;
}

/*
 * Diffuse tail, restating diffRev_kernel (src/gpuRIR_cuda.cu:445-461): unit
 * variance noise shaped by sqrt(A*exp(alpha*(nISM + s - tau_dp))).
 * noise_kind 0: the reference's logistic transform 0.551329*log(u/(1-u+1e-6)).
 * noise_kind 1: Gaussian by Box-Muller on the word pairs (2j, 2j+1).
 *   out : [M][ld], columns [nISM, nISM + nDiff) written.
 */
void orc_tail(const double *A, const double *alpha, const double *tau_dp, long M, int nISM, int nDiff,
              uint64_t seed, uint64_t offset, const uint32_t *rir_index, int noise_kind,
              double *out, long ld)
{
    long nw = ((long)nDiff + 3) / 4 * 4;    /* whole Philox blocks */
    uint32_t *w = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(nw + 4));
    for (long m = 0; m < M; m++) {
        orc_tail_stream(seed, offset, rir_index ? rir_index[m] : (uint32_t)m, nw, w);
        for (int s = 0; s < nDiff; s++) {
            double z;
            if (noise_kind == 0) {
                double u = orc_u01(w[s]);
                z = 0.551329 * log(u / (1.0 - u + 1e-6));
            } else {
                int s0 = s & ~1;
                double u1 = orc_u01(w[s0]), u2 = orc_u01(w[s0 + 1]);
                double r = sqrt(-2.0 * log(u1));
                z = (s & 1) ? r * sin(2.0 * ORC_PI * u2) : r * cos(2.0 * ORC_PI * u2);
            }
            out[m * ld + nISM + s] = orc_tail_sample(A[m], alpha[m], tau_dp[m], nISM, s, z);
        }
    }
    free(w);
}

/* diffRev_kernel (src/gpuRIR_cuda.cu:445-461) applied to given uniforms, as the
 * reference applies it to the uniforms cuRAND wrote: u [M][nDiff] -> out [M][nDiff]. */
void orc_diffuse_from_uniforms(const double *A, const double *alpha, const double *tau_dp, long M,
                               int nISM, int nDiff, const float *u, double *out)
{
    for (long m = 0; m < M; m++)
        for (int s = 0; s < nDiff; s++) {
            const double v = u[m * nDiff + s];
            const double z = 0.551329 * log(v / (1.0 - v + 1e-6));
            out[m * nDiff + s] = orc_tail_sample(A[m], alpha[m], tau_dp[m], nISM, s, z);
        }
}

/* ---------------------------------------------------------------------------
 * FP32 CPU port: the same windowed ISM in float32 with the reference's float
 * formulas (powf, sqrtf, cosf, sinf), threaded with OpenMP over RIRs.  This is
 * the timed CPU baseline; it is not an accuracy reference.
 * ------------------------------------------------------------------------- */
static float orc_directivity_f(const float doa[3], const float orv[3], int pattern)
{
    if (pattern == P_OMNI) return 1.0f;
    float c = doa[0] * orv[0] + doa[1] * orv[1] + doa[2] * orv[2];
    c /= sqrtf(doa[0] * doa[0] + doa[1] * doa[1] + doa[2] * doa[2]);
    c /= sqrtf(orv[0] * orv[0] + orv[1] * orv[1] + orv[2] * orv[2]);
    switch (pattern) {
    case P_HOMNI:   return c > 0.0f ? 1.0f : 0.0f;
    case P_CARD:    return 0.5f + 0.5f * c;
    case P_HYPCARD: return 0.25f + 0.75f * c;
    case P_SUBCARD: return 0.75f + 0.25f * c;
    case P_BIDIR:   return c;
    default:        return 0.0f;
    }
}

/* 1 when every axis index is the central one (the direct path, clust = refl = 0). */
static int cl_all_zero(const int n[3], const int N[3])
{
    return n[0] == N[0] / 2 && n[1] == N[1] / 2 && n[2] == N[2] / 2;
}

/* Envelope and diffuse tail of one RIR in float32, as envPred_kernel and
 * diffRev_kernel compute them per RIR and per sample (src/gpuRIR_cuda.cu:415-461):
 * mean power of the last <= 10 ms after the direct path, A and alpha from the
 * Sabine T60, then noise times sqrtf(A * expf(alpha * (nISM + s - tau_dp))).  The
 * noise comes from the Philox stream of this engine (the reference draws cuRAND
 * uniforms): logistic (noise_kind 0) or Gaussian. */
static void orc_tail_f32(float *h, int nISM, int nDiff, float tau_dp, float Fs, float T60,
                         uint64_t seed, uint64_t offset, uint32_t rir, int noise_kind)
{
    const float w_sz = 10e-3f * Fs;
    float lo = (float)nISM - w_sz;
    if (tau_dp > lo) lo = tau_dp;
    const int ws = (int)ceilf(lo);
    const float alpha = -13.8155f / (T60 * Fs);
    float A = 0.0f;
    if (ws < nISM) {
        const float wc = (float)ws + (float)(nISM - ws) / 2.0f;
        float p = 0.0f;
        for (int t = ws; t < nISM; t++) p += h[t] * h[t];
        p /= (float)(nISM - ws);
        A = p / expf(alpha * (wc - tau_dp));
    }
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int s0 = 0; s0 < nDiff; s0 += 4) {
        const uint32_t ctr[4] = {(uint32_t)(s0 >> 2), rir, (uint32_t)offset, (uint32_t)(offset >> 32)};
        uint32_t w[4];
        orc_philox4x32_10(ctr, key, w);
        float z[4];
        if (noise_kind == 0) {
            for (int q = 0; q < 4; q++) {
                const float u = ((float)(w[q] >> 9) + 0.5f) * 1.1920928955078125e-07f;
                z[q] = 0.551329f * logf(u / (1.0f - u + 1e-6f));
            }
        } else {
            for (int q = 0; q < 4; q += 2) {
                const float u1 = ((float)(w[q] >> 9) + 0.5f) * 1.1920928955078125e-07f;
                const float u2 = ((float)(w[q + 1] >> 9) + 0.5f) * 1.1920928955078125e-07f;
                const float r = sqrtf(-2.0f * logf(u1));
                z[q] = r * cosf(6.283185307f * u2);
                z[q + 1] = r * sinf(6.283185307f * u2);
            }
        }
        for (int q = 0; q < 4 && s0 + q < nDiff; q++) {
            const float env = A * expf(alpha * ((float)(nISM + s0 + q) - tau_dp));
            h[nISM + s0 + q] = sqrtf(env) * z[q];
        }
    }
}

/* rir : [M_src*M_rcv][ld] floats, columns [0, nTotal) written: the early part
 * [0, nISM) and, when nTotal > nISM, the envelope-shaped tail (the reference's
 * whole per-RIR work).  Returns the number of windowed image-sample updates. */
long long orc_rir_f32(const float room[3], const float beta[6],
                      const float *pos_src, int M_src, const float *pos_rcv, int M_rcv,
                      const float *orv_src, const float *orv_rcv, int spkr_pattern, int mic_pattern,
                      const int nb_img[3], float c, float Fs, int nISM, int nTotal, uint64_t seed,
                      uint64_t offset, int noise_kind, float *rir, long ld, int n_threads)
{
    const int N0 = nb_img[0], N1 = nb_img[1], N2 = nb_img[2];
    const float PIf = 3.141592654f;
    const float Tw = (float)orc_window_len(Fs);
    const float H = Tw / 2.0f;
    const long M = (long)M_src * M_rcv;
    /* SabineT60 in float32 as the reference's device function evaluates it (:123-130) */
    const float Sa = ((1.0f - beta[0] * beta[0]) + (1.0f - beta[1] * beta[1])) * room[1] * room[2] +
                     ((1.0f - beta[2] * beta[2]) + (1.0f - beta[3] * beta[3])) * room[0] * room[2] +
                     ((1.0f - beta[4] * beta[4]) + (1.0f - beta[5] * beta[5])) * room[0] * room[1];
    const float T60f = 0.161f * (room[0] * room[1] * room[2]) / Sa;
    long long updates = 0;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : updates)
#endif
    for (long m = 0; m < M; m++) {
        int ms = (int)(m / M_rcv), mr = (int)(m % M_rcv);
        float *h = rir + m * ld;
        for (int t = 0; t < nISM; t++) h[t] = 0.0f;
        float tau_dp = 0.0f;
        for (int n0 = 0; n0 < N0; n0++)
        for (int n1 = 0; n1 < N1; n1++)
        for (int n2 = 0; n2 < N2; n2++) {
            int n[3] = {n0, n1, n2}, N[3] = {N0, N1, N2};
            float att = 1.0f, vec[3], im2rcv[3], osrc[3], dist2 = 0.0f;
            for (int d = 0; d < 3; d++) {
                int cl, rf;
                orc_axis(n[d], N[d], &cl, &rf);
                att *= powf(-beta[2 * d], (float)abs(cl - rf)) * powf(-beta[2 * d + 1], (float)abs(cl));
                vec[d] = cl * 2 * room[d] + (1 - 2 * rf) * pos_src[ms * 3 + d] - pos_rcv[mr * 3 + d];
                dist2 += vec[d] * vec[d];
                osrc[d] = (1 - 2 * rf) * orv_src[ms * 3 + d];
                im2rcv[d] = -vec[d];
            }
            float dist = sqrtf(dist2);
            float a = att / (4 * PIf * dist);
            if (spkr_pattern != P_OMNI) a *= orc_directivity_f(im2rcv, osrc, spkr_pattern);
            if (mic_pattern != P_OMNI) a *= orc_directivity_f(vec, &orv_rcv[mr * 3], mic_pattern);
            float ta = dist / c * Fs;
            if (cl_all_zero(n, N)) tau_dp = ta;
            long t0 = (long)floorf(ta - H);
            if (t0 < 0) t0 = 0;
            for (long t = t0; t < nISM && (float)t < ta + H; t++) {
                float x = (float)t - ta;
                if (fabsf(x) >= H) continue;
                float w = 0.5f * (1.0f + cosf(2.0f * PIf * x / Tw));
                float xs = x * PIf;
                float s = (xs == 0.0f) ? 1.0f : sinf(xs) / xs;
                h[t] += w * a * s;
                updates++;
            }
        }
        if (nTotal > nISM) orc_tail_f32(h, nISM, nTotal - nISM, tau_dp, Fs, T60f, seed, offset,
                                        (uint32_t)m, noise_kind);
    }
    return updates;
}

/* The early part only. */
long long orc_ism_f32(const float room[3], const float beta[6],
                      const float *pos_src, int M_src, const float *pos_rcv, int M_rcv,
                      const float *orv_src, const float *orv_rcv, int spkr_pattern, int mic_pattern,
                      const int nb_img[3], float c, float Fs, int nISM, float *rir, long ld,
                      int n_threads)
{
    return orc_rir_f32(room, beta, pos_src, M_src, pos_rcv, M_rcv, orv_src, orv_rcv, spkr_pattern,
                       mic_pattern, nb_img, c, Fs, nISM, nISM, 0, 0, 0, rir, ld, n_threads);
}
