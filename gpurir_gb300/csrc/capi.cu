// capi.cu -- C ABI and host orchestration of gpurir_gb300.
//
// The host half of gpuRIR (gpuRIR_cuda::cuda_simulateRIR, src/gpuRIR_cuda.cu:
// 766-931) allocates and frees every buffer per call, launches each stage on
// the legacy stream with a device-wide synchronisation after it, and exit()s
// on any error.  Here a handle keeps a grow-only device workspace and pinned
// staging memory, all launch descriptors go to the device in one copy, the
// two kernels run back to back on one stream, and errors come back as codes.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gpurir_internal.cuh"
#include "../../include/gpurir_gb300.h"

namespace gpurir {
size_t ism_forward_smem_bytes(int tpl, int em, int max_nsub);
int ism_forward_max_nsub(int tpl, int em, size_t smem_budget);
int ism_forward_pick_tpl(float H);
int ism_forward_blocks_per_sm(int tpl, size_t smem);
cudaError_t ism_forward_launch(int tpl, const RoomDesc *rooms, const IsmItem *items, int n_items,
                               const float *pos_src, const float *pos_rcv, const float *orv_src,
                               const float *orv_rcv, float *out, int *work_counter, int *status,
                               int em, int max_nsub, int clamp, int grid, cudaStream_t st);
cudaError_t tail_launch(const RoomDesc *rooms, const IsmItem *rirs, int n_rir, int max_n_diff,
                        const float *pos_src, const float *pos_rcv, float *out, uint64_t seed,
                        uint64_t offset, int noise_kind, float *env_out, cudaStream_t st);
cudaError_t philox_stream_launch(uint32_t *out, long n, uint64_t seed, uint64_t offset,
                                 uint32_t rir, cudaStream_t st);
cudaError_t probe_peaks(double *fp32_flops, double *mufu_ops, cudaStream_t st);
}  // namespace gpurir

using namespace gpurir;

static thread_local std::string g_err;

static int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(GPURIR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Per-ISM-launch smem budget: two blocks of 512 threads per SM.
static const size_t kSmemBudget = 113 * 1024;   // two blocks per SM (228 KB less 1 KB each)
static const size_t kSmemBudgetLarge = 220 * 1024;

struct gpurir_sim {
    int mp = 0, lut = 0;
    uint64_t seed = 1234, calls = 0;
    int noise = GPURIR_NOISE_LOGISTIC;
    int device = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    char *d_ws = nullptr;
    size_t d_ws_bytes = 0;
    char *h_stage = nullptr;
    size_t h_stage_bytes = 0;
    cudaEvent_t stage_done = nullptr;
    bool stage_pending = false;
    cudaEvent_t ws_busy = nullptr;   // recorded after the last use of d_ws
    bool ws_recorded = false;
    int *d_ctl = nullptr;      // [0] work counter, [1] status
    int *h_ctl = nullptr;      // pinned copy of the status word
    long last_n_rir = 0;
    size_t env_off = 0;        // offset of the envelope array in d_ws
    int profile = 0;           // record events around each kernel
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool ev_ism = false, ev_tail = false;
    uint64_t last_h2d = 0, last_d2h = 0;
};

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

extern "C" const char *gpurir_version(void) { return "gpurir_gb300 0.1.0 (sm_103a)"; }

extern "C" const char *gpurir_last_error(void) { return g_err.c_str(); }

extern "C" int gpurir_n_samples(float T, float Fs) {
    float p = T * Fs;
    int n = (int)ceilf(p);
    n += n % 2;
    return n;
}

extern "C" int gpurir_create(int mixed_precision, int lookup_table, uint64_t seed, gpurir_sim **out) {
    if (!out) return fail(GPURIR_ERR_INVALID, "gpurir_create: out is NULL");
    *out = nullptr;
    gpurir_sim *s = new gpurir_sim();
    s->seed = seed;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->stage_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ws_busy, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_ctl, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(s->d_ctl, 0, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_ctl, 4 * sizeof(int));
    if (e != cudaSuccess) {
        std::string msg = std::string("gpurir_create: ") + cudaGetErrorString(e);
        gpurir_destroy(s);
        return fail(GPURIR_ERR_CUDA, msg);
    }
    // Same flag logic as the reference constructor: mixed precision first, then LUT.
    gpurir_activate_mixed_precision(s, mixed_precision, nullptr);
    gpurir_activate_lut(s, lookup_table, nullptr);
    *out = s;
    return GPURIR_OK;
}

extern "C" int gpurir_destroy(gpurir_sim *s) {
    if (!s) return GPURIR_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->d_ws) cudaFree(s->d_ws);
    if (s->h_stage) cudaFreeHost(s->h_stage);
    if (s->d_ctl) cudaFree(s->d_ctl);
    if (s->h_ctl) cudaFreeHost(s->h_ctl);
    if (s->stage_done) cudaEventDestroy(s->stage_done);
    if (s->ws_busy) cudaEventDestroy(s->ws_busy);
    for (int i = 0; i < 4; i++)
        if (s->ev[i]) cudaEventDestroy(s->ev[i]);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return GPURIR_OK;
}

extern "C" int gpurir_activate_mixed_precision(gpurir_sim *s, int activate, int *state) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (activate && s->lut) s->lut = 0;   // src/gpuRIR_cuda.cu:1052-1057
    s->mp = activate ? 1 : 0;
    if (state) *state = s->mp;
    return GPURIR_OK;
}

extern "C" int gpurir_activate_lut(gpurir_sim *s, int activate, int *state) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (activate && s->mp) s->mp = 0;     // src/gpuRIR_cuda.cu:1065-1069
    s->lut = activate ? 1 : 0;
    if (state) *state = s->lut;
    return GPURIR_OK;
}

extern "C" int gpurir_get_modes(gpurir_sim *s, int *mp, int *lut) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (mp) *mp = s->mp;
    if (lut) *lut = s->lut;
    return GPURIR_OK;
}

extern "C" int gpurir_set_noise(gpurir_sim *s, int kind) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (kind != GPURIR_NOISE_LOGISTIC && kind != GPURIR_NOISE_GAUSSIAN)
        return fail(GPURIR_ERR_INVALID, "unknown noise kind");
    s->noise = kind;
    return GPURIR_OK;
}

extern "C" int gpurir_set_seed(gpurir_sim *s, uint64_t seed, uint64_t calls) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    s->seed = seed;
    s->calls = calls;
    return GPURIR_OK;
}

extern "C" int gpurir_get_seed(gpurir_sim *s, uint64_t *seed, uint64_t *calls) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (seed) *seed = s->seed;
    if (calls) *calls = s->calls;
    return GPURIR_OK;
}

// ---------------------------------------------------------------------------
// Room description (host)
// ---------------------------------------------------------------------------
// cos(pi u) = (1 - 4u^2) * P(u^2) on |u| <= 1/2; P fitted by Chebyshev least
// squares on u^2 in [0, 1/4] (max error 3.4e-7 in cos, i.e. <7e-7 in the Hann
// window 0.5(1 + cos(2 pi x/Tw)) = cos^2(pi x/Tw) of src/gpuRIR_cuda.cu:110-112).
static const double kWinPoly[4] = {0.9999996612367829, -0.93477502063644,
                                   0.31901188401725716, -0.05416454340086296};

static int pow_table_len(const int nb[3]) {
    int mx = 0;
    for (int d = 0; d < 3; d++)
        for (int n = 0; n < nb[d]; n++) {
            int k = n - nb[d] / 2;
            int cl = (int)std::ceil(k / 2.0), r = std::abs(k % 2);
            mx = std::max(mx, std::max(std::abs(cl - r), std::abs(cl)));
        }
    return mx + 1;
}

static int build_room(RoomDesc &R, const float room[3], const float beta[6], const int nb[3],
                      float Tdiff, float Tmax, float Fs, float c, int spkr, int mic) {
    memset(&R, 0, sizeof(R));
    for (int d = 0; d < 3; d++) {
        if (!(room[d] > 0.0f) || !std::isfinite(room[d]))
            return fail(GPURIR_ERR_INVALID, "room_sz must be positive and finite");
        if (nb[d] < 1) return fail(GPURIR_ERR_INVALID, "nb_img must be >= 1 on every axis");
        R.L[d] = room[d];
        R.nb[d] = nb[d];
    }
    long long nimg = (long long)nb[0] * nb[1] * nb[2];
    if (nimg > (1LL << 30)) return fail(GPURIR_ERR_INVALID, "too many images (nb_img product > 2^30)");
    for (int w = 0; w < 6; w++) {
        if (!std::isfinite(beta[w])) return fail(GPURIR_ERR_INVALID, "beta must be finite");
        R.beta[w] = beta[w];
    }
    if (!(Fs > 0.0f) || !(c > 0.0f) || !std::isfinite(Fs) || !std::isfinite(c))
        return fail(GPURIR_ERR_INVALID, "Fs and c must be positive");
    if (!(Tmax >= 0.0f) || !(Tdiff >= 0.0f))
        return fail(GPURIR_ERR_INVALID, "Tmax and Tdiff must be >= 0");
    if (Tdiff > Tmax) return fail(GPURIR_ERR_INVALID, "Tmax must be equal or greater than Tdiff");
    if (spkr < 0 || spkr > 5 || mic < 0 || mic > 5)
        return fail(GPURIR_ERR_INVALID, "polar pattern must be in 0..5");
    R.n_img = (int)nimg;
    R.n_ism = gpurir_n_samples(Tdiff, Fs);
    R.n_total = gpurir_n_samples(Tmax, Fs);
    if (R.n_ism > R.n_total) R.n_ism = R.n_total;
    R.spkr = spkr;
    R.mic = mic;
    const int Tw = (int)roundf(8e-3f * Fs);          // src/gpuRIR_cuda.cu:629
    if (Tw < 1) return fail(GPURIR_ERR_INVALID, "Fs too small: window shorter than one sample");
    R.H = Tw / 2.0f;
    R.H2 = R.H * R.H;
    const double tw = (double)Tw;
    double scale = 4.0 / (tw * tw), tw2j = 1.0;
    for (int j = 0; j < 4; j++) {
        R.wc[j] = (float)(scale * kWinPoly[j] / tw2j);
        tw2j *= tw * tw;
    }
    const double K = (double)Fs / (double)c;
    R.kh = (float)K;
    R.kl = (float)(K - (double)R.kh);
    // SabineT60 in float32 as the reference evaluates it, src/gpuRIR_cuda.cu:123-130
    float Sa = ((1.0f - beta[0] * beta[0]) + (1.0f - beta[1] * beta[1])) * room[1] * room[2] +
               ((1.0f - beta[2] * beta[2]) + (1.0f - beta[3] * beta[3])) * room[0] * room[2] +
               ((1.0f - beta[4] * beta[4]) + (1.0f - beta[5] * beta[5])) * room[0] * room[1];
    R.T60 = 0.161f * (room[0] * room[1] * room[2]) / Sa;
    R.fs = Fs;
    R.pow_n = pow_table_len(nb);
    if (R.pow_n > kPowMax) return fail(GPURIR_ERR_INVALID, "nb_img too large for the reflection tables");
    for (int w = 0; w < 6; w++)
        for (int k = 0; k < kPowMax; k++)
            R.pw[w][k] = k < R.pow_n ? (float)std::pow(-(double)beta[w], (double)k) : 0.0f;
    return GPURIR_OK;
}

// ---------------------------------------------------------------------------
// Workspace
// ---------------------------------------------------------------------------
static int ensure_device(gpurir_sim *s, size_t bytes) {
    if (bytes <= s->d_ws_bytes) return GPURIR_OK;
    if (s->ws_recorded) CK(cudaEventSynchronize(s->ws_busy));
    if (s->d_ws) CK(cudaFree(s->d_ws));
    s->d_ws = nullptr;
    s->d_ws_bytes = 0;
    size_t want = align_up(bytes + bytes / 4, 1 << 20);
    CK(cudaMalloc(&s->d_ws, want));
    s->d_ws_bytes = want;
    return GPURIR_OK;
}

static int ensure_stage(gpurir_sim *s, size_t bytes) {
    if (s->stage_pending) {
        CK(cudaEventSynchronize(s->stage_done));
        s->stage_pending = false;
    }
    if (bytes <= s->h_stage_bytes) return GPURIR_OK;
    if (s->h_stage) CK(cudaFreeHost(s->h_stage));
    s->h_stage = nullptr;
    s->h_stage_bytes = 0;
    size_t want = align_up(bytes + bytes / 4, 1 << 16);
    CK(cudaMallocHost(&s->h_stage, want));
    s->h_stage_bytes = want;
    return GPURIR_OK;
}

struct Plan {
    int tpl, em, nsub, grid, clamp;
    std::vector<IsmItem> items;
    std::vector<IsmItem> rirs;
};

// Split every RIR of one room into segments and order the work.
static int plan_single_room(gpurir_sim *s, const RoomDesc &R, int M_src, int M_rcv, Plan &P) {
    P.tpl = ism_forward_pick_tpl(R.H);
    if (P.tpl < 0) return fail(GPURIR_ERR_UNSUPPORTED, "window too long (Fs above ~190 kHz)");
    const int sub = 32 * P.tpl;
    P.em = (int)align_up((size_t)std::ceil(R.H) + 2, 4);
    {   // taps k in [floor(-H)+1, floor(H)]: without padding taps, |k - f| < H always holds
        const int k_lo = (int)std::floor(-R.H) + 1, nk = (int)std::floor(R.H) - k_lo + 1;
        P.clamp = (nk != sub || R.H != std::floor(R.H)) ? 1 : 0;
    }
    int max_nsub = ism_forward_max_nsub(P.tpl, P.em, kSmemBudget);
    if (max_nsub < 4)   // long windows (high Fs): one block per SM with the whole shared memory
        max_nsub = ism_forward_max_nsub(P.tpl, P.em, kSmemBudgetLarge);
    if (max_nsub < 1) return fail(GPURIR_ERR_UNSUPPORTED, "window too long for shared memory");
    const long M = (long)M_src * M_rcv;
    const int n_ism = R.n_ism;
    P.items.clear();
    P.rirs.clear();
    P.rirs.reserve(M);
    for (long m = 0; m < M; m++) {
        IsmItem r{};
        r.room = 0; r.src = (int)(m / M_rcv); r.rcv = (int)(m % M_rcv);
        r.rir = (int)m;
        r.out_row = (long long)m * R.n_total;
        P.rirs.push_back(r);
    }
    P.nsub = 1;
    P.grid = 0;
    if (n_ism <= 0) return GPURIR_OK;
    const long seg_max = (long)max_nsub * sub;
    long min_seg = (n_ism + seg_max - 1) / seg_max;
    long target = 4L * s->num_sms;
    long want = (target + M - 1) / M;
    long cap = (n_ism + sub - 1) / sub;
    long n_seg = std::max(min_seg, std::min(want, cap));
    long tseg = align_up((size_t)((n_ism + n_seg - 1) / n_seg), 32);
    if (tseg > seg_max) tseg = seg_max;
    if (tseg > 16384) tseg = 16384;   // image offsets are stored as int16 relative to t_lo
    n_seg = (n_ism + tseg - 1) / tseg;
    P.nsub = (int)((tseg + sub - 1) / sub);
    P.items.reserve(M * n_seg);
    for (long g = n_seg - 1; g >= 0; g--)   // later segments hold more images: start them first
        for (long m = 0; m < M; m++) {
            IsmItem it = P.rirs[m];
            it.t_lo = (int)(g * tseg);
            it.t_hi = (int)std::min<long>((g + 1) * tseg, n_ism);
            P.items.push_back(it);
        }
    size_t smem = ism_forward_smem_bytes(P.tpl, P.em, P.nsub);
    int bps = ism_forward_blocks_per_sm(P.tpl, smem);
    if (bps < 1) return fail(GPURIR_ERR_CUDA, "ISM kernel does not fit on an SM");
    P.grid = (int)std::min<long>((long)P.items.size(), (long)s->num_sms * bps);
    return GPURIR_OK;
}

static int check_status(gpurir_sim *s) {
    if (s->h_ctl[1] != 0) {
        int code = s->h_ctl[1];
        cudaMemsetAsync(s->d_ctl + 1, 0, sizeof(int), s->stream);
        return fail(GPURIR_ERR_DEVICE, "kernel rejected a work item (code " + std::to_string(code) + ")");
    }
    return GPURIR_OK;
}

// Shared body of the host and device entry points.
static int simulate_one_room(gpurir_sim *s, const float room_sz[3], const float beta[6],
                             const float *pos_src, int M_src, const float *pos_rcv,
                             const float *orV_src, const float *orV_rcv, int spkr, int mic,
                             int M_rcv, const int nb_img[3], float Tdiff, float Tmax, float Fs,
                             float c, float *out, bool host_io, cudaStream_t st) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (!room_sz || !beta || !nb_img || !pos_src || !pos_rcv || !out)
        return fail(GPURIR_ERR_INVALID, "NULL argument");
    if (M_src < 1 || M_rcv < 1) return fail(GPURIR_ERR_INVALID, "need at least one source and one receiver");
    if ((spkr != 0 && !orV_src) || (mic != 0 && !orV_rcv))
        return fail(GPURIR_ERR_INVALID, "orientation required for a non-omni pattern");
    if ((long long)M_src * M_rcv > (1LL << 30)) return fail(GPURIR_ERR_INVALID, "too many RIRs");
    RoomDesc R;
    int rc = build_room(R, room_sz, beta, nb_img, Tdiff, Tmax, Fs, c, spkr, mic);
    if (rc) return rc;
    R.n_src = M_src; R.n_rcv = M_rcv;
    Plan P;
    rc = plan_single_room(s, R, M_src, M_rcv, P);
    if (rc) return rc;
    const long M = (long)M_src * M_rcv;
    // Staging layout, mirrored byte for byte in the device workspace.
    size_t o_room = 0;
    size_t o_items = align_up(o_room + sizeof(RoomDesc), 256);
    size_t o_rirs = align_up(o_items + P.items.size() * sizeof(IsmItem), 256);
    size_t o_pos = align_up(o_rirs + P.rirs.size() * sizeof(IsmItem), 256);
    size_t n_pos = host_io ? (size_t)(M_src + M_rcv) * 3 * 2 : 0;
    size_t stage_bytes = align_up(o_pos + n_pos * sizeof(float), 256);
    size_t o_env = stage_bytes;
    size_t o_out = align_up(o_env + (size_t)M * 3 * sizeof(float), 256);
    size_t dev_bytes = o_out + (host_io ? (size_t)M * R.n_total * sizeof(float) : 0);
    if ((rc = ensure_device(s, dev_bytes))) return rc;
    if ((rc = ensure_stage(s, stage_bytes))) return rc;
    char *h = s->h_stage;
    memcpy(h + o_room, &R, sizeof(R));
    if (!P.items.empty()) memcpy(h + o_items, P.items.data(), P.items.size() * sizeof(IsmItem));
    memcpy(h + o_rirs, P.rirs.data(), P.rirs.size() * sizeof(IsmItem));
    const float *dps = pos_src, *dpr = pos_rcv, *dos = orV_src, *dor = orV_rcv;
    char *d = s->d_ws;
    if (host_io) {
        float *hp = reinterpret_cast<float *>(h + o_pos);
        memcpy(hp, pos_src, sizeof(float) * 3 * M_src);
        memcpy(hp + 3 * M_src, pos_rcv, sizeof(float) * 3 * M_rcv);
        if (orV_src) memcpy(hp + 3 * (M_src + M_rcv), orV_src, sizeof(float) * 3 * M_src);
        else memset(hp + 3 * (M_src + M_rcv), 0, sizeof(float) * 3 * M_src);
        if (orV_rcv) memcpy(hp + 3 * (2 * M_src + M_rcv), orV_rcv, sizeof(float) * 3 * M_rcv);
        else memset(hp + 3 * (2 * M_src + M_rcv), 0, sizeof(float) * 3 * M_rcv);
        float *dp = reinterpret_cast<float *>(d + o_pos);
        dps = dp; dpr = dp + 3 * M_src; dos = dp + 3 * (M_src + M_rcv); dor = dp + 3 * (2 * M_src + M_rcv);
    }
    if (s->ws_recorded) CK(cudaStreamWaitEvent(st, s->ws_busy, 0));   // earlier calls, any stream
    CK(cudaMemcpyAsync(d, h, stage_bytes, cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(s->stage_done, st));
    s->stage_pending = true;
    float *dout = host_io ? reinterpret_cast<float *>(d + o_out) : out;
    const RoomDesc *drooms = reinterpret_cast<const RoomDesc *>(d + o_room);
    s->ev_ism = s->ev_tail = false;
    s->last_h2d = stage_bytes;
    s->last_d2h = sizeof(int) + (host_io ? (uint64_t)M * R.n_total * sizeof(float) : 0);
    if (s->profile && P.grid > 0) { CK(cudaEventRecord(s->ev[0], st)); s->ev_ism = true; }
    if (P.grid > 0)
        CK(ism_forward_launch(P.tpl, drooms, reinterpret_cast<const IsmItem *>(d + o_items),
                              (int)P.items.size(), dps, dpr, dos, dor, dout, s->d_ctl, s->d_ctl + 1,
                              P.em, P.nsub, P.clamp, P.grid, st));
    if (s->ev_ism) CK(cudaEventRecord(s->ev[1], st));
    const int n_diff = R.n_total - R.n_ism;
    if (s->profile && n_diff > 0) { CK(cudaEventRecord(s->ev[2], st)); s->ev_tail = true; }
    if (n_diff > 0)
        CK(tail_launch(drooms, reinterpret_cast<const IsmItem *>(d + o_rirs), (int)M, n_diff, dps, dpr,
                       dout, s->seed, s->calls, s->noise, reinterpret_cast<float *>(d + o_env), st));
    if (s->ev_tail) CK(cudaEventRecord(s->ev[3], st));
    s->env_off = o_env;
    s->last_n_rir = n_diff > 0 ? M : 0;
    s->calls++;
    CK(cudaMemcpyAsync(s->h_ctl + 1, s->d_ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (host_io)
        CK(cudaMemcpyAsync(out, dout, (size_t)M * R.n_total * sizeof(float), cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(s->ws_busy, st));
    s->ws_recorded = true;
    if (host_io) {
        CK(cudaStreamSynchronize(st));
        return check_status(s);
    }
    return GPURIR_OK;
}

extern "C" int gpurir_simulate_rir(gpurir_sim *s, const float room_sz[3], const float beta[6],
                                   const float *pos_src, int M_src, const float *pos_rcv,
                                   const float *orV_src, const float *orV_rcv, int spkr_pattern,
                                   int mic_pattern, int M_rcv, const int nb_img[3], float Tdiff,
                                   float Tmax, float Fs, float c, float *rir_out) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    return simulate_one_room(s, room_sz, beta, pos_src, M_src, pos_rcv, orV_src, orV_rcv,
                             spkr_pattern, mic_pattern, M_rcv, nb_img, Tdiff, Tmax, Fs, c, rir_out,
                             true, s->stream);
}

extern "C" int gpurir_simulate_rir_device(gpurir_sim *s, const float room_sz[3], const float beta[6],
                                          const float *d_pos_src, int M_src, const float *d_pos_rcv,
                                          const float *d_orV_src, const float *d_orV_rcv,
                                          int spkr_pattern, int mic_pattern, int M_rcv,
                                          const int nb_img[3], float Tdiff, float Tmax, float Fs,
                                          float c, float *d_rir_out, void *stream) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);   // NULL: the CUDA default stream
    return simulate_one_room(s, room_sz, beta, d_pos_src, M_src, d_pos_rcv, d_orV_src, d_orV_rcv,
                             spkr_pattern, mic_pattern, M_rcv, nb_img, Tdiff, Tmax, Fs, c,
                             d_rir_out, false, st);
}

extern "C" int gpurir_philox_stream_device(uint64_t seed, uint64_t calls, uint32_t rir, long n,
                                           uint32_t *d_out, void *stream) {
    if (n < 0 || (n > 0 && !d_out)) return fail(GPURIR_ERR_INVALID, "bad output");
    CK(philox_stream_launch(d_out, n, seed, calls, rir, reinterpret_cast<cudaStream_t>(stream)));
    return GPURIR_OK;
}

extern "C" int gpurir_last_envelope(gpurir_sim *s, float *out, long n) {
    if (!s || !out) return fail(GPURIR_ERR_INVALID, "NULL argument");
    if (n > s->last_n_rir) return fail(GPURIR_ERR_INVALID, "fewer RIRs had a tail in the last call");
    if (n <= 0) return GPURIR_OK;
    if (s->ws_recorded) CK(cudaEventSynchronize(s->ws_busy));
    CK(cudaMemcpy(out, s->d_ws + s->env_off, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost));
    return GPURIR_OK;
}

extern "C" int gpurir_probe_peaks(double *fp32_flops, double *mufu_ops) {
    if (!fp32_flops || !mufu_ops) return fail(GPURIR_ERR_INVALID, "NULL argument");
    CK(probe_peaks(fp32_flops, mufu_ops, nullptr));
    return GPURIR_OK;
}

extern "C" int gpurir_set_profiling(gpurir_sim *s, int on) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (on && !s->ev[0])
        for (int i = 0; i < 4; i++) CK(cudaEventCreate(&s->ev[i]));
    s->profile = on ? 1 : 0;
    return GPURIR_OK;
}

extern "C" int gpurir_last_timing(gpurir_sim *s, float *ism_ms, float *tail_ms) {
    if (!s || !ism_ms || !tail_ms) return fail(GPURIR_ERR_INVALID, "NULL argument");
    *ism_ms = *tail_ms = 0.0f;
    if (s->ev_ism) {
        CK(cudaEventSynchronize(s->ev[1]));
        CK(cudaEventElapsedTime(ism_ms, s->ev[0], s->ev[1]));
    }
    if (s->ev_tail) {
        CK(cudaEventSynchronize(s->ev[3]));
        CK(cudaEventElapsedTime(tail_ms, s->ev[2], s->ev[3]));
    }
    return GPURIR_OK;
}

extern "C" int gpurir_last_transfer_bytes(gpurir_sim *s, uint64_t *h2d, uint64_t *d2h) {
    if (!s || !h2d || !d2h) return fail(GPURIR_ERR_INVALID, "NULL argument");
    *h2d = s->last_h2d;
    *d2h = s->last_d2h;
    return GPURIR_OK;
}
