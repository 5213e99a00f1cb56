// capi.cu -- C ABI and host orchestration of gpurir_gb300.
//
// The host half of gpuRIR (gpuRIR_cuda::cuda_simulateRIR, src/gpuRIR_cuda.cu:
// 766-931) allocates and frees every buffer per call, launches each stage on
// the legacy stream with a device-wide synchronisation after it, and exit()s
// on any error.  Here a handle keeps a grow-only device workspace and pinned
// staging memory, all launch descriptors go to the device in one copy, the
// two kernels run back to back on one stream, and errors come back as codes.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gpurir_internal.cuh"
#include "../../include/gpurir_gb300.h"

namespace gpurir {
size_t ism_forward_smem_bytes(int tpl, int em, int max_nsub, int mode, int tw);
int ism_forward_max_nsub(int tpl, int em, size_t smem_budget, int mode, int tw);
int ism_forward_pick_tpl(float H);
int ism_forward_blocks_per_sm(int tpl, size_t smem, int mode);
cudaError_t ism_forward_launch(int tpl, const RoomDesc *rooms, const IsmItem *items, int n_items,
                               const float *pos_src, const float *pos_rcv, const float *orv_src,
                               const float *orv_rcv, float *out, int *work_counter, int *status,
                               int em, int max_nsub, int clamp, int grid, cudaStream_t st, int mode,
                               int tw, const TailArgs *tail, float4 *axis_tab, int axis_cap,
                               float *partial, const unsigned char *skip);
cudaError_t item_skip_launch(const RoomDesc *rooms, const IsmItem *items, int n_items, const float *pos_src,
                             const float *pos_rcv, unsigned char *skip, cudaStream_t st);
cudaError_t partial_reduce_launch(const PartGroup *groups, int n_groups, int max_len, const float *part,
                                  float *out, cudaStream_t st);
cudaError_t tail_launch(const RoomDesc *rooms, const IsmItem *rirs, int n_rir, int max_n_diff,
                        const float *pos_src, const float *pos_rcv, float *out, uint64_t seed,
                        uint64_t offset, const uint64_t *offset_ptr, int noise_kind, float *env_out,
                        cudaStream_t st, const unsigned char *pre);
cudaError_t philox_stream_launch(uint32_t *out, long n, uint64_t seed, uint64_t offset,
                                 uint32_t rir, cudaStream_t st);
cudaError_t probe_peaks(double *fp32_flops, double *mufu_ops, cudaStream_t st);
size_t ism_backward_smem_bytes(int tpl, int max_tseg, int pad, int axis_cap);
cudaError_t ism_backward_launch(int tpl, const RoomDesc *rooms, const IsmItem *items, int n_items,
                                const float *pos_src, const float *pos_rcv, const float *orv_src,
                                const float *orv_rcv, const float *grad, float *item_grad,
                                int *work_counter, int *status, int max_tseg, int axis_cap, int grid,
                                int clamp, cudaStream_t st);
cudaError_t grad_reduce_launch(const float *item_grad, const int *const csr[6], int n_rooms, int n_src,
                               int n_rcv, float *const out[5], cudaStream_t st);
int ism_backward_blocks_per_sm(int tpl, int clamp, size_t smem);
size_t fft_smem_bytes(int M);
size_t fft_scratch_floats2(int M, int grid);
cudaError_t twiddle_launch(float2 *w, int n, cudaStream_t st);
cudaError_t segment_spectra_launch(const float *seg, int P, int S, int M, const float2 *W, float2 *Sg,
                                   float2 *scratch, int grid, cudaStream_t st);
cudaError_t rir_conv_launch(const float *rir, int P, int R, int L, int S, int M, const float2 *W,
                            const float2 *Sg, float *out, long out_ld, float2 *scratch, int grid,
                            cudaStream_t st);
cudaError_t ola_launch(const float *conv, long conv_ld, const int *w_ini, const int *w_len, int P, int R,
                       int L, long n_out, int uni_w, double *out, cudaStream_t st);
int traj_adjoint_grid(int M, int P, int num_sms);
cudaError_t traj_adjoint_launch(const double *g, long n_out, const int *w_ini, const int *w_len, const float *rir,
                                int P, int R, int L, int M, const float2 *W, const float2 *Sg, float *gt,
                                float *grad_rir, float *grad_sig, float2 *acc, int grid, cudaStream_t st);
cudaError_t room_beta_launch(RoomDesc *rooms, int n_rooms, const float *beta, cudaStream_t st);
int l2_grad_blocks(long n);
int tuning(int knob);
cudaError_t l2_grad_launch(const float *y, const float *t, long n, float scale, float *g, double *partial,
                           float *loss, cudaStream_t st);
cudaError_t room_beta_skip_launch(RoomDesc *rooms, int n_rooms, const float *beta, const IsmItem *items,
                                  int n_items, const float *pos_src, const float *pos_rcv, unsigned char *skip,
                                  cudaStream_t st);
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
static const long kPartImages = 2048;   // fewest images per part of a split RIR (one chunk)
// Early parts from this many samples on (0.5 s at 16 kHz) are accumulated with
// compensation in the lookup-table mode (policy 1).  Mixed precision is left out
// of the automatic choice: its half-precision window (1.3e-4 rel-L2) dwarfs the
// accumulation error, which compensation brings from 5.8e-7 to 1.9e-7 at 1 s.
static const int kCompMinSamples = 8000;

struct PlanCache;
static void free_plan_cache(PlanCache *c);

struct gpurir_sim {
    int mp = 0, lut = 0;
    int ref_delay = 0;   // image delays in the reference's float32 arithmetic (RoomDesc::ref_delay)
    int comp = 1;        // compensated accumulation: 0 never, 1 long RIRs in LUT mode, 2 always in MP/LUT
    uint64_t seed = 1234, calls = 0;
    int noise = GPURIR_NOISE_LOGISTIC;
    int device = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    char *d_ws = nullptr;
    size_t d_ws_bytes = 0;
    // Pinned staging of descriptors, a ring of kStageRing buffers so that a call never
    // waits for the previous call's upload: h_stage / stage_done / stage_pending are
    // the slot in use (ensure_stage rotates).
    struct StageSlot { char *h = nullptr; size_t bytes = 0; cudaEvent_t ev = nullptr; bool pending = false; };
    static constexpr int kStageRing = 4;
    StageSlot stage_ring[kStageRing];
    int stage_slot = 0;
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
    int host_direct = -1;      // kernels may store into pageable host memory (-1: not yet queried)
    bool last_direct = false;  // the last host call wrote its RIRs from the kernels
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool ev_ism = false, ev_tail = false;
    int last_launches = 0;        // kernels the last simulate call launched
    // The plan of the last simulate call, reused by a call with the same room shapes
    // (sizes, image counts, lengths, source/receiver counts: what the work items depend
    // on); its items stay on the device while ws_gen == the generation they were
    // staged under (a reallocation or another call's upload bumps ws_gen).
    PlanCache *pcache = nullptr;
    uint64_t ws_gen = 0;
    uint64_t last_h2d = 0, last_d2h = 0;
    // convolution: twiddle tables per FFT size, and a grow-only workspace
    std::vector<std::pair<int, float2 *>> twiddles;
    char *d_conv = nullptr;
    size_t d_conv_bytes = 0;
    cudaEvent_t conv_busy = nullptr;
    bool conv_recorded = false;
    // silent tails of host-output calls, streamed by a copy engine from a zero buffer
    cudaStream_t side = nullptr;
    cudaEvent_t side_done = nullptr;
    char *d_zero = nullptr;
    size_t zero_bytes = 0;
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
    for (int k = 0; k < gpurir_sim::kStageRing && e == cudaSuccess; k++)
        e = cudaEventCreateWithFlags(&s->stage_ring[k].ev, cudaEventDisableTiming);
    s->stage_done = s->stage_ring[0].ev;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ws_busy, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->conv_busy, cudaEventDisableTiming);
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
    if (s->side) cudaStreamSynchronize(s->side);
    if (s->d_ws) cudaFree(s->d_ws);
    if (s->d_zero) cudaFree(s->d_zero);
    if (s->side_done) cudaEventDestroy(s->side_done);
    if (s->side) cudaStreamDestroy(s->side);
    free_plan_cache(s->pcache);
    s->stage_ring[s->stage_slot].h = s->h_stage;
    for (int k = 0; k < gpurir_sim::kStageRing; k++)
        if (s->stage_ring[k].h) cudaFreeHost(s->stage_ring[k].h);
    if (s->d_ctl) cudaFree(s->d_ctl);
    if (s->h_ctl) cudaFreeHost(s->h_ctl);
    for (int k = 0; k < gpurir_sim::kStageRing; k++)
        if (s->stage_ring[k].ev) cudaEventDestroy(s->stage_ring[k].ev);
    if (s->ws_busy) cudaEventDestroy(s->ws_busy);
    if (s->conv_busy) cudaEventDestroy(s->conv_busy);
    for (auto &t : s->twiddles) cudaFree(t.second);
    if (s->d_conv) cudaFree(s->d_conv);
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

extern "C" int gpurir_set_reference_delays(gpurir_sim *s, int activate, int *state) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    s->ref_delay = activate ? 1 : 0;
    if (state) *state = s->ref_delay;
    return GPURIR_OK;
}

extern "C" int gpurir_set_compensation(gpurir_sim *s, int policy) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (policy < 0 || policy > 2) return fail(GPURIR_ERR_INVALID, "compensation policy must be 0, 1 or 2");
    s->comp = policy;
    return GPURIR_OK;
}

extern "C" int gpurir_get_reference_delays(gpurir_sim *s, int *state) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (state) *state = s->ref_delay;
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
    // the kernels split image indices with float arithmetic: exact below 2^24
    if (nimg > (1LL << 24)) return fail(GPURIR_ERR_UNSUPPORTED, "too many images (nb_img product > 2^24)");
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
    R.c = c;
    R.pow_n = pow_table_len(nb);
    if (R.pow_n > kPowMax) return fail(GPURIR_ERR_INVALID, "nb_img too large for the reflection tables");
    // (-beta)^k by repeated FP64 products rounded to float32: the room-table kernel of
    // the device-beta entries forms them the same way, so both paths agree bit for bit
    for (int w = 0; w < 6; w++) {
        const double m = -(double)beta[w];
        double p = 1.0;
        for (int k = 0; k < kPowMax; k++) {
            R.pw[w][k] = k < R.pow_n ? (float)p : 0.0f;
            p *= m;
        }
    }
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
    s->ws_gen++;
    CK(cudaMalloc(&s->d_ws, want));
    s->d_ws_bytes = want;
    return GPURIR_OK;
}

static int ensure_stage(gpurir_sim *s, size_t bytes) {
    // park the slot in use, take the next one (its upload was issued kStageRing calls ago)
    gpurir_sim::StageSlot &cur = s->stage_ring[s->stage_slot];
    cur.h = s->h_stage;
    cur.bytes = s->h_stage_bytes;
    cur.pending = s->stage_pending;
    s->stage_slot = (s->stage_slot + 1) % gpurir_sim::kStageRing;
    gpurir_sim::StageSlot &g = s->stage_ring[s->stage_slot];
    if (g.pending) {
        CK(cudaEventSynchronize(g.ev));
        g.pending = false;
    }
    if (bytes > g.bytes) {
        if (g.h) CK(cudaFreeHost(g.h));
        g.h = nullptr;
        g.bytes = 0;
        size_t want = align_up(bytes + bytes / 4, 1 << 16);
        CK(cudaMallocHost(&g.h, want));
        g.bytes = want;
    }
    s->h_stage = g.h;
    s->h_stage_bytes = g.bytes;
    s->stage_done = g.ev;
    s->stage_pending = false;
    return GPURIR_OK;
}

struct Plan {
    int tpl, em, nsub, grid, clamp;
    long unfused_tails = 0;   // RIRs whose tail the separate tail kernel writes
    int axis_cap = 0;         // per-axis table entries per block (max over rooms of N0 + N1 + N2)
    std::vector<PartGroup> groups;   // partial segments to add up (RIRs split by images)
    long long part_floats = 0;       // size of the partial-segment buffer
    int max_part_len = 0;
    int mode = 0, tw = 0;   // tap evaluation mode (0 FP32, 1 mixed precision, 2 LUT), window length
    int max_n_diff;
    bool skip_flags = false;   // some segment starts past the rooms' delay bound: test items on the device
    std::vector<IsmItem> items;
    std::vector<IsmItem> rirs;
};

// Launch geometry shared by every room of a launch (all rooms use one Fs).
static int plan_window(float H, Plan &P, int &max_nsub) {
    P.tw = (int)std::lround(2.0 * H);
    P.tpl = ism_forward_pick_tpl(H);
    if (P.tpl < 0) return fail(GPURIR_ERR_UNSUPPORTED, "window too long (Fs above ~190 kHz)");
    const int sub = 32 * P.tpl;
    P.em = (int)align_up((size_t)std::ceil(H) + 2, 4);
    {   // taps k in [floor(-H)+1, floor(H)]: without padding taps, |k - f| < H always holds
        const int k_lo = (int)std::floor(-H) + 1, nk = (int)std::floor(H) - k_lo + 1;
        P.clamp = (nk != sub || H != std::floor(H)) ? 1 : 0;
    }
    max_nsub = ism_forward_max_nsub(P.tpl, P.em, kSmemBudget, P.mode, P.tw);
    if (max_nsub < 4)   // long windows (high Fs): one block per SM with the whole shared memory
        max_nsub = ism_forward_max_nsub(P.tpl, P.em, kSmemBudgetLarge, P.mode, P.tw);
    if (max_nsub < 1) return fail(GPURIR_ERR_UNSUPPORTED, "window too long for shared memory");
    return GPURIR_OK;
}

// Latest sample any image of the room can reach while source and receiver are inside
// it: |receiver -> image| <= (N/2 + 1) L per axis, plus the window and a margin.
static double room_span(const RoomDesc &r) {
    double reach2 = 0.0;
    for (int a = 0; a < 3; a++) {
        const double e = (double)(r.nb[a] / 2 + 1) * r.L[a];
        reach2 += e * e;
    }
    return std::sqrt(reach2) * ((double)r.kh + r.kl) + r.H + 2.0;
}

// Work items for a set of rooms.  Every RIR is cut into segments of at most
// what one block's shared memory holds; RIRs of small launches are cut finer so
// that the persistent grid has work for every SM.  Items are ordered by an
// estimate of their cost, largest first (longest-processing-time order).
static int plan_rooms(gpurir_sim *s, const std::vector<RoomDesc> &R, Plan &P) {
    int max_nsub = 0;
    P.mode = s->lut ? 2 : (s->mp ? 1 : 0);
    if (P.mode != 0 && s->comp > 0) {   // compensated accumulation (mode flag 4, ism_forward.cu)
        int longest = 0;
        for (const RoomDesc &r : R) longest = std::max(longest, r.n_ism);
        if (s->comp == 2 || (P.mode == 2 && longest >= kCompMinSamples)) P.mode |= 4;
    }
    int rc = plan_window(R[0].H, P, max_nsub);
    if (rc) return rc;
    const int sub = 32 * P.tpl;
    long M_tot = 0;
    P.max_n_diff = 0;
    P.axis_cap = 0;
    for (const RoomDesc &r : R) {
        M_tot += (long)r.n_src * r.n_rcv;
        P.max_n_diff = std::max(P.max_n_diff, r.n_total - r.n_ism);
        P.axis_cap = std::max(P.axis_cap, r.nb[0] + r.nb[1] + r.nb[2]);
    }
    P.items.clear();
    P.rirs.clear();
    P.skip_flags = false;
    P.groups.clear();
    P.part_floats = 0;
    P.max_part_len = 0;
    P.unfused_tails = 0;
    P.rirs.reserve(M_tot);
    const long seg_max = std::min<long>((long)max_nsub * sub, 16384);   // int16 image offsets
    const long target = 4L * s->num_sms;
    const long want = (target + M_tot - 1) / std::max<long>(M_tot, 1);
    std::vector<IsmItem> work;
    std::vector<std::pair<double, int>> cost;   // (estimated cost, index into work)
    work.reserve(M_tot);
    cost.reserve(M_tot);
    P.nsub = 1;
    for (size_t ri = 0; ri < R.size(); ri++) {
        const RoomDesc &r = R[ri];
        const long M = (long)r.n_src * r.n_rcv;
        long n_seg = 0, n_part = 1;
        std::vector<std::pair<int, int>> segs;   // [t_lo, t_hi) of each segment
        // Latest delay of any image while source and receiver are inside the room:
        // |receiver -> image| <= (N/2 + 1) L per axis.  Only an estimate for the cost
        // order (segments beyond it hold no image); the kernels test each item against
        // the actual positions and skip the image work of segments no image reaches.
        const double span = room_span(r);
        auto cut = [&](long lo, long hi, long n) {   // n segments of [lo, hi), 32-aligned
            const long t = std::min<long>(align_up((size_t)((hi - lo + n - 1) / n), 32), seg_max);
            for (long a = lo; a < hi; a += t) segs.push_back({(int)a, (int)std::min(a + t, hi)});
        };
        if (r.n_ism > 0) {
            const long min_seg = (r.n_ism + seg_max - 1) / seg_max;
            const long cap = (r.n_ism + sub - 1) / sub;
            // Small launches need more items than RIRs.  Splitting an RIR's images into
            // parts (partial segments added up afterwards) costs no extra image work;
            // cutting its time axis finer makes every segment walk all the images.  So
            // parts first, at least kPartImages images each, then finer segments.
            n_part = std::max<long>(1, std::min<long>((want + min_seg - 1) / min_seg,
                                                        r.n_img / kPartImages));
            n_seg = std::max(min_seg, std::min((want + n_part - 1) / n_part, cap));
            // (cutting only the images' span finer, and the zeros after it into few long
            // segments, was slower on small launches: more items, each with its fixed
            // setup, planning and output)
            cut(0, r.n_ism, n_seg);
            n_seg = (long)segs.size();
            for (auto &g : segs) P.nsub = std::max<int>(P.nsub, (g.second - g.first + sub - 1) / sub);
        }
        // a single-segment RIR holding all its images gets its tail from the ISM
        // kernel's epilogue
        const bool fused = n_seg == 1 && n_part == 1 && r.n_total > r.n_ism;
        for (long m = 0; m < M; m++) {
            IsmItem it{};
            it.room = (int)ri;
            it.src = r.src_off + (int)(m / r.n_rcv);
            it.rcv = r.rcv_off + (int)(m % r.n_rcv);
            it.rir = r.rir_off + (int)m;
            it.out_row = r.out_off + (long long)m * r.n_total;
            IsmItem ref = it;
            ref.t_hi = fused ? -1 : 0;   // -1: the tail kernel skips this RIR
            P.rirs.push_back(ref);
            if (!fused && r.n_total > r.n_ism) P.unfused_tails++;
            for (long g = 0; g < n_seg; g++) {
                IsmItem w = it;
                w.t_lo = segs[g].first;
                w.t_hi = segs[g].second;
                w.part_off = -1;
                const int len = w.t_hi - w.t_lo;
                if (n_part > 1) {
                    P.groups.push_back({it.out_row + w.t_lo, P.part_floats, len, (int)n_part});
                    P.max_part_len = std::max(P.max_part_len, len);
                }
                // images in the segment's delay range (density grows with delay^2, none
                // beyond the span), the geometry pass over every image of the part when
                // any can reach the segment, and the samples written
                const double S = std::max(span, 1.0);
                const double a = std::min<double>(w.t_lo, S) / S, b = std::min<double>(w.t_hi, S) / S;
                const double walk = w.t_lo < S ? 0.15 : 0.0;
                for (long p = 0; p < n_part; p++) {
                    w.i_lo = (int)((long long)r.n_img * p / n_part);
                    w.i_hi = (int)((long long)r.n_img * (p + 1) / n_part);
                    if (n_part > 1) {
                        w.part_off = P.part_floats;
                        P.part_floats += len;
                    }
                    cost.push_back({(w.i_hi - w.i_lo) * ((b * b * b - a * a * a) + walk) + 2e-3 * len,
                                    (int)work.size()});
                    P.skip_flags |= w.t_lo > 0 && w.t_lo >= S;
                    work.push_back(w);
                }
            }
        }
    }
    // largest first, ties in plan order; a single room cut into one segment per RIR
    // (all costs equal) is already in that order
    bool sorted = true;
    for (size_t i = 1; i < cost.size() && sorted; i++) sorted = cost[i - 1].first >= cost[i].first;
    if (!sorted)
        std::stable_sort(cost.begin(), cost.end(), [](const std::pair<double, int> &x,
                                                      const std::pair<double, int> &y) { return x.first > y.first; });
    P.items.reserve(work.size());
    for (auto &c : cost) P.items.push_back(work[c.second]);

    P.grid = 0;
    if (P.items.empty()) return GPURIR_OK;
    size_t smem = ism_forward_smem_bytes(P.tpl, P.em, P.nsub, P.mode, P.tw);
    int bps = ism_forward_blocks_per_sm(P.tpl, smem, P.mode);
    if (bps < 1) return fail(GPURIR_ERR_CUDA, "ISM kernel does not fit on an SM");
    if (tuning(1) > 0) bps = std::min(bps, tuning(1));   // ism_blocks_per_sm (tuning.cu)
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

// Byte layout of one launch's descriptors (mirrored host staging -> device).
struct Layout {
    size_t o_rooms, o_items, o_rirs, o_groups, o_pos, o_pre, stage_bytes, o_env, o_axis, o_part, o_skip, o_out,
        dev_bytes;
};

static Layout make_layout(const Plan &P, size_t n_rooms, long n_src, long n_rcv, long M,
                          long long out_elems, bool host_io) {
    Layout L;
    // rooms and positions first: the part of an upload that changes from call to call
    L.o_rooms = 0;
    L.o_pos = align_up(L.o_rooms + n_rooms * sizeof(RoomDesc), 256);
    size_t n_pos = host_io ? (size_t)(n_src + n_rcv) * 3 * 2 : 0;
    L.o_pre = align_up(L.o_pos + n_pos * sizeof(float), 256);   // per-RIR silent-tail flags (host I/O)
    L.o_items = align_up(L.o_pre + (host_io ? (size_t)M : 0), 256);
    L.o_rirs = align_up(L.o_items + P.items.size() * sizeof(IsmItem), 256);
    L.o_groups = align_up(L.o_rirs + P.rirs.size() * sizeof(IsmItem), 256);
    L.stage_bytes = align_up(L.o_groups + P.groups.size() * sizeof(PartGroup), 256);
    L.o_env = L.stage_bytes;
    L.o_axis = align_up(L.o_env + (size_t)M * 3 * sizeof(float), 256);
    L.o_part = align_up(L.o_axis + (size_t)P.grid * P.axis_cap * sizeof(float4), 256);
    L.o_skip = align_up(L.o_part + (size_t)P.part_floats * sizeof(float), 256);
    L.o_out = align_up(L.o_skip + (P.skip_flags ? P.items.size() : 0), 256);
    L.dev_bytes = L.o_out + (host_io ? (size_t)out_elems * sizeof(float) : 0);
    return L;
}

struct PlanCache {
    std::vector<double> key;
    Plan P;
    Layout L;
    uint64_t gen = ~0ull;   // ws_gen under which P's items were uploaded
};

static void free_plan_cache(PlanCache *c) { delete c; }

// What the plan of simulate_rooms depends on: per room the sizes, image counts,
// lengths, window, Fs/c, source/receiver counts and patterns; the evaluation mode;
// where the output goes.
static std::vector<double> plan_key(const gpurir_sim *s, const std::vector<RoomDesc> &R, bool host_io,
                                    long long out_elems) {
    std::vector<double> k;
    k.reserve(4 + 16 * R.size());
    k.push_back((double)s->mp);
    k.push_back((double)s->lut);
    k.push_back((double)s->comp);
    k.push_back((double)tuning(1));   // the launch shape follows ism_blocks_per_sm
    k.push_back(host_io ? 1.0 : 0.0);
    k.push_back((double)out_elems);
    for (const RoomDesc &r : R) {
        for (int a = 0; a < 3; a++) k.push_back(r.L[a]);
        for (int a = 0; a < 3; a++) k.push_back((double)r.nb[a]);
        k.push_back((double)r.n_ism);
        k.push_back((double)r.n_total);
        k.push_back((double)r.n_src);
        k.push_back((double)r.n_rcv);
        k.push_back(r.H);
        k.push_back(r.kh);
        k.push_back(r.kl);
        k.push_back((double)r.spkr);
        k.push_back((double)r.mic);
    }
    return k;
}

static void fill_stage(char *h, const Layout &L, const std::vector<RoomDesc> &R, const Plan &P) {
    memcpy(h + L.o_rooms, R.data(), R.size() * sizeof(RoomDesc));
    if (!P.items.empty()) memcpy(h + L.o_items, P.items.data(), P.items.size() * sizeof(IsmItem));
    if (!P.rirs.empty()) memcpy(h + L.o_rirs, P.rirs.data(), P.rirs.size() * sizeof(IsmItem));
    if (!P.groups.empty()) memcpy(h + L.o_groups, P.groups.data(), P.groups.size() * sizeof(PartGroup));
}

// Enqueue the ISM and tail kernels of one planned launch on `st`.
static int enqueue_kernels(gpurir_sim *s, const Plan &P, const char *d, const Layout &L, long M,
                           const float *dps, const float *dpr, const float *dos, const float *dor,
                           float *dout, int *work_counter, const uint64_t *offset_ptr,
                           cudaStream_t st, bool record, bool skip_ready = false,
                           const unsigned char *tail_pre = nullptr) {
    const RoomDesc *drooms = reinterpret_cast<const RoomDesc *>(d + L.o_rooms);
    if (record && s->profile && P.grid > 0) { CK(cudaEventRecord(s->ev[0], st)); s->ev_ism = true; }
    TailArgs ta;
    ta.seed = s->seed;
    ta.offset = s->calls;
    ta.offset_ptr = offset_ptr;
    ta.noise_kind = s->noise;
    ta.env_out = reinterpret_cast<float *>(const_cast<char *>(d) + L.o_env);
    ta.fuse = 1;
    ta.pre = tail_pre;
    if (record) s->last_launches = (P.grid > 0 ? 1 : 0);
    unsigned char *skip = nullptr;
    if (P.grid > 0 && P.skip_flags) {   // segments no image may reach: flags at the current positions
        skip = reinterpret_cast<unsigned char *>(const_cast<char *>(d) + L.o_skip);
        if (!skip_ready) {   // (else written by room_beta_skip_kernel just before)
            CK(item_skip_launch(drooms, reinterpret_cast<const IsmItem *>(d + L.o_items), (int)P.items.size(),
                                dps, dpr, skip, st));
            if (record) s->last_launches += 1;
        }
    }
    if (P.grid > 0)
        CK(ism_forward_launch(P.tpl, drooms, reinterpret_cast<const IsmItem *>(d + L.o_items),
                              (int)P.items.size(), dps, dpr, dos, dor, dout, work_counter,
                              s->d_ctl + 1, P.em, P.nsub, P.clamp, P.grid, st, P.mode, P.tw, &ta,
                              reinterpret_cast<float4 *>(const_cast<char *>(d) + L.o_axis), P.axis_cap,
                              reinterpret_cast<float *>(const_cast<char *>(d) + L.o_part), skip));
    if (!P.groups.empty()) {   // RIRs split by images: add up their partial segments
        if (record) s->last_launches += 1;
        CK(partial_reduce_launch(reinterpret_cast<const PartGroup *>(d + L.o_groups), (int)P.groups.size(),
                                 P.max_part_len, reinterpret_cast<const float *>(d + L.o_part), dout, st));
    }
    if (record && s->ev_ism) CK(cudaEventRecord(s->ev[1], st));
    const bool tail_kernel = P.max_n_diff > 0 && (P.unfused_tails > 0 || P.grid == 0);
    if (record && s->profile && tail_kernel) { CK(cudaEventRecord(s->ev[2], st)); s->ev_tail = true; }
    if (record && tail_kernel) s->last_launches += 1;
    if (tail_kernel)
        CK(tail_launch(drooms, reinterpret_cast<const IsmItem *>(d + L.o_rirs), (int)M, P.max_n_diff,
                       dps, dpr, dout, s->seed, s->calls, offset_ptr, s->noise,
                       reinterpret_cast<float *>(const_cast<char *>(d) + L.o_env), st, tail_pre));
    if (record && s->ev_tail) CK(cudaEventRecord(s->ev[3], st));
    return GPURIR_OK;
}

// Device-usable address of a host output buffer, or nullptr when the kernels
// do not store to it (then the result is copied).  Pinned / registered memory
// has a mapped device address.  Pageable memory is copied into by default: a
// GPU that reads the host page tables (address translation services) can
// store into it, but pages not yet touched fault one by one from the GPU side,
// far slower than the copy.  GPURIR_HOST_DIRECT=0 turns direct stores off,
// =2 allows them into pageable memory as well.
static float *host_output_pointer(gpurir_sim *s, float *out, bool *pinned = nullptr) {
    if (pinned) *pinned = false;
    if (s->host_direct < 0) {
        const char *env = getenv("GPURIR_HOST_DIRECT");
        int pageable = 0, host_tables = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, s->device);
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, s->device);
        s->host_direct = (env && env[0] == '0') ? 0 : ((env && env[0] == '2' && pageable && host_tables) ? 2 : 1);
        cudaGetLastError();
    }
    if (s->host_direct == 0) return nullptr;
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, out) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (pa.type == cudaMemoryTypeHost && pa.devicePointer) {
        if (pinned) *pinned = true;
        return static_cast<float *>(pa.devicePointer);
    }
    if (pa.type == cudaMemoryTypeUnregistered && s->host_direct == 2) return out;
    return nullptr;
}

// True when the diffuse tail of the RIR (source ps, receiver pr) of room r is certainly
// silent: its envelope window [w_start, nISM) is empty, or no image of the pair can
// reach it (then every window sample is an exact zero and A = 0).  Conservative: the
// window start is taken one sample early, and images_miss_segment keeps a margin.
static bool tail_silent(const RoomDesc &r, const float *ps, const float *pr) {
    double d2 = 0.0;
    for (int a = 0; a < 3; a++) d2 += ((double)ps[a] - pr[a]) * ((double)ps[a] - pr[a]);
    const double tau_dp = std::sqrt(d2) * ((double)r.kh + r.kl);
    const double w = std::max((double)r.n_ism - 0.01 * r.fs, tau_dp);
    if (w - 1.0 >= (double)r.n_ism) return true;
    return images_miss_segment(r.L, r.nb, ps, pr, r.kh, r.H, (int)std::ceil(w) - 1, r.n_ism);
}

// Silent tails of a host-output call: flags per RIR into `flags` (the ISM kernel's
// epilogue, or the tail kernel for RIRs cut into segments, then writes only their
// envelope) and, on the side stream, one 2-D copy from a device zero buffer per run of
// consecutive rows, so that those bytes cross the host link while the ISM kernel
// computes the early parts.  Returns whether any tail was taken.
static int stream_silent_tails(gpurir_sim *s, const std::vector<RoomDesc> &R, const Plan &P,
                               const float *pos_src, const float *pos_rcv, float *out, unsigned char *flags,
                               bool &any) {
    any = false;
    const long M = (long)P.rirs.size();
    memset(flags, 0, (size_t)M);
    // Per room first: with every source and receiver inside the room, an image lies
    // within (N/2 + 1) L of the receiver on each axis, and every window starts at
    // nISM - 10 ms or later; when even that farthest delay stays clear of the earliest
    // window, all the room's tails are silent without a test per pair.
    std::vector<char> room_silent(R.size(), 0);
    for (size_t k = 0; k < R.size(); k++) {
        const RoomDesc &r = R[k];
        bool inside = true;
        for (int i = 0; i < r.n_src && inside; i++)
            for (int a = 0; a < 3; a++) {
                const float v = pos_src[3 * (r.src_off + i) + a];
                inside &= v >= 0.0f && v <= r.L[a];
            }
        for (int i = 0; i < r.n_rcv && inside; i++)
            for (int a = 0; a < 3; a++) {
                const float v = pos_rcv[3 * (r.rcv_off + i) + a];
                inside &= v >= 0.0f && v <= r.L[a];
            }
        if (!inside) continue;
        double reach2 = 0.0;
        for (int a = 0; a < 3; a++) {
            const double e = (double)(r.nb[a] / 2 + 1) * r.L[a];
            reach2 += e * e;
        }
        const double tau_hi = std::sqrt(reach2) * ((double)r.kh + r.kl);
        const double w_min = (double)r.n_ism - 0.01 * r.fs - 1.0;
        room_silent[k] = tau_hi < w_min - r.H - 2.0 - 1e-5 * tau_hi;
    }
    struct Run { long long row; long n; int room; };
    std::vector<Run> runs;
    size_t need = 0;
    for (long m = 0; m < M; m++) {
        const IsmItem &it = P.rirs[m];
        const RoomDesc &r = R[it.room];
        if (r.n_total <= r.n_ism) continue;   // no tail
        if (!room_silent[it.room] && !tail_silent(r, pos_src + 3 * it.src, pos_rcv + 3 * it.rcv)) continue;
        flags[it.rir] = 1;
        if (!runs.empty() && runs.back().room == it.room &&
            runs.back().row + runs.back().n * r.n_total == it.out_row)
            runs.back().n++;
        else
            runs.push_back({it.out_row, 1, it.room});
        need = std::max(need, (size_t)runs.back().n * (size_t)(r.n_total - r.n_ism) * sizeof(float));
    }
    if (runs.empty()) return GPURIR_OK;
    if (!s->side) {
        CK(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&s->side_done, cudaEventDisableTiming));
    }
    if (need > s->zero_bytes) {
        if (s->d_zero) {
            CK(cudaStreamSynchronize(s->side));
            CK(cudaFree(s->d_zero));
            s->d_zero = nullptr;
            s->zero_bytes = 0;
        }
        CK(cudaMalloc(&s->d_zero, need));
        CK(cudaMemsetAsync(s->d_zero, 0, need, s->side));
        s->zero_bytes = need;
    }
    for (const Run &u : runs) {
        const RoomDesc &r = R[u.room];
        const size_t width = (size_t)(r.n_total - r.n_ism) * sizeof(float);
        CK(cudaMemcpy2DAsync(out + u.row + r.n_ism, (size_t)r.n_total * sizeof(float), s->d_zero, width, width,
                             (size_t)u.n, cudaMemcpyDeviceToHost, s->side));
    }
    CK(cudaEventRecord(s->side_done, s->side));
    any = true;
    return GPURIR_OK;
}

// Shared body of the single-room and batched entry points, host or device I/O.
// Rooms carry their source/receiver/RIR/output offsets already.
static int simulate_rooms(gpurir_sim *s, std::vector<RoomDesc> &R, long n_src, long n_rcv,
                          const float *pos_src, const float *pos_rcv, const float *orV_src,
                          const float *orV_rcv, float *out, long long out_elems, bool host_io,
                          cudaStream_t st, const float *d_beta = nullptr) {
    int rc;
    for (RoomDesc &r : R) r.ref_delay = s->ref_delay;
    std::vector<double> key = plan_key(s, R, host_io, out_elems);
    const bool hit = s->pcache && s->pcache->key == key;
    if (!hit) {
        if (!s->pcache) s->pcache = new PlanCache();
        s->pcache->key.clear();   // invalid until planned
        s->pcache->gen = ~0ull;
        if ((rc = plan_rooms(s, R, s->pcache->P))) return rc;
        s->pcache->key = std::move(key);
    }
    const Plan &P = s->pcache->P;
    const long M = (long)P.rirs.size();
    if (!hit) s->pcache->L = make_layout(P, R.size(), n_src, n_rcv, M, out_elems, host_io);
    const Layout &L = s->pcache->L;
    if ((rc = ensure_device(s, L.dev_bytes))) return rc;
    if ((rc = ensure_stage(s, L.stage_bytes))) return rc;
    // the items of an unchanged plan are still on the device unless something else
    // was uploaded there since: then only the rooms and positions go up
    const bool items_resident = hit && s->pcache->gen == s->ws_gen;
    const size_t up_bytes = items_resident ? L.o_items : L.stage_bytes;
    char *h = s->h_stage;
    if (items_resident) memcpy(h + L.o_rooms, R.data(), R.size() * sizeof(RoomDesc));
    else fill_stage(h, L, R, P);
    const float *dps = pos_src, *dpr = pos_rcv, *dos = orV_src, *dor = orV_rcv;
    char *d = s->d_ws;
    // Host output the GPU can store to directly (pinned memory, or any host memory on
    // systems whose GPU shares the CPU's page tables, e.g. over NVLink-C2C): the kernels
    // write the RIRs there during compute and no device->host copy follows.
    bool direct = false, pinned = false;
    float *hout = nullptr;
    if (host_io) {
        hout = host_output_pointer(s, out, &pinned);
        direct = hout != nullptr;
    }
    // ... and, into page-locked memory, tails silent by geometry are streamed by a copy
    // engine meanwhile
    bool pre = false;
    if (host_io && pinned && P.grid > 0 && P.max_n_diff > 0)
        if ((rc = stream_silent_tails(s, R, P, pos_src, pos_rcv, out,
                                      reinterpret_cast<unsigned char *>(h + L.o_pre), pre)))
            return rc;
    if (host_io) {
        float *hp = reinterpret_cast<float *>(h + L.o_pos);
        memcpy(hp, pos_src, sizeof(float) * 3 * n_src);
        memcpy(hp + 3 * n_src, pos_rcv, sizeof(float) * 3 * n_rcv);
        if (orV_src) memcpy(hp + 3 * (n_src + n_rcv), orV_src, sizeof(float) * 3 * n_src);
        else memset(hp + 3 * (n_src + n_rcv), 0, sizeof(float) * 3 * n_src);
        if (orV_rcv) memcpy(hp + 3 * (2 * n_src + n_rcv), orV_rcv, sizeof(float) * 3 * n_rcv);
        else memset(hp + 3 * (2 * n_src + n_rcv), 0, sizeof(float) * 3 * n_rcv);
        float *dp = reinterpret_cast<float *>(d + L.o_pos);
        dps = dp; dpr = dp + 3 * n_src; dos = dp + 3 * (n_src + n_rcv); dor = dp + 3 * (2 * n_src + n_rcv);
    }
    if (s->ws_recorded) CK(cudaStreamWaitEvent(st, s->ws_busy, 0));   // earlier calls, any stream
    CK(cudaMemcpyAsync(d, h, up_bytes, cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(s->stage_done, st));
    s->stage_pending = true;
    if (!items_resident) s->pcache->gen = ++s->ws_gen;
    if (d_beta) CK(room_beta_launch(reinterpret_cast<RoomDesc *>(d + L.o_rooms), (int)R.size(), d_beta, st));
    float *dout = host_io ? (direct ? hout : reinterpret_cast<float *>(d + L.o_out)) : out;
    s->last_direct = direct;
    s->ev_ism = s->ev_tail = false;
    s->last_h2d = up_bytes;
    s->last_d2h = sizeof(int) + (host_io ? (uint64_t)out_elems * sizeof(float) : 0);
    if ((rc = enqueue_kernels(s, P, d, L, M, dps, dpr, dos, dor, dout, s->d_ctl, nullptr, st, true, false,
                              pre ? reinterpret_cast<const unsigned char *>(d + L.o_pre) : nullptr)))
        return rc;
    if (pre) CK(cudaStreamWaitEvent(st, s->side_done, 0));   // the call ends after the streamed tails
    s->env_off = L.o_env;
    s->last_n_rir = P.max_n_diff > 0 ? M : 0;
    s->calls++;
    CK(cudaMemcpyAsync(s->h_ctl + 1, s->d_ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (host_io && !direct)
        CK(cudaMemcpyAsync(out, dout, (size_t)out_elems * sizeof(float), cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(s->ws_busy, st));
    s->ws_recorded = true;
    if (host_io) {
        CK(cudaStreamSynchronize(st));
        return check_status(s);
    }
    return GPURIR_OK;
}

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
    std::vector<RoomDesc> R(1);
    int rc = build_room(R[0], room_sz, beta, nb_img, Tdiff, Tmax, Fs, c, spkr, mic);
    if (rc) return rc;
    R[0].n_src = M_src; R[0].n_rcv = M_rcv;
    return simulate_rooms(s, R, M_src, M_rcv, pos_src, pos_rcv, orV_src, orV_rcv, out,
                          (long long)M_src * M_rcv * R[0].n_total, host_io, st);
}

// Room table of a batch: offsets of sources, receivers, RIRs and output rows.
static int build_batch(int n_rooms, const gpurir_room *rooms, float Fs, float c,
                       std::vector<RoomDesc> &R, long &n_src, long &n_rcv, long long &out_elems) {
    if (n_rooms < 1 || !rooms) return fail(GPURIR_ERR_INVALID, "need at least one room");
    R.assign(n_rooms, RoomDesc{});
    n_src = n_rcv = 0;
    out_elems = 0;
    long n_rir = 0;
    for (int i = 0; i < n_rooms; i++) {
        const gpurir_room &g = rooms[i];
        if (g.n_src < 1 || g.n_rcv < 1)
            return fail(GPURIR_ERR_INVALID, "room " + std::to_string(i) + ": need a source and a receiver");
        int rc = build_room(R[i], g.room_sz, g.beta, g.nb_img, g.Tdiff, g.Tmax, Fs, c,
                            g.spkr_pattern, g.mic_pattern);
        if (rc) return fail(rc, "room " + std::to_string(i) + ": " + g_err);
        R[i].n_src = g.n_src;
        R[i].n_rcv = g.n_rcv;
        R[i].src_off = (int)n_src;
        R[i].rcv_off = (int)n_rcv;
        R[i].rir_off = (int)n_rir;
        R[i].out_off = out_elems;
        n_src += g.n_src;
        n_rcv += g.n_rcv;
        n_rir += (long)g.n_src * g.n_rcv;
        out_elems += (long long)g.n_src * g.n_rcv * R[i].n_total;
        if (n_rir > (1L << 30) || n_src > (1L << 30) || n_rcv > (1L << 30))
            return fail(GPURIR_ERR_INVALID, "batch too large");
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

extern "C" int gpurir_last_launch_count(gpurir_sim *s, int *kernels) {
    if (!s || !kernels) return fail(GPURIR_ERR_INVALID, "NULL argument");
    *kernels = s->last_launches;
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

extern "C" int gpurir_batch_layout(int n_rooms, const gpurir_room *rooms, float Fs,
                                   long long *rir_offsets) {
    if (!rir_offsets) return fail(GPURIR_ERR_INVALID, "NULL argument");
    std::vector<RoomDesc> R;
    long ns, nr;
    long long tot;
    int rc = build_batch(n_rooms, rooms, Fs, 343.0f, R, ns, nr, tot);
    if (rc) return rc;
    for (int i = 0; i < n_rooms; i++) rir_offsets[i] = R[i].out_off;
    rir_offsets[n_rooms] = tot;
    return GPURIR_OK;
}

static int batch_device(gpurir_sim *s, int n_rooms, const gpurir_room *rooms, float Fs, float c,
                        const float *d_beta, const float *d_pos_src, const float *d_pos_rcv,
                        const float *d_orV_src, const float *d_orV_rcv, float *d_out, void *stream);

extern "C" int gpurir_simulate_batch_device(gpurir_sim *s, int n_rooms, const gpurir_room *rooms,
                                            float Fs, float c, const float *d_pos_src,
                                            const float *d_pos_rcv, const float *d_orV_src,
                                            const float *d_orV_rcv, float *d_out, void *stream) {
    return batch_device(s, n_rooms, rooms, Fs, c, nullptr, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv,
                        d_out, stream);
}

extern "C" int gpurir_simulate_batch_device_beta(gpurir_sim *s, int n_rooms, const gpurir_room *rooms,
                                                 float Fs, float c, const float *d_beta,
                                                 const float *d_pos_src, const float *d_pos_rcv,
                                                 const float *d_orV_src, const float *d_orV_rcv,
                                                 float *d_out, void *stream) {
    if (!d_beta) return fail(GPURIR_ERR_INVALID, "NULL d_beta");
    return batch_device(s, n_rooms, rooms, Fs, c, d_beta, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv,
                        d_out, stream);
}

static int batch_device(gpurir_sim *s, int n_rooms, const gpurir_room *rooms, float Fs, float c,
                        const float *d_beta, const float *d_pos_src, const float *d_pos_rcv,
                        const float *d_orV_src, const float *d_orV_rcv, float *d_out, void *stream) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (!d_pos_src || !d_pos_rcv || !d_out) return fail(GPURIR_ERR_INVALID, "NULL argument");
    std::vector<RoomDesc> R;
    long ns, nr;
    long long tot;
    int rc = build_batch(n_rooms, rooms, Fs, c, R, ns, nr, tot);
    if (rc) return rc;
    for (int i = 0; i < n_rooms; i++)
        if ((R[i].spkr != 0 && !d_orV_src) || (R[i].mic != 0 && !d_orV_rcv))
            return fail(GPURIR_ERR_INVALID, "orientation required for a non-omni pattern");
    return simulate_rooms(s, R, ns, nr, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv, d_out, tot, false,
                          reinterpret_cast<cudaStream_t>(stream), d_beta);
}

// ---------------------------------------------------------------------------
// Captured batch: descriptors uploaded once, the launch sequence recorded in a
// CUDA graph and replayed.  Positions and orientations are read from the same
// device buffers at every replay, so callers may update them in place.
// ---------------------------------------------------------------------------
struct gpurir_batch {
    gpurir_sim *sim = nullptr;
    char *d = nullptr;            // descriptors + envelope + work counter + call offset
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long n_rir = 0;
    long long out_elems = 0;
};

namespace gpurir {
cudaError_t advance_counter_launch(uint64_t *counter, cudaStream_t st);
}

extern "C" int gpurir_batch_create(gpurir_sim *s, int n_rooms, const gpurir_room *rooms, float Fs,
                                   float c, const float *d_pos_src, const float *d_pos_rcv,
                                   const float *d_orV_src, const float *d_orV_rcv, float *d_out,
                                   gpurir_batch **out) {
    if (!s || !out) return fail(GPURIR_ERR_INVALID, "NULL argument");
    *out = nullptr;
    std::vector<RoomDesc> R;
    long ns, nr;
    long long tot;
    int rc = build_batch(n_rooms, rooms, Fs, c, R, ns, nr, tot);
    if (rc) return rc;
    for (RoomDesc &r : R) r.ref_delay = s->ref_delay;
    Plan P;
    if ((rc = plan_rooms(s, R, P))) return rc;
    const long M = (long)P.rirs.size();
    Layout L = make_layout(P, R.size(), ns, nr, M, tot, false);
    const size_t o_ctl = align_up(L.o_out, 256);           // work counter, then the call offset
    const size_t bytes = o_ctl + 256;
    std::vector<char> h(L.stage_bytes);
    fill_stage(h.data(), L, R, P);
    gpurir_batch *b = new gpurir_batch();
    b->sim = s;
    b->n_rir = M;
    b->out_elems = tot;
    cudaStream_t cap = nullptr;
    cudaError_t e = cudaMalloc(&b->d, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(b->d, h.data(), L.stage_bytes, cudaMemcpyHostToDevice);
    uint64_t start = s->calls;
    if (e == cudaSuccess) e = cudaMemcpy(b->d + o_ctl + 8, &start, sizeof(start), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        if (cap) cudaStreamDestroy(cap);
        gpurir_batch_destroy(b);
        return fail(GPURIR_ERR_CUDA, std::string("gpurir_batch_create: ") + cudaGetErrorString(e));
    }
    int *counter = reinterpret_cast<int *>(b->d + o_ctl);
    uint64_t *offset = reinterpret_cast<uint64_t *>(b->d + o_ctl + 8);
    e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        rc = enqueue_kernels(s, P, b->d, L, M, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv, d_out,
                             counter, offset, cap, false);
        if (rc == GPURIR_OK && P.max_n_diff > 0) {
            cudaError_t e2 = advance_counter_launch(offset, cap);   // next replay draws new noise
            if (e2 != cudaSuccess) rc = fail(GPURIR_ERR_CUDA, cudaGetErrorString(e2));
        }
        cudaError_t e3 = cudaStreamEndCapture(cap, &b->graph);
        if (rc == GPURIR_OK && e3 != cudaSuccess) rc = fail(GPURIR_ERR_CUDA, cudaGetErrorString(e3));
    } else {
        rc = fail(GPURIR_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaStreamDestroy(cap);
    if (rc == GPURIR_OK) {
        e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        if (e != cudaSuccess) rc = fail(GPURIR_ERR_CUDA, std::string("graph: ") + cudaGetErrorString(e));
    }
    if (rc != GPURIR_OK) {
        gpurir_batch_destroy(b);
        return rc;
    }
    *out = b;
    return GPURIR_OK;
}

extern "C" int gpurir_batch_launch(gpurir_batch *b, void *stream) {
    if (!b || !b->exec) return fail(GPURIR_ERR_INVALID, "NULL batch");
    CK(cudaGraphLaunch(b->exec, reinterpret_cast<cudaStream_t>(stream)));
    return GPURIR_OK;
}

extern "C" int gpurir_batch_info(gpurir_batch *b, long long *n_rir, long long *out_elems) {
    if (!b) return fail(GPURIR_ERR_INVALID, "NULL batch");
    if (n_rir) *n_rir = b->n_rir;
    if (out_elems) *out_elems = b->out_elems;
    return GPURIR_OK;
}

extern "C" int gpurir_batch_destroy(gpurir_batch *b) {
    if (!b) return GPURIR_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d) {
        cudaDeviceSynchronize();
        cudaFree(b->d);
    }
    delete b;
    return GPURIR_OK;
}

extern "C" int gpurir_device_status(gpurir_sim *s) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    int v = 0;
    CK(cudaMemcpy(&v, s->d_ctl + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (v != 0) {
        CK(cudaMemset(s->d_ctl + 1, 0, sizeof(int)));
        return fail(GPURIR_ERR_DEVICE, "kernel rejected a work item (code " + std::to_string(v) + ")");
    }
    return GPURIR_OK;
}

// ---------------------------------------------------------------------------
// Adjoint
// ---------------------------------------------------------------------------
static void csr(const std::vector<IsmItem> &items, int n_target, int IsmItem::*field, int base_sub,
                std::vector<int> &ptr, std::vector<int> &list) {
    ptr.assign(n_target + 1, 0);
    for (const IsmItem &it : items) ptr[it.*field - base_sub + 1]++;
    for (int t = 0; t < n_target; t++) ptr[t + 1] += ptr[t];
    list.assign(items.size(), 0);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (size_t i = 0; i < items.size(); i++) list[fill[items[i].*field - base_sub]++] = (int)i;
}

// Adjoint work items: the forward's, in the same order, except that the items of an
// incomplete last wave of G blocks (all of them when there is only one) are cut by
// images into up to 8 parts, as many as fill the wave.  The adjoint's items of one
// batch cost about the same, so whole items would leave that wave mostly idle; the
// parts fill it (each part restages its segment of dL/dh, which is why the full waves
// stay whole).  On the inverse problem (512 items, 456 blocks) the adjoint takes ~66 us
// instead of ~76 us; cutting every item in two gave ~70 us, in three ~78 us.  Items past
// every image's delay stay whole (they only test and leave) and go last.
static std::vector<IsmItem> adjoint_items(const Plan &P, const std::vector<RoomDesc> &R, long G) {
    G = std::max<long>(G, 1);
    std::vector<IsmItem> real, bitems, empties;
    for (const IsmItem &it : P.items) {
        const bool empty = it.t_lo > 0 && it.t_lo >= room_span(R[it.room]);
        (empty ? empties : real).push_back(it);
    }
    const long n_real = (long)real.size();
    const long rem = n_real % G;   // items of the last, incomplete wave
    for (long i = 0; i < n_real; i++) {
        const IsmItem &it = real[i];
        const int n = it.i_hi - it.i_lo;
        int parts = 1;
        if (rem > 0 && i >= n_real - rem) parts = (int)std::max<long>(2, std::min<long>(8, G / rem));
        parts = std::min(parts, std::max(n, 1));
        for (int k = 0; k < parts; k++) {
            IsmItem h = it;
            h.i_lo = it.i_lo + (int)((long long)n * k / parts);
            h.i_hi = it.i_lo + (int)((long long)n * (k + 1) / parts);
            bitems.push_back(h);
        }
    }
    bitems.insert(bitems.end(), empties.begin(), empties.end());
    return bitems;
}

static int backward_batch(gpurir_sim *s, int n_rooms, const gpurir_room *rooms, float Fs, float c,
                          const float *d_beta, const float *d_pos_src, const float *d_pos_rcv,
                          const float *d_orV_src, const float *d_orV_rcv, const float *d_grad_rir,
                          float *d_grad_beta, float *d_grad_pos_src, float *d_grad_pos_rcv,
                          float *d_grad_orV_src, float *d_grad_orV_rcv, void *stream);

extern "C" int gpurir_ism_backward_batch_device(gpurir_sim *s, int n_rooms, const gpurir_room *rooms,
                                                float Fs, float c, const float *d_pos_src,
                                                const float *d_pos_rcv, const float *d_orV_src,
                                                const float *d_orV_rcv, const float *d_grad_rir,
                                                float *d_grad_beta, float *d_grad_pos_src,
                                                float *d_grad_pos_rcv, float *d_grad_orV_src,
                                                float *d_grad_orV_rcv, void *stream) {
    return backward_batch(s, n_rooms, rooms, Fs, c, nullptr, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv,
                          d_grad_rir, d_grad_beta, d_grad_pos_src, d_grad_pos_rcv, d_grad_orV_src,
                          d_grad_orV_rcv, stream);
}

extern "C" int gpurir_ism_backward_batch_device_beta(gpurir_sim *s, int n_rooms, const gpurir_room *rooms,
                                                     float Fs, float c, const float *d_beta,
                                                     const float *d_pos_src, const float *d_pos_rcv,
                                                     const float *d_orV_src, const float *d_orV_rcv,
                                                     const float *d_grad_rir, float *d_grad_beta,
                                                     float *d_grad_pos_src, float *d_grad_pos_rcv,
                                                     float *d_grad_orV_src, float *d_grad_orV_rcv,
                                                     void *stream) {
    if (!d_beta) return fail(GPURIR_ERR_INVALID, "NULL d_beta");
    return backward_batch(s, n_rooms, rooms, Fs, c, d_beta, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv,
                          d_grad_rir, d_grad_beta, d_grad_pos_src, d_grad_pos_rcv, d_grad_orV_src,
                          d_grad_orV_rcv, stream);
}

static int backward_batch(gpurir_sim *s, int n_rooms, const gpurir_room *rooms, float Fs, float c,
                          const float *d_beta, const float *d_pos_src, const float *d_pos_rcv,
                          const float *d_orV_src, const float *d_orV_rcv, const float *d_grad_rir,
                          float *d_grad_beta, float *d_grad_pos_src, float *d_grad_pos_rcv,
                          float *d_grad_orV_src, float *d_grad_orV_rcv, void *stream) {
    if (!s) return fail(GPURIR_ERR_INVALID, "NULL handle");
    if (!d_pos_src || !d_pos_rcv || !d_grad_rir) return fail(GPURIR_ERR_INVALID, "NULL argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    std::vector<RoomDesc> R;
    long ns, nr;
    long long tot;
    int rc = build_batch(n_rooms, rooms, Fs, c, R, ns, nr, tot);
    if (rc) return rc;
    for (int i = 0; i < n_rooms; i++)
        if ((R[i].spkr != 0 && !d_orV_src) || (R[i].mic != 0 && !d_orV_rcv))
            return fail(GPURIR_ERR_INVALID, "orientation required for a non-omni pattern");
    Plan P;
    if ((rc = plan_rooms(s, R, P))) return rc;
    int max_tseg = 1;
    for (const IsmItem &it : P.items) max_tseg = std::max(max_tseg, it.t_hi - it.t_lo);
    const int pad = 64 * P.tpl;
    const size_t smem = ism_backward_smem_bytes(P.tpl, max_tseg, pad, P.axis_cap);
    int bps = 0;
    if (!P.items.empty()) {
        if (smem > 227 * 1024) return fail(GPURIR_ERR_UNSUPPORTED, "segment too long for the adjoint");
        bps = ism_backward_blocks_per_sm(P.tpl, P.clamp, smem);
        if (bps < 1) return fail(GPURIR_ERR_CUDA, "adjoint kernel does not fit on an SM");
    }
    // work items split as the training batch splits them (gpurir_adjoint_create)
    const std::vector<IsmItem> bi = adjoint_items(P, R, (long)s->num_sms * bps);
    if (!P.items.empty() && tuning(2) > 0) bps = std::min(bps, tuning(2));   // adjoint_blocks_per_sm (tuning.cu)
    const int n_items = (int)bi.size();
    std::vector<int> p_room, l_room, p_src, l_src, p_rcv, l_rcv;
    csr(bi, n_rooms, &IsmItem::room, 0, p_room, l_room);
    csr(bi, (int)ns, &IsmItem::src, 0, p_src, l_src);
    csr(bi, (int)nr, &IsmItem::rcv, 0, p_rcv, l_rcv);
    // staging: rooms | items | csr arrays ; device adds item partials
    size_t o_rooms = 0;
    size_t o_items = align_up(R.size() * sizeof(RoomDesc), 256);
    size_t o_csr = align_up(o_items + bi.size() * sizeof(IsmItem), 256);
    const std::vector<int> *arrs[6] = {&p_room, &l_room, &p_src, &l_src, &p_rcv, &l_rcv};
    size_t o_arr[6], off = o_csr;
    for (int a = 0; a < 6; a++) { o_arr[a] = off; off = align_up(off + arrs[a]->size() * sizeof(int), 256); }
    const size_t stage_bytes = off;
    const size_t o_ig = stage_bytes;
    const size_t dev_bytes = align_up(o_ig + (size_t)std::max(n_items, 1) * 18 * sizeof(float), 256);
    if ((rc = ensure_device(s, dev_bytes))) return rc;
    if ((rc = ensure_stage(s, stage_bytes))) return rc;
    char *h = s->h_stage;
    memcpy(h + o_rooms, R.data(), R.size() * sizeof(RoomDesc));
    if (n_items) memcpy(h + o_items, bi.data(), bi.size() * sizeof(IsmItem));
    for (int a = 0; a < 6; a++)
        if (!arrs[a]->empty()) memcpy(h + o_arr[a], arrs[a]->data(), arrs[a]->size() * sizeof(int));
    char *d = s->d_ws;
    if (s->ws_recorded) CK(cudaStreamWaitEvent(st, s->ws_busy, 0));
    CK(cudaMemcpyAsync(d, h, stage_bytes, cudaMemcpyHostToDevice, st));
    s->ws_gen++;   // the cached plan's items were overwritten
    CK(cudaEventRecord(s->stage_done, st));
    s->stage_pending = true;
    if (d_beta) CK(room_beta_launch(reinterpret_cast<RoomDesc *>(d + o_rooms), n_rooms, d_beta, st));
    float *ig = reinterpret_cast<float *>(d + o_ig);
    if (n_items == 0) {
        CK(cudaMemsetAsync(ig, 0, 18 * sizeof(float), st));
    } else {
        const int grid = std::min(n_items, s->num_sms * bps);
        CK(ism_backward_launch(P.tpl, reinterpret_cast<const RoomDesc *>(d + o_rooms),
                               reinterpret_cast<const IsmItem *>(d + o_items), n_items, d_pos_src,
                               d_pos_rcv, d_orV_src, d_orV_rcv, d_grad_rir, ig, s->d_ctl, s->d_ctl + 1,
                               max_tseg, P.axis_cap, grid, P.clamp, st));
    }
    const int *dp[6];
    for (int a = 0; a < 6; a++) dp[a] = reinterpret_cast<const int *>(d + o_arr[a]);
    float *const outs[5] = {d_grad_beta, d_grad_pos_src, d_grad_pos_rcv, d_grad_orV_src, d_grad_orV_rcv};
    CK(grad_reduce_launch(ig, dp, n_rooms, (int)ns, (int)nr, outs, st));
    CK(cudaEventRecord(s->ws_busy, st));
    s->ws_recorded = true;
    return GPURIR_OK;
}

// ---------------------------------------------------------------------------
// Training-loop batch: descriptors, work items and gradient lists uploaded once;
// the forward and the adjoint then only enqueue kernels (no host work, no
// synchronisation), so a whole step can be recorded in a CUDA graph.
// ---------------------------------------------------------------------------
struct gpurir_adjoint {
    gpurir_sim *sim = nullptr;
    char *d = nullptr;
    Plan P;
    Layout L;
    int n_rooms = 0;
    long ns = 0, nr = 0, M = 0;
    long long out_elems = 0;
    int max_tseg = 1, grid_b = 0;
    bool need_orv_src = false, need_orv_rcv = false;
    bool rooms_written = false;   // a forward call has written the room tables
    size_t o_arr[6] = {}, o_ig = 0, o_bitems = 0, o_ctl = 0;
    int n_bitems = 0;             // adjoint work items (the forward's, split; see gpurir_adjoint_create)
    float *d_g = nullptr;         // dL/dRIR of the fused L2 step (allocated by its first call)
    double *d_partial = nullptr;  // per-block partial sums of the loss
};

extern "C" int gpurir_adjoint_destroy(gpurir_adjoint *a) {
    if (!a) return GPURIR_OK;
    if (a->d_g || a->d_partial) cudaDeviceSynchronize();
    if (a->d) cudaFree(a->d);
    if (a->d_g) cudaFree(a->d_g);
    if (a->d_partial) cudaFree(a->d_partial);
    delete a;
    return GPURIR_OK;
}

extern "C" int gpurir_adjoint_create(gpurir_sim *s, int n_rooms, const gpurir_room *rooms, float Fs,
                                     float c, gpurir_adjoint **out) {
    if (!s || !out) return fail(GPURIR_ERR_INVALID, "NULL argument");
    *out = nullptr;
    gpurir_adjoint *a = new gpurir_adjoint();
    a->sim = s;
    a->n_rooms = n_rooms;
    std::vector<RoomDesc> R;
    int rc = build_batch(n_rooms, rooms, Fs, c, R, a->ns, a->nr, a->out_elems);
    if (rc == GPURIR_OK) rc = plan_rooms(s, R, a->P);
    if (rc) { delete a; return rc; }
    for (const RoomDesc &r : R) {
        a->need_orv_src |= r.spkr != 0;
        a->need_orv_rcv |= r.mic != 0;
    }
    const Plan &P = a->P;
    a->M = (long)P.rirs.size();
    a->L = make_layout(P, R.size(), a->ns, a->nr, a->M, a->out_elems, false);
    for (const IsmItem &it : P.items) a->max_tseg = std::max(a->max_tseg, it.t_hi - it.t_lo);
    if (!P.items.empty() && ism_backward_smem_bytes(P.tpl, a->max_tseg, 64 * P.tpl, P.axis_cap) > 227 * 1024) {
        delete a;
        return fail(GPURIR_ERR_UNSUPPORTED, "segment too long for the adjoint");
    }
    int bps = 0, bps_occ = 0;
    if (!P.items.empty()) {
        bps = ism_backward_blocks_per_sm(P.tpl, P.clamp, ism_backward_smem_bytes(P.tpl, a->max_tseg, 64 * P.tpl,
                                                                                P.axis_cap));
        if (bps < 1) {
            delete a;
            return fail(GPURIR_ERR_CUDA, "adjoint kernel does not fit on an SM");
        }
        bps_occ = bps;
        if (tuning(2) > 0) bps = std::min(bps, tuning(2));   // adjoint_blocks_per_sm (tuning.cu)
    }
    // (the wave of the occupancy limit, not of a tuned grid: the items, and so the bits
    // of the gradients, do not depend on the launch-shape knob)
    const std::vector<IsmItem> bitems = adjoint_items(P, R, (long)s->num_sms * bps_occ);
    const int n_items = (int)bitems.size();
    a->n_bitems = n_items;
    a->grid_b = std::min(n_items, s->num_sms * bps);
    std::vector<int> lists[6];
    csr(bitems, n_rooms, &IsmItem::room, 0, lists[0], lists[1]);
    csr(bitems, (int)a->ns, &IsmItem::src, 0, lists[2], lists[3]);
    csr(bitems, (int)a->nr, &IsmItem::rcv, 0, lists[4], lists[5]);
    size_t off = align_up(a->L.o_out, 256);
    for (int k = 0; k < 6; k++) { a->o_arr[k] = off; off = align_up(off + lists[k].size() * sizeof(int), 256); }
    a->o_ig = off;
    a->o_bitems = align_up(a->o_ig + (size_t)std::max(n_items, 1) * 18 * sizeof(float), 256);
    a->o_ctl = align_up(a->o_bitems + bitems.size() * sizeof(IsmItem), 256);
    const size_t bytes = a->o_ctl + 256;   // [0] forward counter, [1] adjoint counter, [2] status, +16 call offset
    std::vector<char> h(a->o_ctl + 256, 0);
    fill_stage(h.data(), a->L, R, P);
    for (int k = 0; k < 6; k++)
        if (!lists[k].empty()) memcpy(h.data() + a->o_arr[k], lists[k].data(), lists[k].size() * sizeof(int));
    if (!bitems.empty()) memcpy(h.data() + a->o_bitems, bitems.data(), bitems.size() * sizeof(IsmItem));
    const uint64_t start = s->calls;
    memcpy(h.data() + a->o_ctl + 16, &start, sizeof(start));
    cudaError_t e = cudaMalloc(&a->d, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(a->d, h.data(), bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        gpurir_adjoint_destroy(a);
        return fail(GPURIR_ERR_CUDA, std::string("gpurir_adjoint_create: ") + cudaGetErrorString(e));
    }
    *out = a;
    return GPURIR_OK;
}

extern "C" int gpurir_adjoint_forward(gpurir_adjoint *a, const float *d_beta, const float *d_pos_src,
                                      const float *d_pos_rcv, const float *d_orV_src,
                                      const float *d_orV_rcv, float *d_out, void *stream) {
    if (!a || !d_beta || !d_pos_src || !d_pos_rcv || !d_out) return fail(GPURIR_ERR_INVALID, "NULL argument");
    if ((a->need_orv_src && !d_orV_src) || (a->need_orv_rcv && !d_orV_rcv))
        return fail(GPURIR_ERR_INVALID, "orientation required for a non-omni pattern");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int *ctl = reinterpret_cast<int *>(a->d + a->o_ctl);
    uint64_t *offset = reinterpret_cast<uint64_t *>(a->d + a->o_ctl + 16);
    const bool fuse_skip = a->P.grid > 0 && a->P.skip_flags;
    if (fuse_skip)   // room tables and the items' skip flags in one launch
        CK(room_beta_skip_launch(reinterpret_cast<RoomDesc *>(a->d + a->L.o_rooms), a->n_rooms, d_beta,
                                 reinterpret_cast<const IsmItem *>(a->d + a->L.o_items), (int)a->P.items.size(),
                                 d_pos_src, d_pos_rcv, reinterpret_cast<unsigned char *>(a->d + a->L.o_skip), st));
    else
        CK(room_beta_launch(reinterpret_cast<RoomDesc *>(a->d + a->L.o_rooms), a->n_rooms, d_beta, st));
    a->rooms_written = true;
    int rc = enqueue_kernels(a->sim, a->P, a->d, a->L, a->M, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv,
                             d_out, ctl, offset, st, false, fuse_skip);
    if (rc) return rc;
    if (a->P.max_n_diff > 0) CK(advance_counter_launch(offset, st));   // the next call draws new noise
    return GPURIR_OK;
}

extern "C" int gpurir_adjoint_backward(gpurir_adjoint *a, const float *d_beta, const float *d_pos_src,
                                       const float *d_pos_rcv, const float *d_orV_src,
                                       const float *d_orV_rcv, const float *d_grad_rir, float *d_grad_beta,
                                       float *d_grad_pos_src, float *d_grad_pos_rcv, float *d_grad_orV_src,
                                       float *d_grad_orV_rcv, void *stream) {
    if (!a || !d_pos_src || !d_pos_rcv || !d_grad_rir) return fail(GPURIR_ERR_INVALID, "NULL argument");
    if (!d_beta && !a->rooms_written)
        return fail(GPURIR_ERR_INVALID, "d_beta is NULL but no forward call has written the room tables");
    if ((a->need_orv_src && !d_orV_src) || (a->need_orv_rcv && !d_orV_rcv))
        return fail(GPURIR_ERR_INVALID, "orientation required for a non-omni pattern");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int *ctl = reinterpret_cast<int *>(a->d + a->o_ctl);
    const Plan &P = a->P;
    const int n_items = a->n_bitems;
    float *ig = reinterpret_cast<float *>(a->d + a->o_ig);
    const RoomDesc *drooms = reinterpret_cast<const RoomDesc *>(a->d + a->L.o_rooms);
    if (d_beta) CK(room_beta_launch(reinterpret_cast<RoomDesc *>(a->d + a->L.o_rooms), a->n_rooms, d_beta, st));
    if (n_items == 0) {
        CK(cudaMemsetAsync(ig, 0, 18 * sizeof(float), st));
    } else {
        CK(ism_backward_launch(P.tpl, drooms, reinterpret_cast<const IsmItem *>(a->d + a->o_bitems), n_items,
                               d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv, d_grad_rir, ig, ctl + 1, ctl + 2,
                               a->max_tseg, P.axis_cap, a->grid_b, P.clamp, st));
    }
    const int *dp[6];
    for (int k = 0; k < 6; k++) dp[k] = reinterpret_cast<const int *>(a->d + a->o_arr[k]);
    float *const outs[5] = {d_grad_beta, d_grad_pos_src, d_grad_pos_rcv, d_grad_orV_src, d_grad_orV_rcv};
    CK(grad_reduce_launch(ig, dp, a->n_rooms, (int)a->ns, (int)a->nr, outs, st));
    return GPURIR_OK;
}

extern "C" int gpurir_adjoint_l2_step(gpurir_adjoint *a, const float *d_beta, const float *d_pos_src,
                                      const float *d_pos_rcv, const float *d_orV_src, const float *d_orV_rcv,
                                      const float *d_target, float scale, float *d_out, float *d_loss,
                                      float *d_grad_beta, float *d_grad_pos_src, float *d_grad_pos_rcv,
                                      float *d_grad_orV_src, float *d_grad_orV_rcv, void *stream) {
    if (!a || !d_target || !d_out || !d_loss) return fail(GPURIR_ERR_INVALID, "NULL argument");
    if ((reinterpret_cast<uintptr_t>(d_target) | reinterpret_cast<uintptr_t>(d_out)) & 15)
        return fail(GPURIR_ERR_INVALID, "d_target and d_out must be 16-byte aligned");
    if (!a->d_g) {   // first call: the gradient buffer and the loss partials
        CK(cudaMalloc(&a->d_g, sizeof(float) * std::max<long long>(a->out_elems, 4)));
        CK(cudaMalloc(&a->d_partial, sizeof(double) * 1024));
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int rc = gpurir_adjoint_forward(a, d_beta, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv, d_out, stream);
    if (rc) return rc;
    CK(l2_grad_launch(d_out, d_target, (long)a->out_elems, scale, a->d_g, a->d_partial, d_loss, st));
    // the room tables of the forward just enqueued serve the adjoint (same beta)
    return gpurir_adjoint_backward(a, nullptr, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv, a->d_g, d_grad_beta,
                                   d_grad_pos_src, d_grad_pos_rcv, d_grad_orV_src, d_grad_orV_rcv, stream);
}

extern "C" int gpurir_adjoint_status(gpurir_adjoint *a, int *status) {
    if (!a || !status) return fail(GPURIR_ERR_INVALID, "NULL argument");
    CK(cudaMemcpy(status, a->d + a->o_ctl + 2 * sizeof(int), sizeof(int), cudaMemcpyDeviceToHost));
    return GPURIR_OK;
}

// ---------------------------------------------------------------------------
// Convolution of trajectory segments with their RIRs (cuda_convolutions,
// src/gpuRIR_cuda.cu:933-1023) and the overlap-add of simulateTrajectory.
// ---------------------------------------------------------------------------
static const int kFftMaxN = 1 << 24;

static int fft_size(long n) {   // pow2roundup of gpuRIR (src/gpuRIR_cuda.cu:95-105), at least 8
    long N = 8;
    while (N < n) N <<= 1;
    return (int)N;
}

static int get_twiddles(gpurir_sim *s, int N, cudaStream_t st, const float2 **out) {
    for (auto &t : s->twiddles)
        if (t.first == N) { *out = t.second; return GPURIR_OK; }
    float2 *w = nullptr;
    CK(cudaMalloc(&w, sizeof(float2) * N));
    CK(twiddle_launch(w, N, st));
    s->twiddles.push_back({N, w});
    *out = w;
    return GPURIR_OK;
}

static int ensure_conv(gpurir_sim *s, size_t bytes) {
    if (bytes <= s->d_conv_bytes) return GPURIR_OK;
    if (s->conv_recorded) CK(cudaEventSynchronize(s->conv_busy));
    if (s->d_conv) CK(cudaFree(s->d_conv));
    s->d_conv = nullptr;
    s->d_conv_bytes = 0;
    size_t want = align_up(bytes + bytes / 4, 1 << 20);
    CK(cudaMalloc(&s->d_conv, want));
    s->d_conv_bytes = want;
    return GPURIR_OK;
}

// Row pitch of the intermediate convolution rows: whole float4s, so that the
// convolution kernel stores them 16 bytes at a time.
static long conv_ld(long n) { return (n + 3) & ~3L; }

struct ConvPlan {
    int N, M, grid_seg, grid_conv;
    size_t o_sg, o_scr, o_conv, o_win, o_in_seg, o_in_rir, bytes;
};

// Workspace layout: segment spectra | FFT scratch | conv output (optional) |
// window table (optional) | host-staged inputs (optional).
static int plan_conv(gpurir_sim *s, int P, int S, int R, int L, bool need_conv, bool need_win,
                     bool stage_inputs, ConvPlan &C) {
    if (P < 1 || R < 1 || S < 1 || L < 1) return fail(GPURIR_ERR_INVALID, "empty convolution");
    const long n = (long)S + L - 1;
    if (n > kFftMaxN) return fail(GPURIR_ERR_UNSUPPORTED, "segment + RIR longer than 2^24 samples");
    C.N = fft_size(n);
    C.M = C.N / 2;
    const bool smem = fft_smem_bytes(C.M) > 0;
    C.grid_seg = std::min(P, smem ? s->num_sms : 2 * s->num_sms);
    C.grid_conv = std::min(P * R, smem ? s->num_sms : 2 * s->num_sms);
    const int grid_scr = std::max(C.grid_seg, C.grid_conv);
    C.o_sg = 0;
    C.o_scr = align_up(C.o_sg + (size_t)P * (C.M + 1) * sizeof(float2), 256);
    C.o_conv = align_up(C.o_scr + fft_scratch_floats2(C.M, grid_scr) * sizeof(float2), 256);
    C.o_win = align_up(C.o_conv + (need_conv ? (size_t)P * R * conv_ld(n) * sizeof(float) : 0), 256);
    C.o_in_seg = align_up(C.o_win + (need_win ? (size_t)2 * (P + 1) * sizeof(int) : 0), 256);
    C.o_in_rir = align_up(C.o_in_seg + (stage_inputs ? (size_t)P * S * sizeof(float) : 0), 256);
    C.bytes = align_up(C.o_in_rir + (stage_inputs ? (size_t)P * R * L * sizeof(float) : 0), 256);
    return ensure_conv(s, C.bytes);
}

static int run_conv(gpurir_sim *s, const ConvPlan &C, const float *d_seg, int P, int S,
                    const float *d_rir, int R, int L, float *d_out, long out_ld, cudaStream_t st) {
    const float2 *W = nullptr;
    int rc = get_twiddles(s, C.N, st, &W);
    if (rc) return rc;
    float2 *Sg = reinterpret_cast<float2 *>(s->d_conv + C.o_sg);
    float2 *scr = reinterpret_cast<float2 *>(s->d_conv + C.o_scr);
    CK(segment_spectra_launch(d_seg, P, S, C.M, W, Sg, scr, C.grid_seg, st));
    CK(rir_conv_launch(d_rir, P, R, L, S, C.M, W, Sg, d_out, out_ld, scr, C.grid_conv, st));
    return GPURIR_OK;
}

extern "C" int gpurir_convolutions_device(gpurir_sim *s, const float *d_segments, int M_src,
                                          int segment_len, const float *d_rir, int M_rcv, int rir_len,
                                          float *d_out, void *stream) {
    if (!s || !d_segments || !d_rir || !d_out) return fail(GPURIR_ERR_INVALID, "NULL argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (s->conv_recorded) CK(cudaStreamWaitEvent(st, s->conv_busy, 0));
    ConvPlan C;
    int rc = plan_conv(s, M_src, segment_len, M_rcv, rir_len, false, false, false, C);
    if (rc) return rc;
    rc = run_conv(s, C, d_segments, M_src, segment_len, d_rir, M_rcv, rir_len, d_out,
                  (long)segment_len + rir_len - 1, st);
    if (rc) return rc;
    CK(cudaEventRecord(s->conv_busy, st));
    s->conv_recorded = true;
    return GPURIR_OK;
}

extern "C" int gpurir_convolutions(gpurir_sim *s, const float *source_segments, int M_src,
                                   int segment_len, const float *RIR, int M_rcv, int RIR_len,
                                   float *out) {
    if (!s || !source_segments || !RIR || !out) return fail(GPURIR_ERR_INVALID, "NULL argument");
    cudaStream_t st = s->stream;
    if (s->conv_recorded) CK(cudaStreamWaitEvent(st, s->conv_busy, 0));
    ConvPlan C;
    int rc = plan_conv(s, M_src, segment_len, M_rcv, RIR_len, true, false, true, C);
    if (rc) return rc;
    float *dseg = reinterpret_cast<float *>(s->d_conv + C.o_in_seg);
    float *drir = reinterpret_cast<float *>(s->d_conv + C.o_in_rir);
    float *dout = reinterpret_cast<float *>(s->d_conv + C.o_conv);
    const long n = (long)segment_len + RIR_len - 1;
    CK(cudaMemcpyAsync(dseg, source_segments, sizeof(float) * M_src * segment_len, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(drir, RIR, sizeof(float) * (size_t)M_src * M_rcv * RIR_len, cudaMemcpyHostToDevice, st));
    rc = run_conv(s, C, dseg, M_src, segment_len, drir, M_rcv, RIR_len, dout, n, st);
    if (rc) return rc;
    CK(cudaMemcpyAsync(out, dout, sizeof(float) * (size_t)M_src * M_rcv * n, cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(s->conv_busy, st));
    s->conv_recorded = true;
    CK(cudaStreamSynchronize(st));
    return GPURIR_OK;
}

static int check_windows(const int *w_ini, int n_pts, int seg_len, std::vector<int> &win) {
    win.assign(2 * (n_pts + 1), 0);
    if (w_ini[0] != 0) return fail(GPURIR_ERR_INVALID, "The first timestamp must be 0");
    for (int p = 0; p < n_pts; p++) {
        const int len = w_ini[p + 1] - w_ini[p];
        if (len < 0) return fail(GPURIR_ERR_INVALID, "timestamps must not decrease");
        if (len > seg_len) return fail(GPURIR_ERR_INVALID, "segment longer than segment_len");
        win[p] = w_ini[p];
        win[n_pts + 1 + p] = len;
    }
    win[n_pts] = w_ini[n_pts];
    return GPURIR_OK;
}

// Shared body: segments and RIRs on the device, output [n_samples + L - 1][R] float64.
static int trajectory_core(gpurir_sim *s, const float *d_seg, int n_pts, int seg_len,
                           const int *w_ini, const float *d_rir, int n_rcv, int rir_len,
                           double *d_out, const float *h_seg, const float *h_rir, cudaStream_t st) {
    std::vector<int> win;
    int rc = check_windows(w_ini, n_pts, seg_len, win);
    if (rc) return rc;
    if (s->conv_recorded) CK(cudaStreamWaitEvent(st, s->conv_busy, 0));
    ConvPlan C;
    const bool stage = h_seg != nullptr;
    if ((rc = plan_conv(s, n_pts, seg_len, n_rcv, rir_len, true, true, stage, C))) return rc;
    if (stage) {
        float *dseg = reinterpret_cast<float *>(s->d_conv + C.o_in_seg);
        float *drir = reinterpret_cast<float *>(s->d_conv + C.o_in_rir);
        CK(cudaMemcpyAsync(dseg, h_seg, sizeof(float) * n_pts * seg_len, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(drir, h_rir, sizeof(float) * (size_t)n_pts * n_rcv * rir_len,
                           cudaMemcpyHostToDevice, st));
        d_seg = dseg;
        d_rir = drir;
    }
    if ((rc = ensure_stage(s, win.size() * sizeof(int)))) return rc;
    memcpy(s->h_stage, win.data(), win.size() * sizeof(int));
    int *dwin = reinterpret_cast<int *>(s->d_conv + C.o_win);
    CK(cudaMemcpyAsync(dwin, s->h_stage, win.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(s->stage_done, st));
    s->stage_pending = true;
    const long n = (long)seg_len + rir_len - 1;
    float *conv = reinterpret_cast<float *>(s->d_conv + C.o_conv);
    if ((rc = run_conv(s, C, d_seg, n_pts, seg_len, d_rir, n_rcv, rir_len, conv, conv_ld(n), st))) return rc;
    // segments back to back with one width (the default segmentation): the overlap-add
    // finds each sample's points by division instead of searching the window table
    int uni_w = n_pts > 0 ? w_ini[1] - w_ini[0] : 0;
    for (int p = 0; p < n_pts && uni_w > 0; p++)
        if (w_ini[p] != p * uni_w || w_ini[p + 1] - w_ini[p] != uni_w) uni_w = 0;
    CK(ola_launch(conv, conv_ld(n), dwin, dwin + n_pts + 1, n_pts, n_rcv, rir_len,
                  (long)w_ini[n_pts] + rir_len - 1, uni_w, d_out, st));
    CK(cudaEventRecord(s->conv_busy, st));
    s->conv_recorded = true;
    return GPURIR_OK;
}

extern "C" int gpurir_trajectory_device(gpurir_sim *s, const float *d_segments, int n_pts, int seg_len,
                                        const int *w_ini, const float *d_rir, int n_rcv, int rir_len,
                                        double *d_out, void *stream) {
    if (!s || !d_segments || !w_ini || !d_rir || !d_out) return fail(GPURIR_ERR_INVALID, "NULL argument");
    return trajectory_core(s, d_segments, n_pts, seg_len, w_ini, d_rir, n_rcv, rir_len, d_out, nullptr,
                           nullptr, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int gpurir_trajectory_adjoint_device(gpurir_sim *s, const float *d_segments, int n_pts, int seg_len,
                                                const int *w_ini, const float *d_rir, int n_rcv, int rir_len,
                                                const double *d_grad_out, float *d_grad_signal,
                                                float *d_grad_rir, void *stream) {
    if (!s || !d_segments || !w_ini || !d_rir || !d_grad_out) return fail(GPURIR_ERR_INVALID, "NULL argument");
    if (n_pts < 1 || n_rcv < 1 || seg_len < 1 || rir_len < 1) return fail(GPURIR_ERR_INVALID, "empty trajectory");
    std::vector<int> win;
    int rc = check_windows(w_ini, n_pts, seg_len, win);
    if (rc) return rc;
    if (!d_grad_signal && !d_grad_rir) return GPURIR_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const long n = (long)seg_len + rir_len - 1;
    if (n > 16384) return fail(GPURIR_ERR_UNSUPPORTED, "trajectory adjoint: segment + RIR longer than 16384 samples");
    // the register FFT kernels cover N = 2048 .. 16384: shorter problems are zero-padded to 2048
    const int N = std::max(fft_size(n), 2048), M = N / 2;
    const long n_out = (long)w_ini[n_pts] + rir_len - 1;
    const int grid = traj_adjoint_grid(M, n_pts, s->num_sms);
    if (s->conv_recorded) CK(cudaStreamWaitEvent(st, s->conv_busy, 0));
    const size_t o_sg = 0;
    const size_t o_gt = align_up(o_sg + (size_t)n_pts * (M + 1) * sizeof(float2), 256);
    const size_t o_acc = align_up(o_gt + (size_t)n_rcv * n_out * sizeof(float), 256);
    const size_t o_win = align_up(o_acc + (size_t)grid * (M + 1) * sizeof(float2), 256);
    const size_t bytes = align_up(o_win + win.size() * sizeof(int), 256);
    if ((rc = ensure_conv(s, bytes))) return rc;
    const float2 *W = nullptr;
    if ((rc = get_twiddles(s, N, st, &W))) return rc;
    if ((rc = ensure_stage(s, win.size() * sizeof(int)))) return rc;
    memcpy(s->h_stage, win.data(), win.size() * sizeof(int));
    int *dwin = reinterpret_cast<int *>(s->d_conv + o_win);
    CK(cudaMemcpyAsync(dwin, s->h_stage, win.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(s->stage_done, st));
    s->stage_pending = true;
    float2 *Sg = reinterpret_cast<float2 *>(s->d_conv + o_sg);
    CK(segment_spectra_launch(d_segments, n_pts, seg_len, M, W, Sg, nullptr, s->num_sms, st));
    CK(traj_adjoint_launch(d_grad_out, n_out, dwin, dwin + n_pts + 1, d_rir, n_pts, n_rcv, rir_len, M, W, Sg,
                           reinterpret_cast<float *>(s->d_conv + o_gt), d_grad_rir, d_grad_signal,
                           reinterpret_cast<float2 *>(s->d_conv + o_acc), grid, st));
    CK(cudaEventRecord(s->conv_busy, st));
    s->conv_recorded = true;
    return GPURIR_OK;
}

extern "C" int gpurir_trajectory(gpurir_sim *s, const float *segments, int n_pts, int seg_len,
                                 const int *w_ini, const float *rir, int n_rcv, int rir_len,
                                 double *out) {
    if (!s || !segments || !w_ini || !rir || !out) return fail(GPURIR_ERR_INVALID, "NULL argument");
    const long n_out = (long)w_ini[n_pts] + rir_len - 1;
    if (n_pts < 1 || n_out < 1) return fail(GPURIR_ERR_INVALID, "empty trajectory");
    double *dout = nullptr;
    CK(cudaMallocAsync(reinterpret_cast<void **>(&dout), sizeof(double) * n_out * n_rcv, s->stream));
    int rc = trajectory_core(s, segments, n_pts, seg_len, w_ini, rir, n_rcv, rir_len, dout, segments,
                             rir, s->stream);
    if (rc == GPURIR_OK) {
        cudaError_t e = cudaMemcpyAsync(out, dout, sizeof(double) * n_out * n_rcv, cudaMemcpyDeviceToHost,
                                        s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) rc = fail(GPURIR_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFreeAsync(dout, s->stream);
    cudaStreamSynchronize(s->stream);
    return rc;
}

// ---------------------------------------------------------------------------
// Helpers shared with the fixed-scratch entry point (ism_noalloc.cu).
// ---------------------------------------------------------------------------
namespace gpurir {
int describe_room(RoomDesc &R, const float room[3], const float beta[6], const int nb[3], float Tdiff,
                  float Tmax, float Fs, float c, int spkr, int mic) {
    return build_room(R, room, beta, nb, Tdiff, Tmax, Fs, c, spkr, mic);
}

int window_plan(float H, int &tpl, int &em, int &clamp, int &max_nsub) {
    Plan P;   // FP32 mode
    int rc = plan_window(H, P, max_nsub);
    tpl = P.tpl;
    em = P.em;
    clamp = P.clamp;
    return rc;
}

int set_last_error(int code, const char *msg) { return fail(code, msg); }
}  // namespace gpurir

extern "C" int gpurir_host_alloc(size_t bytes, void **ptr) {
    if (!ptr) return fail(GPURIR_ERR_INVALID, "gpurir_host_alloc: ptr is NULL");
    *ptr = nullptr;
    if (bytes == 0) return GPURIR_OK;
    cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocPortable | cudaHostAllocMapped);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        cudaGetLastError();
        return fail(GPURIR_ERR_CUDA, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    }
    return GPURIR_OK;
}

extern "C" int gpurir_host_free(void *ptr) {
    if (!ptr) return GPURIR_OK;
    cudaError_t e = cudaFreeHost(ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(GPURIR_ERR_CUDA, std::string("cudaFreeHost: ") + cudaGetErrorString(e));
    }
    return GPURIR_OK;
}

extern "C" int gpurir_last_output_direct(gpurir_sim *s, int *direct) {
    if (!s || !direct) return fail(GPURIR_ERR_INVALID, "NULL argument");
    *direct = s->last_direct ? 1 : 0;
    return GPURIR_OK;
}
