// ism_noalloc.cu -- an image-source entry point that allocates no memory.
//
// Who needs it: code that may not call cudaMalloc at the moment it simulates.
// A real-time audio callback must not block, and cudaMalloc can stall on an
// implicit device synchronisation; an application that owns a fixed device
// memory budget (a plugin host, a game engine) forbids plugins from growing
// their footprint after start-up; code recording work under global stream
// capture may not allocate at all.  Such callers get the early part of the
// RIRs through gpurir_simulate_ism_noalloc, whose only scratch -- the room
// descriptor, the work-item table, the work counter and the status word -- is
// the fixed array below, present on every GPU that loads the library until the
// process exits.  The kernel is the fused forward kernel of ism_forward.cu.
//
// The forward kernel can flag an inconsistent work item in the status word of
// the scratch, but the items here are built by noalloc_prepare_kernel from
// sizes the host has already checked, so no flag is ever raised on this path;
// the word is cleared by the next call and not reported.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "gpurir_internal.cuh"
#include "../../include/gpurir_gb300.h"

namespace gpurir {
size_t ism_forward_smem_bytes(int tpl, int em, int max_nsub, int mode, int tw);
int ism_forward_blocks_per_sm(int tpl, size_t smem, int mode);
cudaError_t ism_forward_launch(int tpl, const RoomDesc *rooms, const IsmItem *items, int n_items,
                               const float *pos_src, const float *pos_rcv, const float *orv_src,
                               const float *orv_rcv, float *out, int *work_counter, int *status,
                               int em, int max_nsub, int clamp, int grid, cudaStream_t st, int mode,
                               int tw, const TailArgs *tail, float4 *axis_tab, int axis_cap,
                               float *partial, const unsigned char *skip);
int describe_room(RoomDesc &R, const float room[3], const float beta[6], const int nb[3], float Tdiff,
                  float Tmax, float Fs, float c, int spkr, int mic);
int window_plan(float H, int &tpl, int &em, int &clamp, int &max_nsub);
int set_last_error(int code, const char *msg);
}  // namespace gpurir

using namespace gpurir;

// Limits of the fixed scratch.
constexpr int kNoAllocMaxItems = 8192;   // RIRs x segments per call
constexpr size_t kNoAllocCtl = 256;      // work counter (int) and status word (int)
constexpr size_t kNoAllocRoom = (sizeof(RoomDesc) + 255) / 256 * 256;
constexpr size_t kNoAllocBytes = kNoAllocCtl + kNoAllocRoom + (size_t)kNoAllocMaxItems * sizeof(IsmItem);

// The scratch: 256 B of control words, one RoomDesc, kNoAllocMaxItems IsmItems
// (about 390 KB).  Shared by every call on this device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch per device, with the id of the CUDA context it
// was looked up in.  A device reset destroys the context and the module with it,
// and the array may then live at another address: a call whose current context
// differs from the cached one looks the address up again (cudaGetSymbolAddress
// allocates nothing; on the first call in a context it may load the module).
// The cache is guarded by a mutex (no allocation either).
constexpr int kMaxDevices = 64;
struct ScratchSlot {
    unsigned long long ctx_id;
    unsigned char *ptr;
};
static ScratchSlot g_scratch[kMaxDevices];
static std::mutex g_scratch_mu;

typedef int (*CtxGetCurrentFn)(void **ctx);
typedef int (*CtxGetIdFn)(void *ctx, unsigned long long *id);
static CtxGetCurrentFn g_ctx_get_current = nullptr;
static CtxGetIdFn g_ctx_get_id = nullptr;
static std::once_flag g_ctx_fns_once;

// Id of the current CUDA context (0: none current, or the driver lacks the query).
static unsigned long long current_context_id() {
    std::call_once(g_ctx_fns_once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f);
        cudaGetLastError();
    });
    if (!g_ctx_get_current || !g_ctx_get_id) return 0;
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&ctx) != 0 || !ctx) return 0;
    if (g_ctx_get_id(ctx, &id) != 0) return 0;
    return id;
}

static int scratch_for_current_device(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_last_error(GPURIR_ERR_CUDA, "gpurir_simulate_ism_noalloc: cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices)
        return set_last_error(GPURIR_ERR_UNSUPPORTED, "gpurir_simulate_ism_noalloc: device index above 63");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    unsigned long long id = current_context_id();
    ScratchSlot &slot = g_scratch[dev];
    if (id == 0 || !slot.ptr || slot.ctx_id != id) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_last_error(GPURIR_ERR_CUDA,
                                  "gpurir_simulate_ism_noalloc: cudaGetSymbolAddress of the scratch failed");
        slot.ptr = static_cast<unsigned char *>(p);
        slot.ctx_id = current_context_id();   // the lookup made the primary context current
    }
    *out = slot.ptr;
    return GPURIR_OK;
}

// Fills the scratch for one call: control words zeroed, the room descriptor,
// and the work items (one per RIR and segment, later segments first; rows of
// n_ism samples).  Names the scratch array directly.
__global__ void noalloc_prepare_kernel(RoomDesc R, long M, int M_rcv, long n_seg, long tseg,
                                       long n_items) {
    int *ctl = reinterpret_cast<int *>(g_noalloc_scratch);
    RoomDesc *room = reinterpret_cast<RoomDesc *>(g_noalloc_scratch + kNoAllocCtl);
    IsmItem *items = reinterpret_cast<IsmItem *>(g_noalloc_scratch + kNoAllocCtl + kNoAllocRoom);
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) {
        for (size_t i = 0; i < kNoAllocCtl / sizeof(int); i++) ctl[i] = 0;
        *room = R;
    }
    if (k >= n_items) return;
    const long g = n_seg - 1 - k / M, m = k % M;
    IsmItem it;
    it.room = 0;
    it.src = (int)(m / M_rcv);
    it.rcv = (int)(m % M_rcv);
    it.rir = (int)m;
    it.out_row = (long long)m * R.n_ism;
    it.t_lo = (int)(g * tseg);
    it.t_hi = (int)min((g + 1) * tseg, (long)R.n_ism);
    it.i_lo = 0;
    it.i_hi = R.n_img;
    it.part_off = -1;
    items[k] = it;
}

extern "C" int gpurir_simulate_ism_noalloc(const float room_sz[3], const float beta[6],
                                           const float *d_pos_src, int M_src, const float *d_pos_rcv,
                                           const float *d_orV_src, const float *d_orV_rcv,
                                           int spkr_pattern, int mic_pattern, int M_rcv,
                                           const int nb_img[3], float T, float Fs, float c,
                                           float *d_rir_out, void *stream) {
    if (!room_sz || !beta || !nb_img || !d_pos_src || !d_pos_rcv || !d_rir_out)
        return set_last_error(GPURIR_ERR_INVALID, "gpurir_simulate_ism_noalloc: NULL argument");
    if (M_src < 1 || M_rcv < 1)
        return set_last_error(GPURIR_ERR_INVALID, "gpurir_simulate_ism_noalloc: need a source and a receiver");
    if ((spkr_pattern != 0 && !d_orV_src) || (mic_pattern != 0 && !d_orV_rcv))
        return set_last_error(GPURIR_ERR_INVALID,
                              "gpurir_simulate_ism_noalloc: orientation required for a non-omni pattern");
    const long M = (long)M_src * M_rcv;
    if (M > kNoAllocMaxItems)
        return set_last_error(GPURIR_ERR_INVALID,
                              "gpurir_simulate_ism_noalloc: more than 8192 RIRs (fixed scratch limit)");
    RoomDesc R;
    int rc = describe_room(R, room_sz, beta, nb_img, T, T, Fs, c, spkr_pattern, mic_pattern);
    if (rc) return rc;
    R.n_src = M_src;
    R.n_rcv = M_rcv;
    int tpl, em, clamp, max_nsub;
    if ((rc = window_plan(R.H, tpl, em, clamp, max_nsub))) return rc;
    unsigned char *scr = nullptr;
    if ((rc = scratch_for_current_device(&scr))) return rc;
    if (R.n_ism <= 0) return GPURIR_OK;

    // Segments: as many per RIR as the fixed item table and the SM count call for.
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return set_last_error(GPURIR_ERR_CUDA, "gpurir_simulate_ism_noalloc: device query failed");
    const int sub = 32 * tpl;
    const long seg_max = std::min<long>((long)max_nsub * sub, 16384);
    long n_seg = std::max<long>((R.n_ism + seg_max - 1) / seg_max,
                                std::min<long>((4L * sms + M - 1) / M, (R.n_ism + sub - 1) / sub));
    if (M * n_seg > kNoAllocMaxItems) n_seg = kNoAllocMaxItems / M;
    long tseg = (R.n_ism + n_seg - 1) / n_seg;
    tseg = std::min<long>((tseg + 31) / 32 * 32, seg_max);
    n_seg = (R.n_ism + tseg - 1) / tseg;
    if (M * n_seg > kNoAllocMaxItems)
        return set_last_error(GPURIR_ERR_INVALID,
                              "gpurir_simulate_ism_noalloc: RIRs x segments above 8192 (fixed scratch limit; "
                              "long RIRs are cut into several segments)");
    const int nsub = (int)((tseg + sub - 1) / sub);
    const int tw = (int)std::lround(2.0 * R.H);
    const size_t smem = ism_forward_smem_bytes(tpl, em, nsub, 0, tw);
    const int bps = ism_forward_blocks_per_sm(tpl, smem, 0);
    if (bps < 1) return set_last_error(GPURIR_ERR_CUDA, "gpurir_simulate_ism_noalloc: kernel does not fit");
    const long n_items = M * n_seg;
    const int grid = (int)std::min<long>(n_items, (long)sms * bps);

    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int *ctl = reinterpret_cast<int *>(scr);
    RoomDesc *d_room = reinterpret_cast<RoomDesc *>(scr + kNoAllocCtl);
    IsmItem *d_items = reinterpret_cast<IsmItem *>(scr + kNoAllocCtl + kNoAllocRoom);
    // The room descriptor travels as a kernel parameter; the prepare kernel
    // writes it, the work items and zeroed control words into the scratch.
    noalloc_prepare_kernel<<<(unsigned)((n_items + 255) / 256), 256, 0, st>>>(R, M, M_rcv, n_seg, tseg,
                                                                             n_items);
    if (cudaGetLastError() != cudaSuccess)
        return set_last_error(GPURIR_ERR_CUDA, "gpurir_simulate_ism_noalloc: prepare launch failed");
    if (ism_forward_launch(tpl, d_room, d_items, (int)n_items, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv,
                           d_rir_out, ctl, ctl + 1, em, nsub, clamp, grid, st, 0, tw, nullptr, nullptr, 0, nullptr,
                           nullptr) != cudaSuccess)
        return set_last_error(GPURIR_ERR_CUDA, "gpurir_simulate_ism_noalloc: kernel launch failed");
    return GPURIR_OK;
}
