// tuning.cu -- process-wide launch-shape knobs chosen by the autotuner.
//
// Every knob here changes how work is laid out on the GPU (rows per block,
// resident blocks per SM), never which operations are applied to which data
// in which order: a tuned launch computes the same bits as the default one.
// gpurir_gb300/tune.py measures the candidates on the current GPU and stores
// the winners in a cache keyed by the GPU's name; the Python package applies
// that cache when it loads the library.  gpuRIR fixes the equivalent choices
// as compile-time constants (src/gpuRIR_cuda.cu:20-45).
#include <atomic>
#include <cstdio>
#include <cstring>

#include <cuda_runtime.h>

#include "../../include/gpurir_gb300.h"

namespace gpurir {

int set_last_error(int code, const char *msg);

enum TuneKnob { kTuneConvRows = 0, kTuneIsmBlocksPerSm, kTuneBwdBlocksPerSm, kTuneTrajBlocksPerSm, kTuneCount };

struct KnobInfo {
    const char *name;
    int def, lo, hi;   // default, allowed range (0 = the occupancy maximum where noted)
};

static const KnobInfo kKnobs[kTuneCount] = {
    {"conv_rows", 2, 1, 2},               // RIR rows transformed together per block (convolution)
    {"ism_blocks_per_sm", 0, 0, 4},       // forward ISM kernel: 0 = as many as fit
    {"adjoint_blocks_per_sm", 0, 0, 8},   // adjoint ISM kernel: 0 = as many as fit
    {"traj_adjoint_blocks_per_sm", 0, 0, 2},  // trajectory adjoint: 0 = 1 at N = 16384, else 2
};

static std::atomic<int> g_knob[kTuneCount] = {{2}, {0}, {0}, {0}};

int tuning(int knob) { return g_knob[knob].load(std::memory_order_relaxed); }

}  // namespace gpurir

using namespace gpurir;

extern "C" int gpurir_set_tuning(const char *knob, int value) {
    if (!knob) return set_last_error(GPURIR_ERR_INVALID, "gpurir_set_tuning: NULL knob");
    for (int k = 0; k < kTuneCount; k++)
        if (strcmp(knob, kKnobs[k].name) == 0) {
            if (value < kKnobs[k].lo || value > kKnobs[k].hi)
                return set_last_error(GPURIR_ERR_INVALID, "gpurir_set_tuning: value out of range");
            g_knob[k].store(value, std::memory_order_relaxed);
            return GPURIR_OK;
        }
    return set_last_error(GPURIR_ERR_INVALID, "gpurir_set_tuning: unknown knob");
}

extern "C" int gpurir_get_tuning(const char *knob, int *value) {
    if (!knob || !value) return set_last_error(GPURIR_ERR_INVALID, "gpurir_get_tuning: NULL argument");
    for (int k = 0; k < kTuneCount; k++)
        if (strcmp(knob, kKnobs[k].name) == 0) {
            *value = g_knob[k].load(std::memory_order_relaxed);
            return GPURIR_OK;
        }
    return set_last_error(GPURIR_ERR_INVALID, "gpurir_get_tuning: unknown knob");
}

extern "C" int gpurir_reset_tuning(void) {
    for (int k = 0; k < kTuneCount; k++) g_knob[k].store(kKnobs[k].def, std::memory_order_relaxed);
    return GPURIR_OK;
}

extern "C" int gpurir_device_name(char *name, int len) {
    if (!name || len < 1) return set_last_error(GPURIR_ERR_INVALID, "gpurir_device_name: no buffer");
    int dev = 0;
    cudaDeviceProp p;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
        cudaGetLastError();
        return set_last_error(GPURIR_ERR_CUDA, "gpurir_device_name: no CUDA device");
    }
    snprintf(name, (size_t)len, "%s (sm_%d%d, %d SMs)", p.name, p.major, p.minor, p.multiProcessorCount);
    return GPURIR_OK;
}
