// rooms.cu -- room descriptors refreshed on the device from device-resident wall
// coefficients, so that a differentiable step (forward, loss, adjoint, update of
// beta) runs without a host round trip of beta.
//
// Per room: beta, the Sabine T60 of src/gpuRIR_cuda.cu:123-130 in float32 (as the
// reference and the host path evaluate it), and the power tables
// pw[w][k] = (-beta_w)^k, k < pow_n, formed in FP64 by repeated multiplication and
// rounded to float32, exactly as the host builds them (the same bits); the serial
// chain stops at pow_n, the entries after it are zero from the host's descriptor.
#include "gpurir_internal.cuh"

namespace gpurir {

__device__ __forceinline__ void room_beta_kernel_body(RoomDesc *rooms, int r, const float *beta) {
    RoomDesc &R = rooms[r];
    const int w = threadIdx.x;   // one thread per wall
    if (w < 6) {
        const float b = beta[6 * r + w];
        R.beta[w] = b;
        const double m = -(double)b;
        const int n = R.pow_n;   // entries from pow_n on stay the zeros the host wrote
        double p = 1.0;
        for (int k = 0; k < n; k++) {
            R.pw[w][k] = (float)p;
            p *= m;
        }
    }
    if (w == 0) {
        const float *b = beta + 6 * r;
        const float Sa = ((1.0f - b[0] * b[0]) + (1.0f - b[1] * b[1])) * R.L[1] * R.L[2] +
                         ((1.0f - b[2] * b[2]) + (1.0f - b[3] * b[3])) * R.L[0] * R.L[2] +
                         ((1.0f - b[4] * b[4]) + (1.0f - b[5] * b[5])) * R.L[0] * R.L[1];
        R.T60 = 0.161f * (R.L[0] * R.L[1] * R.L[2]) / Sa;
    }
}

__global__ void room_beta_kernel(RoomDesc *rooms, int n_rooms, const float *beta) {
    if ((int)blockIdx.x < n_rooms) room_beta_kernel_body(rooms, blockIdx.x, beta);
}

// room_beta_kernel's work in blocks [0, n_rooms) and, in the blocks after them, the
// per-item skip flags of item_skip_kernel (independent of beta: room geometry and
// positions only), so that a differentiable forward step needs one launch for both.
__global__ void room_beta_skip_kernel(RoomDesc *rooms, int n_rooms, const float *beta, const IsmItem *items,
                                      int n_items, const float *pos_src, const float *pos_rcv,
                                      unsigned char *skip) {
    if ((int)blockIdx.x < n_rooms) {
        if (threadIdx.x < 32) room_beta_kernel_body(rooms, blockIdx.x, beta);
        return;
    }
    const int k = (blockIdx.x - n_rooms) * blockDim.x + threadIdx.x;
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

cudaError_t room_beta_skip_launch(RoomDesc *rooms, int n_rooms, const float *beta, const IsmItem *items,
                                  int n_items, const float *pos_src, const float *pos_rcv, unsigned char *skip,
                                  cudaStream_t st) {
    const int blocks = n_rooms + (n_items + 255) / 256;
    if (blocks <= 0) return cudaSuccess;
    room_beta_skip_kernel<<<blocks, 256, 0, st>>>(rooms, n_rooms, beta, items, n_items, pos_src, pos_rcv, skip);
    return cudaGetLastError();
}

cudaError_t room_beta_launch(RoomDesc *rooms, int n_rooms, const float *beta, cudaStream_t st) {
    if (n_rooms <= 0) return cudaSuccess;
    room_beta_kernel<<<n_rooms, 32, 0, st>>>(rooms, n_rooms, beta);
    return cudaGetLastError();
}

}  // namespace gpurir
