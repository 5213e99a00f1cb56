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

__global__ void room_beta_kernel(RoomDesc *rooms, int n_rooms, const float *beta) {
    const int r = blockIdx.x;
    if (r >= n_rooms) return;
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

cudaError_t room_beta_launch(RoomDesc *rooms, int n_rooms, const float *beta, cudaStream_t st) {
    if (n_rooms <= 0) return cudaSuccess;
    room_beta_kernel<<<n_rooms, 32, 0, st>>>(rooms, n_rooms, beta);
    return cudaGetLastError();
}

}  // namespace gpurir
