/*
 * gpurir_gb300.h -- C ABI of the gpurir_gb300 room-impulse-response engine
 * (image-source method on one NVIDIA GB300, sm_103a).
 *
 * Plain pointers, sizes and status codes only: no C++ or torch types cross
 * this boundary.  Every function returns GPURIR_OK (0) or a negative status;
 * gpurir_last_error() gives a message for the calling thread.  Nothing here
 * calls exit(), unlike the reference's gpuErrchk (src/gpuRIR_cuda.cu:68-93).
 *
 * A handle owns one CUDA stream, a grow-only device workspace and pinned
 * staging memory.  A handle is not thread-safe: use one per host thread.
 * Functions with a `stream` argument are stream-ordered on that stream
 * (NULL is the CUDA default stream, as in the runtime API) and return before
 * the GPU finishes; the others run on the handle's own stream and block until
 * their results are on the host.
 *
 * Array layouts are C order; positions are [count][3] float32 metres.
 * Polar patterns: 0 omni, 1 homni, 2 card, 3 hypcard, 4 subcard, 5 bidir
 * (src/gpuRIR_cuda.h:2-8).
 */
#ifndef GPURIR_GB300_H
#define GPURIR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPURIR_OK 0
#define GPURIR_ERR_INVALID (-1)   /* bad argument: sizes, patterns, lengths */
#define GPURIR_ERR_CUDA (-2)      /* a CUDA runtime call failed */
#define GPURIR_ERR_DEVICE (-3)    /* a kernel reported an inconsistent work item */
#define GPURIR_ERR_UNSUPPORTED (-4)

#define GPURIR_NOISE_LOGISTIC 0   /* the reference's transform, src/gpuRIR_cuda.cu:454-455 */
#define GPURIR_NOISE_GAUSSIAN 1   /* Box-Muller on the same Philox words */

typedef struct gpurir_sim gpurir_sim;

/* Version string of the library. */
const char *gpurir_version(void);

/* Message of the last failed call on this host thread ("" if none). */
const char *gpurir_last_error(void);

/* Create a simulator on the current CUDA device.
 * Replaces gpuRIR_cuda::gpuRIR_cuda(bool, bool), src/gpuRIR_cuda.cu:1025-1048
 * (flags as the Python binding's default, src/python_bind.cpp:15).
 * The tail noise is keyed by `seed` (the reference fixes cuRAND's seed to 1234,
 * src/gpuRIR_cuda.cu:1046-1047); every simulate call advances a call counter so
 * successive calls draw different noise, as the stateful generator does. */
int gpurir_create(int mixed_precision, int lookup_table, uint64_t seed, gpurir_sim **out);

/* Release a simulator and its workspace. */
int gpurir_destroy(gpurir_sim *sim);

/* Mode flags.  Replace gpuRIR_cuda::activate_mixed_precision / activate_lut,
 * src/gpuRIR_cuda.cu:1050-1073: the two modes exclude each other, turning one
 * on turns the other off.  *state receives the resulting flag (may be NULL). */
int gpurir_activate_mixed_precision(gpurir_sim *sim, int activate, int *state);
int gpurir_activate_lut(gpurir_sim *sim, int activate, int *state);

/* Read the flags. */
int gpurir_get_modes(gpurir_sim *sim, int *mixed_precision, int *lookup_table);

/* Delay model of the image sources.  Off (default): each delay is the exact
 * distance * Fs / c, to ~1e-10 samples.  On: the delay is rounded in float32
 * step by step as gpuRIR's calcAmpTau_kernel forms it (src/gpuRIR_cuda.cu:
 * 336-369: cluster offset, receiver->image components, squared distance,
 * sqrtf, dist / c * Fs), and the direct-path delay of the diffuse tail's
 * envelope likewise, so that the output matches the reference build's up to
 * the rounding of the tap arithmetic; the reference's delays are up to ~4e-4
 * samples off the exact ones at 0.3 s.  Applies to every mode (FP32, mixed
 * precision, lookup table) and to the simulate and batch entries of `sim`; the
 * adjoint entries always differentiate the exact model.  The reference has no
 * such switch (its delays are always the float32 ones).  *state receives the
 * resulting flag (may be NULL). */
int gpurir_set_reference_delays(gpurir_sim *sim, int activate, int *state);
int gpurir_get_reference_delays(gpurir_sim *sim, int *state);

/* Compensated accumulation of the taps in the mixed-precision and lookup-table
 * modes: each chunk of images is summed into FP32 buffers as usual, then added
 * into a running (hi, lo) pair per sample by an error-free two-sum, so the
 * rounding error of a late, dense sample does not grow with the number of
 * images reaching it (lookup table at 1 s: 1.9e-7 rel-L2 late in the RIR
 * instead of 5.8e-7).  policy 0: never; 1 (default): lookup-table mode when an
 * early part is at least 8000 samples long; 2: always, mixed precision too
 * (where the half-precision window, 1.3e-4, dominates anyway).  It costs shared
 * memory (shorter segments: ~1.5x the time on a 1 s RIR), not arithmetic per
 * tap.  The FP32 mode is not affected.  The
 * reference accumulates its half2 path in half precision
 * (src/gpuRIR_cuda.cu:501-506); it has no such switch. */
int gpurir_set_compensation(gpurir_sim *sim, int policy);

/* Noise transform of the tail (GPURIR_NOISE_*), and the (seed, call counter)
 * pair that keys it.  The counter advances by one per simulate call. */
int gpurir_set_noise(gpurir_sim *sim, int noise_kind);
int gpurir_set_seed(gpurir_sim *sim, uint64_t seed, uint64_t call_counter);
int gpurir_get_seed(gpurir_sim *sim, uint64_t *seed, uint64_t *call_counter);

/* Number of samples for a duration: ceil(T*Fs) in float32, rounded up to even
 * (src/gpuRIR_cuda.cu:831-835, src/python_bind.cpp:82-83). */
int gpurir_n_samples(float T, float Fs);

/*
 * Simulate the RIRs of one room, host buffers in and out.
 * Replaces gpuRIR_cuda::cuda_simulateRIR, src/gpuRIR_cuda.cu:766-931, called
 * by gpuRIR_bind::simulateRIR_bind, src/python_bind.cpp:29-88.  Same argument
 * order and meaning; the caller owns `rir_out`, a float32 buffer of
 * M_src * M_rcv * gpurir_n_samples(Tmax, Fs) values laid out
 * [M_src][M_rcv][nSamples] (the reference malloc()s it and returns it).
 * orV_src / orV_rcv may be NULL for omni patterns.
 */
int gpurir_simulate_rir(gpurir_sim *sim, const float room_sz[3], const float beta[6],
                        const float *pos_src, int M_src, const float *pos_rcv,
                        const float *orV_src, const float *orV_rcv, int spkr_pattern,
                        int mic_pattern, int M_rcv, const int nb_img[3], float Tdiff,
                        float Tmax, float Fs, float c, float *rir_out);

/* Same computation with device pointers, stream-ordered: positions and
 * orientations on the device, `d_rir_out` a device buffer of the same shape.
 * No host synchronisation. */
int gpurir_simulate_rir_device(gpurir_sim *sim, const float room_sz[3], const float beta[6],
                               const float *d_pos_src, int M_src, const float *d_pos_rcv,
                               const float *d_orV_src, const float *d_orV_rcv, int spkr_pattern,
                               int mic_pattern, int M_rcv, const int nb_img[3], float Tdiff,
                               float Tmax, float Fs, float c, float *d_rir_out, void *stream);

/* One room of a batch.  All rooms of a batch share Fs and c. */
typedef struct gpurir_room {
    float room_sz[3];      /* [m] */
    float beta[6];         /* reflection coefficients, order x0 x1 y0 y1 z0 z1 */
    int nb_img[3];         /* images per axis */
    float Tdiff;           /* [s] end of the ISM part (<= Tmax) */
    float Tmax;            /* [s] RIR length */
    int n_src, n_rcv;      /* sources and receivers of this room */
    int spkr_pattern, mic_pattern;
} gpurir_room;

/* Ragged output layout of a batch: rir_offsets[r] is the element offset of room
 * r's RIRs, C order [n_src][n_rcv][nSamples_r]; rir_offsets[n_rooms] is the
 * total.  `rir_offsets` holds n_rooms + 1 values.  gpuRIR has no batching: a
 * batch replaces a Python loop of cuda_simulateRIR calls (src/gpuRIR_cuda.cu:766). */
int gpurir_batch_layout(int n_rooms, const gpurir_room *rooms, float Fs, long long *rir_offsets);

/* Simulate a batch of rooms in one persistent launch (device I/O, stream-ordered).
 * Sources of room r are rows [sum of earlier n_src, +n_src) of d_pos_src (and of
 * d_orV_src), receivers likewise; d_out is laid out by gpurir_batch_layout. */
int gpurir_simulate_batch_device(gpurir_sim *sim, int n_rooms, const gpurir_room *rooms, float Fs,
                                 float c, const float *d_pos_src, const float *d_pos_rcv,
                                 const float *d_orV_src, const float *d_orV_rcv, float *d_out,
                                 void *stream);

/* As gpurir_simulate_batch_device, with the wall coefficients read on the device
 * from d_beta [n_rooms][6] (the rooms' beta fields are not used): the power tables
 * and Sabine T60 are refreshed by a kernel, so a differentiable step never copies
 * beta to the host.  No counterpart in the reference. */
int gpurir_simulate_batch_device_beta(gpurir_sim *sim, int n_rooms, const gpurir_room *rooms, float Fs,
                                      float c, const float *d_beta, const float *d_pos_src,
                                      const float *d_pos_rcv, const float *d_orV_src,
                                      const float *d_orV_rcv, float *d_out, void *stream);

/* A batch planned once and captured in a CUDA graph.  gpurir_batch_launch
 * replays it on `stream`; positions/orientations are re-read from the device
 * buffers given at creation on every replay, and each replay draws the next
 * noise of the handle's seed.  No counterpart in the reference. */
typedef struct gpurir_batch gpurir_batch;
int gpurir_batch_create(gpurir_sim *sim, int n_rooms, const gpurir_room *rooms, float Fs, float c,
                        const float *d_pos_src, const float *d_pos_rcv, const float *d_orV_src,
                        const float *d_orV_rcv, float *d_out, gpurir_batch **out);
int gpurir_batch_launch(gpurir_batch *batch, void *stream);
int gpurir_batch_info(gpurir_batch *batch, long long *n_rir, long long *out_elems);
int gpurir_batch_destroy(gpurir_batch *batch);

/* Adjoint of the early (ISM) part of a batch.  Given dL/dRIR in the packed
 * layout of gpurir_batch_layout (`d_grad_rir`; only the early samples are
 * read: the diffuse tail is not differentiated), writes
 *   d_grad_beta [n_rooms][6], d_grad_pos_src / d_grad_orV_src [sum n_src][3],
 *   d_grad_pos_rcv / d_grad_orV_rcv [sum n_rcv][3]
 * (each may be NULL).  Image amplitudes and delays are recomputed, not stored.
 * Deterministic.  gpuRIR has no counterpart (it is not differentiable). */
int gpurir_ism_backward_batch_device(gpurir_sim *sim, int n_rooms, const gpurir_room *rooms,
                                     float Fs, float c, const float *d_pos_src,
                                     const float *d_pos_rcv, const float *d_orV_src,
                                     const float *d_orV_rcv, const float *d_grad_rir,
                                     float *d_grad_beta, float *d_grad_pos_src,
                                     float *d_grad_pos_rcv, float *d_grad_orV_src,
                                     float *d_grad_orV_rcv, void *stream);

/* The adjoint with the wall coefficients read on the device from d_beta [n_rooms][6],
 * as gpurir_simulate_batch_device_beta.  No counterpart in the reference. */
int gpurir_ism_backward_batch_device_beta(gpurir_sim *sim, int n_rooms, const gpurir_room *rooms,
                                          float Fs, float c, const float *d_beta,
                                          const float *d_pos_src, const float *d_pos_rcv,
                                          const float *d_orV_src, const float *d_orV_rcv,
                                          const float *d_grad_rir, float *d_grad_beta,
                                          float *d_grad_pos_src, float *d_grad_pos_rcv,
                                          float *d_grad_orV_src, float *d_grad_orV_rcv, void *stream);

/* A batch prepared once for training loops: room descriptors, work items and the
 * gradient reduction lists are uploaded at creation; gpurir_adjoint_forward and
 * gpurir_adjoint_backward then only enqueue kernels on `stream` (no host work, no
 * synchronisation, no allocation), reading the wall coefficients from d_beta
 * [n_rooms][6] at every call, so a whole step (forward, loss, adjoint) can be
 * recorded in a CUDA graph.  Arguments as gpurir_simulate_batch_device_beta and
 * gpurir_ism_backward_batch_device_beta, except that gpurir_adjoint_backward takes
 * d_beta = NULL to reuse the room tables of the last gpurir_adjoint_forward on the
 * same handle (stream-ordered after it, with the same coefficients: one launch less
 * per step).  gpurir_adjoint_status returns the kernels' error word (0: none).
 * No counterpart in the reference. */
typedef struct gpurir_adjoint gpurir_adjoint;
int gpurir_adjoint_create(gpurir_sim *sim, int n_rooms, const gpurir_room *rooms, float Fs, float c,
                          gpurir_adjoint **out);
int gpurir_adjoint_forward(gpurir_adjoint *adj, const float *d_beta, const float *d_pos_src,
                           const float *d_pos_rcv, const float *d_orV_src, const float *d_orV_rcv,
                           float *d_out, void *stream);
int gpurir_adjoint_backward(gpurir_adjoint *adj, const float *d_beta, const float *d_pos_src,
                            const float *d_pos_rcv, const float *d_orV_src, const float *d_orV_rcv,
                            const float *d_grad_rir, float *d_grad_beta, float *d_grad_pos_src,
                            float *d_grad_pos_rcv, float *d_grad_orV_src, float *d_grad_orV_rcv,
                            void *stream);
int gpurir_adjoint_status(gpurir_adjoint *adj, int *status);

/* One fused training step of the L2 fit of a batch to target RIRs: the forward
 * pass into d_out (packed layout), loss = scale * sum (d_out - d_target)^2 into
 * d_loss (one float on the device) and, in the same pass over the samples, the
 * gradient 2 scale (d_out - d_target) that the adjoint then consumes; the
 * gradients are written as by gpurir_adjoint_backward (each may be NULL).  The
 * loss is summed in a fixed order (bitwise reproducible).  Enqueues kernels only,
 * except that the first call on `adj` allocates its gradient buffer
 * (out_elems floats): make it before any stream capture.  d_target and d_out
 * 16-byte aligned.  Used for the inverse problem; no counterpart in the reference. */
int gpurir_adjoint_l2_step(gpurir_adjoint *adj, const float *d_beta, const float *d_pos_src,
                           const float *d_pos_rcv, const float *d_orV_src, const float *d_orV_rcv,
                           const float *d_target, float scale, float *d_out, float *d_loss,
                           float *d_grad_beta, float *d_grad_pos_src, float *d_grad_pos_rcv,
                           float *d_grad_orV_src, float *d_grad_orV_rcv, void *stream);
int gpurir_adjoint_destroy(gpurir_adjoint *adj);

/* Batched FFT convolutions of trajectory segments with their RIRs, host
 * buffers.  Replaces gpuRIR_cuda::cuda_convolutions, src/gpuRIR_cuda.cu:933-1023
 * (called by gpuRIR_bind::gpu_conv, src/python_bind.cpp:90-119), same argument
 * order: source_segments [M_src][segment_len], RIR [M_src][M_rcv][RIR_len];
 * the caller owns `out`, float32 [M_src][M_rcv][segment_len + RIR_len - 1]. */
int gpurir_convolutions(gpurir_sim *sim, const float *source_segments, int M_src, int segment_len,
                        const float *RIR, int M_rcv, int RIR_len, float *out);

/* Same on device buffers, stream-ordered. */
int gpurir_convolutions_device(gpurir_sim *sim, const float *d_segments, int M_src, int segment_len,
                               const float *d_rir, int M_rcv, int rir_len, float *d_out, void *stream);

/* simulateTrajectory's convolutions and overlap-add in one call (gpuRIR does
 * the overlap-add in a Python loop, gpuRIR/__init__.py:215-219).  Segment p
 * starts at sample w_ini[p] of the signal and is w_ini[p+1] - w_ini[p] long
 * (w_ini: host array of n_pts + 1 values, w_ini[0] = 0, w_ini[n_pts] = signal
 * length); segments [n_pts][seg_len] zero-padded; RIRs [n_pts][n_rcv][rir_len].
 * Output float64 [w_ini[n_pts] + rir_len - 1][n_rcv], summed over points in
 * increasing order (compensated float32 sums).  Device buffers, stream-ordered. */
int gpurir_trajectory_device(gpurir_sim *sim, const float *d_segments, int n_pts, int seg_len,
                             const int *w_ini, const float *d_rir, int n_rcv, int rir_len,
                             double *d_out, void *stream);

/* Same with host buffers (blocking). */
int gpurir_trajectory(gpurir_sim *sim, const float *segments, int n_pts, int seg_len, const int *w_ini,
                      const float *rir, int n_rcv, int rir_len, double *out);

/* Adjoint of gpurir_trajectory_device (same segments, windows and RIRs): given
 * d_grad_out = dL/dout, float64 [w_ini[n_pts] + rir_len - 1][n_rcv], writes
 *   d_grad_signal  float32 [w_ini[n_pts]]: dL/dsignal (sample w_ini[p] + t is
 *                  sample t of segment p), and
 *   d_grad_rir     float32 [n_pts][n_rcv][rir_len]: dL/dRIR,
 * either may be NULL.  FFT correlations with the segment's spectrum (dL/dRIR)
 * and with the RIRs' spectra summed over receivers (dL/dsignal), FP32, for
 * seg_len + rir_len - 1 <= 16384.  Device buffers, stream-ordered.  gpuRIR's
 * simulateTrajectory (gpuRIR/__init__.py:177-221) is not differentiable; this
 * has no counterpart there. */
int gpurir_trajectory_adjoint_device(gpurir_sim *sim, const float *d_segments, int n_pts, int seg_len,
                                     const int *w_ini, const float *d_rir, int n_rcv, int rir_len,
                                     const double *d_grad_out, float *d_grad_signal, float *d_grad_rir,
                                     void *stream);

/* Early part of one room's RIRs without allocating any memory.  No counterpart
 * in the reference.  For callers that must not call cudaMalloc while they run:
 * real-time audio threads (cudaMalloc may block on a device synchronisation),
 * hosts with a fixed device-memory budget, work recorded under global stream
 * capture.  The kernel's scratch is a fixed ~390 KB array in this library,
 * held on every GPU that loads it until the process exits.  It holds 8192 work
 * items: a call needs M_src * M_rcv * n_seg <= 8192, where n_seg is the number
 * of segments an RIR is cut into, ceil(nSamples / S) with S the longest segment
 * one block's shared memory holds (5120 samples at 16 kHz).  Example: at 16 kHz,
 * T = 0.3 s (4800 samples, one segment) allows up to 8192 RIRs; T = 2 s (32000
 * samples, 7 segments) up to 1170.  Larger calls fail with GPURIR_ERR_INVALID
 * before anything is enqueued.  Computes the image-source part only, as
 * gpurir_simulate_rir_device with Tdiff = Tmax = T: d_rir_out is
 * [M_src][M_rcv][gpurir_n_samples(T, Fs)].  The first call on a device (and the
 * first after a device reset) looks up the scratch address
 * (cudaGetSymbolAddress); make it before any stream capture.  The call only
 * enqueues two kernels on `stream` and returns without waiting: synchronise on
 * the stream before reading d_rir_out.  Work items are built on the device from
 * sizes checked here, so the kernel never rejects one and no device status is
 * reported.  Every call shares the one scratch array: calls whose GPU work
 * overlaps (other streams, other host threads) race and must be serialised by
 * the caller. */
int gpurir_simulate_ism_noalloc(const float room_sz[3], const float beta[6], const float *d_pos_src,
                                int M_src, const float *d_pos_rcv, const float *d_orV_src,
                                const float *d_orV_rcv, int spkr_pattern, int mic_pattern, int M_rcv,
                                const int nb_img[3], float T, float Fs, float c, float *d_rir_out,
                                void *stream);

/* Reads and clears the device status word that kernels set when they reject a
 * work item (the stream-ordered entries cannot report it synchronously). */
int gpurir_device_status(gpurir_sim *sim);

/* Raw Philox4x32-10 words of the tail stream of one RIR (counter blocks
 * (j, rir_index, call_lo, call_hi), key (seed_lo, seed_hi)), into device
 * memory; for checking the stream bit-exactly against a host replay. */
int gpurir_philox_stream_device(uint64_t seed, uint64_t call_counter, uint32_t rir_index,
                                long n_words, uint32_t *d_out, void *stream);

/* Envelope of the last simulate call on this handle: per RIR (A, alpha, tau_dp)
 * as the tail used them (src/gpuRIR_cuda.cu:415-443).  `out` holds 3*n floats. */
int gpurir_last_envelope(gpurir_sim *sim, float *out, long n);

/* Whether the last gpurir_simulate_rir call stored the RIRs into the caller's
 * host buffer from the kernels (1: page-locked memory, e.g. from
 * gpurir_host_alloc) or copied them after the kernels (0: pageable memory).
 * GPURIR_HOST_DIRECT=0 in the environment forces the copy; =2 also stores
 * straight into pageable memory on a GPU that reads the host page tables
 * (GB300 over NVLink-C2C), which is slow for pages never touched before.
 * No counterpart in the reference. */
int gpurir_last_output_direct(gpurir_sim *sim, int *direct);

/* Page-locked, device-mapped host memory for result buffers (cudaHostAlloc):
 * gpurir_simulate_rir stores into it from the kernels, overlapping the
 * transfer with the computation.  No counterpart in the reference, which
 * copies every result into a fresh pageable buffer (src/gpuRIR_cuda.cu:900-915,
 * python_bind.cpp:77-86). */
int gpurir_host_alloc(size_t bytes, void **ptr);
int gpurir_host_free(void *ptr);

/* Number of kernels the last simulate call on `sim` launched (ISM kernel, plus
 * the tail kernel when some RIR spans several work items).  No counterpart in
 * the reference. */
int gpurir_last_launch_count(gpurir_sim *sim, int *kernels);

/* Kernel timing: when on, each simulate call records CUDA events on its
 * stream around the ISM kernel and the tail kernel; gpurir_last_timing waits
 * for them and returns the two durations in ms (0 for a kernel not launched).
 * No counterpart in the reference. */
int gpurir_set_profiling(gpurir_sim *sim, int on);
int gpurir_last_timing(gpurir_sim *sim, float *ism_ms, float *tail_ms);

/* Bytes the last simulate call copied host->device (descriptors, and for the
 * host entry the positions) and device->host (status word, and for the host
 * entry the RIRs).  No counterpart in the reference. */
int gpurir_last_transfer_bytes(gpurir_sim *sim, uint64_t *h2d, uint64_t *d2h);

/* Launch-shape tuning knobs, process-wide: "conv_rows" (1 or 2 RIR rows per
 * block of the convolution), "ism_blocks_per_sm" (resident blocks of the forward
 * ISM kernel, 0 = as many as fit), "adjoint_blocks_per_sm" (same for the adjoint
 * kernel), "traj_adjoint_blocks_per_sm" (trajectory adjoint, 0 = by FFT size).
 * No knob changes any result bit: they choose how work is laid out on the GPU,
 * not the arithmetic.  Batches and adjoint handles created before a change keep
 * their launch shape; simulate calls plan again.  The
 * autotuner (gpurir_gb300/tune.py) picks them per GPU and caches them on disk.
 * The reference fixes these choices at compile time (src/gpuRIR_cuda.cu:20-45). */
int gpurir_set_tuning(const char *knob, int value);
int gpurir_get_tuning(const char *knob, int *value);
int gpurir_reset_tuning(void);

/* Name of the current device with its compute capability and SM count (the key
 * of the autotuner's cache), into name[len]. */
int gpurir_device_name(char *name, int len);

/* Measured throughput of this device's FP32 FMA pipe (FLOP/s, 2 per FMA) and
 * MUFU pipe (reciprocals/s): the peaks of the sinc-accumulation roofline.
 * No counterpart in the reference (which has no roofline accounting). */
int gpurir_probe_peaks(double *fp32_flops, double *mufu_ops);

#ifdef __cplusplus
}
#endif

#endif /* GPURIR_GB300_H */
