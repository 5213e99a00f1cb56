"""Moving-source filtering: simulateTrajectory (gpuRIR/__init__.py:177-221).

The signal is cut into one segment per trajectory point, each segment is
convolved with the RIRs of its point, and the convolutions are overlap-added.
gpuRIR does the convolutions with cuFFT (src/gpuRIR_cuda.cu:933-1023) and the
overlap-add as a Python double loop in float64; here both run on the GPU in
hand-written FFT kernels behind the C ABI (gpurir_trajectory_*).
"""
import numpy as np


def segment_signal(source_signal, n_pts, timestamps=None, fs=None):
    """Segmentation of gpuRIR/__init__.py:198-213.

    Returns (segments float32 [n_pts, max_len], w_ini int [n_pts + 1], w_len int [n_pts]).
    """
    n = len(source_signal)
    assert timestamps is None or fs is not None, "fs must be indicated for custom timestamps"
    assert timestamps is None or timestamps[0] == 0, "The first timestamp must be 0"
    if timestamps is None:
        fs = n / n_pts
        timestamps = np.arange(n_pts)
    w_ini = np.append((np.asarray(timestamps) * fs).astype(int), n)
    w_len = np.diff(w_ini)
    segments = np.zeros((n_pts, w_len.max()))
    for p in range(n_pts):
        segments[p, 0:w_len[p]] = source_signal[w_ini[p]:w_ini[p + 1]]
    return segments.astype('float32', order='C', copy=False), w_ini, w_len


def simulate_trajectory(source_signal, RIRs, timestamps=None, fs=None):
    raise NotImplementedError("simulateTrajectory: the GPU convolution kernels are not built yet")
