"""GPU checks of the hand-written FFT convolution (gpu_conv) and of
simulateTrajectory (convolution + on-device overlap-add) against FP64 direct
convolution and against the reference's own overlap-add (golden vectors).

Tolerance: max-abs error <= 2e-6 of the output's peak (float32 FFT of length
N = pow2roundup(S + L - 1), as gpuRIR's cuFFT path)."""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _direct(seg, rir):
    P, S = seg.shape
    _, R, L = rir.shape
    out = np.zeros((P, R, S + L - 1))
    for p in range(P):
        for r in range(R):
            out[p, r] = np.convolve(seg[p].astype(np.float64), rir[p, r].astype(np.float64))
    return out


@pytest.mark.parametrize("P,S,R,L", [(3, 5, 2, 4), (7, 401, 3, 257), (4, 1000, 2, 3000),
                                     (2, 400, 8, 12800), (2, 3000, 2, 14000), (1, 1, 1, 1),
                                     (5, 64, 1, 65), (3, 700, 1, 1500), (5, 400, 3, 12800)])
def test_gpu_conv_matches_direct(built, P, S, R, L):
    """Covers shared-memory FFTs (N <= 16384) and global-scratch FFTs (N = 32768); the
    register kernels transform two rows per block, so odd row counts (a last block with
    one row) and pairs of rows from different points are included."""
    from gpurir_gb300.trajectory import gpu_conv
    rng = np.random.default_rng(P * 1000 + S)
    seg = rng.standard_normal((P, S)).astype(np.float32)
    rir = (rng.standard_normal((P, R, L)) * np.exp(-np.arange(L) / (L / 4 + 1))).astype(np.float32)
    got = gpu_conv(seg, rir)
    want = _direct(seg, rir)
    assert got.shape == want.shape and got.dtype == np.float32
    assert np.abs(got - want).max() <= 2e-6 * np.abs(want).max()


@pytest.mark.parametrize("custom", [False, True])
def test_simulate_trajectory_matches_reference_golden(built, custom):
    import gpurir_gb300 as G
    g = np.load(os.path.join(HERE, "golden", "reference_python.npz"))
    if custom:
        got = G.simulateTrajectory(g["traj_signal"], g["traj_rirs"], g["traj_custom_ts"], 16000)
        want = g["traj_custom"]
    else:
        got = G.simulateTrajectory(g["traj_signal"], g["traj_rirs"])
        want = g["traj_default"]
    assert got.dtype == np.float64 and got.shape == want.shape
    assert np.abs(got - want).max() <= 2e-6 * np.abs(want).max()


def test_trajectory_workload_scale(built):
    """The moving-source workload's shapes (400 points, 8 mics, 12800-sample RIRs,
    10 s of signal), host and device paths, against FP64 direct convolution + OLA."""
    import torch
    import gpurir_gb300 as G
    rng = np.random.default_rng(4)
    n_pts, R, L = 400, 8, 12800
    sig = rng.standard_normal(160000).astype(np.float32)
    rirs = (rng.standard_normal((n_pts, R, L)) * np.exp(-np.arange(L) / 2000.0) * 0.1).astype(np.float32)
    got = G.simulateTrajectory(sig, rirs)
    want = oracle.trajectory(sig, rirs)
    assert got.shape == (160000 + L - 1, R)
    assert np.abs(got - want).max() <= 2e-6 * np.abs(want).max()
    dev = G.simulateTrajectory(sig, torch.from_numpy(rirs).cuda())
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), got)


def test_trajectory_rejects_bad_timestamps(built):
    import gpurir_gb300 as G
    sig = np.ones(100, np.float32)
    rirs = np.ones((3, 1, 5), np.float32)
    with pytest.raises(AssertionError):
        G.simulateTrajectory(sig, rirs, timestamps=np.array([0.0, 0.5, 0.2]))   # fs missing
    with pytest.raises(AssertionError):
        G.simulateTrajectory(sig, rirs, timestamps=np.array([0.1, 0.2, 0.3]), fs=100)
