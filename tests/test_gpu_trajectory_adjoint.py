"""Adjoint of simulateTrajectory on the GPU (gpurir_trajectory_adjoint_device
through gpurir_gb300.trajectory.simulate_trajectory_torch).

  * dL/dsignal and dL/dRIRs against the FP64 oracle's direct correlations
    (oracle.trajectory_adjoint), for back-to-back and for custom timestamps,
    short RIRs (the FFT is padded to N = 2048) and the trajectory workload's
    12800-sample RIRs (N = 16384); tolerance: relative L2 <= 2e-6 (float32 FFT).
  * The chain into the image-source adjoint: dL/dbeta of a loss of the filtered
    signal, RIRs from the differentiable batch (gpurir_gb300.autograd), against
    FP64 central differences (step 2^-17 ~ 1e-5, exact in float32) of the same
    loss computed by the FP64 oracle end to end; tolerance 2e-3 relative.
"""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _case(seed, P, R, L, n, timestamps=None, fs=None):
    import torch
    rng = np.random.default_rng(seed)
    sig = rng.standard_normal(n).astype(np.float32)
    rir = (rng.standard_normal((P, R, L)) * np.exp(-np.arange(L) / (L / 4 + 1))).astype(np.float32)
    dev = torch.device("cuda")
    ts = torch.from_numpy(sig).to(dev).requires_grad_(True)
    tr = torch.from_numpy(rir).to(dev).requires_grad_(True)
    return sig, rir, ts, tr, rng


@pytest.mark.parametrize("P,R,L,n,timestamps,fs", [
    (6, 3, 37, 300, None, None),                        # back to back, N = 2048 (padded)
    (5, 2, 200, 1000, [0.0, 0.13, 0.2, 0.55, 0.71], 1000.0),   # uneven segments
    (7, 1, 1500, 3500, None, None),                     # odd point count, N = 4096
    (12, 8, 12800, 4800, None, None),                   # the trajectory workload's RIRs, N = 16384
])
def test_trajectory_adjoint_matches_oracle(built, P, R, L, n, timestamps, fs):
    import torch
    from gpurir_gb300.trajectory import simulate_trajectory_torch
    sig, rir, ts, tr, rng = _case(P * 100 + L, P, R, L, n, timestamps, fs)
    y = simulate_trajectory_torch(ts, tr, timestamps, fs)
    y_ref = oracle.trajectory(sig, rir, timestamps, fs)
    assert rel_l2(y.detach().cpu().numpy(), y_ref) < 2e-6
    G = rng.standard_normal(y_ref.shape)
    y.backward(torch.from_numpy(G).to(y.device))
    gs_ref, gr_ref = oracle.trajectory_adjoint(sig, rir, G, timestamps, fs)
    gs, gr = ts.grad.cpu().numpy(), tr.grad.cpu().numpy()
    assert rel_l2(gs, gs_ref) < 2e-6, rel_l2(gs, gs_ref)
    assert rel_l2(gr, gr_ref) < 2e-6, rel_l2(gr, gr_ref)


def test_trajectory_adjoint_only_requested_gradients(built):
    """Only the RIRs require grad: the signal gradient is not formed (and the
    other way round), with the same values as when both are formed."""
    import torch
    from gpurir_gb300.trajectory import simulate_trajectory_torch
    sig, rir, ts, tr, rng = _case(5, 4, 2, 300, 800)
    G = torch.from_numpy(rng.standard_normal((800 + 299, 2))).cuda()
    y = simulate_trajectory_torch(ts, tr)
    y.backward(G)
    both_s, both_r = ts.grad.clone(), tr.grad.clone()
    ts2 = ts.detach().clone()
    tr2 = tr.detach().clone().requires_grad_(True)
    simulate_trajectory_torch(ts2, tr2).backward(G)
    assert torch.equal(tr2.grad, both_r)
    ts3 = ts.detach().clone().requires_grad_(True)
    simulate_trajectory_torch(ts3, tr.detach()).backward(G)
    assert torch.equal(ts3.grad, both_s)


def _loss_fp64(beta, scene, sig, wts):
    rirs = oracle.simulate_rir(scene["room_sz"], beta, scene["pos_src"], scene["pos_rcv"], scene["nb_img"],
                               scene["Tmax"], scene["fs"])
    y = oracle.trajectory(sig, rirs)
    return float(np.sum(wts * y))


def test_trajectory_beta_gradient_central_differences(built):
    """Loss = sum(w * trajectory(signal, RIRs(beta))): the autograd gradient
    through the trajectory adjoint and the image-source adjoint against FP64
    central differences of the oracle pipeline."""
    import torch
    from gpurir_gb300.autograd import TorchBatch
    from gpurir_gb300.trajectory import simulate_trajectory_torch
    rng = np.random.default_rng(11)
    room = np.array([5.0, 4.0, 3.0], np.float32)
    P, R, fs, T = 6, 2, 16000.0, 0.05
    t = np.linspace(0.1, 0.9, P)[:, None]
    ps = (np.array([1.0, 1.0, 1.5]) * (1 - t) + np.array([4.0, 3.0, 1.5]) * t).astype(np.float32)
    pr = (0.5 + rng.random((R, 3)) * (room - 1.0)).astype(np.float32)
    # walls on a 2^-17 grid: beta +- h is exact in the oracle's float32 inputs
    beta = (np.round(rng.uniform(0.7, 0.9, 6) * 2 ** 17) / 2 ** 17).astype(np.float32)
    scene = dict(room_sz=room, pos_src=ps, pos_rcv=pr, nb_img=[5, 5, 5], Tmax=T, Tdiff=T, fs=fs)
    n = 600
    sig = rng.standard_normal(n).astype(np.float32)
    L = oracle.n_samples(T, fs)
    wts = rng.standard_normal((n + L - 1, R))
    model = TorchBatch([dict(scene, beta=beta, spkr_pattern="omni", mic_pattern="omni")], fs)
    dev = torch.device("cuda")
    b = torch.from_numpy(beta).to(dev).reshape(1, 6).requires_grad_(True)
    rirs = model(b, torch.from_numpy(ps).to(dev), torch.from_numpy(pr).to(dev)).view(P, R, L)
    y = simulate_trajectory_torch(torch.from_numpy(sig).to(dev), rirs)
    (y * torch.from_numpy(wts).to(dev)).sum().backward()
    got = b.grad.cpu().numpy().ravel().astype(np.float64)
    h = 2.0 ** -17   # ~7.6e-6: the central-difference step
    want = np.zeros(6)
    for w in range(6):
        bp, bm = beta.astype(np.float64).copy(), beta.astype(np.float64).copy()
        bp[w] += h
        bm[w] -= h
        want[w] = (_loss_fp64(bp, scene, sig, wts) - _loss_fp64(bm, scene, sig, wts)) / (2 * h)
    assert np.abs(got - want).max() <= 2e-3 * np.abs(want).max(), (got, want)
