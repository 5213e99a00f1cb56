"""The two other evaluation modes of gpuRIR's API on the GPU.

activateMixedPrecision: half2 window, FP32 reciprocal and accumulation; the
  early part within 2e-3 relative L2 of the FP64 oracle.
activateLUT: gpuRIR's lookup-table semantics (16x oversampled Hann x sinc,
  8-bit interpolation weight, support |t - tau| < Tw/2 in integers); within
  1e-5 relative L2 of the oracle's restatement of those semantics, and within
  the table's own accuracy (5e-3) of the exact FP64 result.
"""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _scene(seed, fs=16000.0):
    rng = np.random.default_rng(seed)
    room = np.array([5.0, 4.0, 3.0], np.float32)
    ps = (0.5 + rng.random((3, 3)) * 4.0 * np.array([1, 0.75, 0.5])).astype(np.float32)
    pr = (0.5 + rng.random((4, 3)) * 3.0 * np.array([1, 0.9, 0.6])).astype(np.float32)
    orv = rng.standard_normal((4, 3)).astype(np.float32)
    return room, rng.uniform(0.7, 0.95, 6).astype(np.float32), ps, pr, orv


def _run(mode, seed, fs=16000.0, nb=(7, 7, 9), T=0.12):
    import gpurir_gb300 as G
    room, beta, ps, pr, orv = _scene(seed, fs)
    sim = G.Simulator()
    if mode == "mp":
        assert sim.activate_mixed_precision(True)
    elif mode == "lut":
        assert sim.activate_lut(True)
    out = sim.simulate_rir(room, beta, ps, pr, None, orv, 0, 2, nb, T, T, fs)
    amp, tau, _ = oracle.amp_tau(room, beta, ps, pr, nb, fs, mic_pattern="card", orV_rcv=orv)
    n = oracle.n_samples(T, fs)
    exact = oracle.ism_sum(amp.reshape(12, -1), tau.reshape(12, -1), n, fs)
    lut = oracle.ism_sum_lut(amp.reshape(12, -1), tau.reshape(12, -1), n, fs)
    return out.reshape(12, -1), exact, lut


@pytest.mark.parametrize("fs", [16000.0, 44100.0])
def test_mixed_precision_within_2e3(built, fs):
    out, exact, _ = _run("mp", 50, fs)
    e = rel_l2(out, exact)
    assert e <= 2e-3, e


@pytest.mark.parametrize("fs", [16000.0, 22050.0, 44100.0])
def test_lut_mode_matches_gpuRIR_lut_semantics(built, fs):
    out, exact, lut = _run("lut", 51, fs)
    assert rel_l2(out, lut) <= 1e-5
    assert rel_l2(lut, exact) <= 5e-3
    assert rel_l2(out, exact) <= 5e-3


def test_mode_flags_exclude_each_other(built):
    import gpurir_gb300 as G
    sim = G.Simulator()
    assert sim.modes() == dict(mixed_precision=False, lut=False, reference_delays=False)
    sim.activate_lut(True)
    sim.activate_mixed_precision(True)
    assert sim.modes() == dict(mixed_precision=True, lut=False, reference_delays=False)
    sim.activate_lut(True)
    assert sim.modes() == dict(mixed_precision=False, lut=True, reference_delays=False)
    sim.activate_lut(False)
    assert sim.modes() == dict(mixed_precision=False, lut=False, reference_delays=False)
    # the delay model is independent of the evaluation mode
    sim.activate_reference_delays(True)
    sim.activate_mixed_precision(True)
    assert sim.modes() == dict(mixed_precision=True, lut=False, reference_delays=True)
    sim.activate_reference_delays(False)
    assert sim.modes() == dict(mixed_precision=True, lut=False, reference_delays=False)


def _long_room_errors(T, mode, policy):
    import gpurir_gb300 as G
    room = [4.0, 3.0, 2.5]
    ps = np.array([[1.1, 1.3, 1.2]], np.float32)
    pr = np.array([[2.9, 1.9, 1.4], [3.3, 0.8, 1.9]], np.float32)
    beta, fs = [0.97] * 6, 16000.0
    nb = [int(np.ceil(2 * 343 * T / d)) for d in room]
    amp, tau, _ = oracle.amp_tau(room, beta, ps, pr, nb, fs)
    n = oracle.n_samples(T, fs)
    a, t = amp.reshape(2, -1), tau.reshape(2, -1)
    want = oracle.ism_sum_lut(a, t, n, fs) if mode == "lut" else oracle.ism_sum(a, t, n, fs)
    sim = G.Simulator(mixed_precision=(mode == "mp"), lut=(mode == "lut"))
    sim.set_compensation(policy)
    got = sim.simulate_rir(room, beta, ps, pr, None, None, 0, 0, nb, T, T, fs).reshape(2, -1)
    q = 3 * n // 4   # the last quarter: the densest samples
    return rel_l2(got[:, q:], want[:, q:])


def test_compensated_accumulation_on_long_dense_rirs(built):
    """A small, reverberant room with every image up to T (nb_img = t2n(T)): at
    0.75 s the lookup-table mode's error late in the RIR, with compensated
    accumulation (the default for long RIRs), stays where it is at 0.25 s and
    below the uncompensated error; mixed precision is flat in T (its FP32
    accumulation never was the bottleneck)."""
    lut_short = _long_room_errors(0.25, "lut", 1)
    lut_long = _long_room_errors(0.75, "lut", 1)
    lut_long_plain = _long_room_errors(0.75, "lut", 0)
    mp_short = _long_room_errors(0.25, "mp", 1)
    mp_long = _long_room_errors(0.75, "mp", 2)
    print("lut %.2e -> %.2e (plain %.2e), mp %.2e -> %.2e" % (lut_short, lut_long, lut_long_plain, mp_short,
                                                           mp_long))
    assert lut_long <= 1.3 * lut_short
    assert lut_long < lut_long_plain
    assert mp_long <= 1.2 * mp_short


@pytest.mark.parametrize("mode", ["lut", "mp"])
def test_image_exactly_on_sample_in_each_mode(built, mode):
    """Direct path of exactly 50 samples (c = 320 m/s, fs = 16 kHz, 1 m apart): in
    lookup-table mode the taps at |t - tau| = Tw/2 stay outside the support."""
    import gpurir_gb300 as G
    room = np.array([4.0, 4.0, 3.0], np.float32)
    ps = np.array([[1.0, 2.0, 1.5]], dtype=np.float32)
    pr = np.array([[2.0, 2.0, 1.5]], dtype=np.float32)
    nb, T, fs, c = (3, 3, 3), 0.05, 16000.0, 320.0
    sim = G.Simulator()
    assert (sim.activate_lut(True) if mode == "lut" else sim.activate_mixed_precision(True))
    out = sim.simulate_rir(room, [0.7] * 6, ps, pr, None, None, 0, 0, nb, T, T, fs, c=c)
    amp, tau, _ = oracle.amp_tau(room, [0.7] * 6, ps, pr, nb, fs, c=c)
    assert abs(tau.reshape(-1)[np.argmin(tau)] - 50.0) < 1e-9
    n = oracle.n_samples(T, fs)
    exact = oracle.ism_sum(amp.reshape(1, -1), tau.reshape(1, -1), n, fs)
    if mode == "lut":
        lut = oracle.ism_sum_lut(amp.reshape(1, -1), tau.reshape(1, -1), n, fs)
        assert rel_l2(out.reshape(1, -1), lut) <= 1e-5
    else:
        assert rel_l2(out.reshape(1, -1), exact) <= 2e-3
