"""The CPU oracle against hand-derived known answers of the reference's
formulas (src/gpuRIR_cuda.cu), and its Philox stream against cuRAND's host
Philox4x32-10 generator (an independent implementation of the same algorithm).
"""
import ctypes
import os

import numpy as np
import pytest

import oracle
from conftest import rel_l2


def test_lengths_use_float32_arithmetic():
    # ceil(T*Fs) in float32, then rounded up to even (src/gpuRIR_cuda.cu:831-835)
    assert oracle.n_samples(0.5, 16000) == 8000
    assert oracle.n_samples(0.3, 16000) == 4800
    assert oracle.n_samples(0.0001, 16000) == 2
    assert oracle.n_samples(1.0 / 3.0, 44100) == 14700
    for T in np.linspace(0.01, 1.3, 57):
        p = np.float32(T) * np.float32(16000)
        n = int(np.ceil(p))
        assert oracle.n_samples(T, 16000) == n + n % 2
    assert oracle.window_len(16000) == 128 and oracle.window_len(44100) == 353


def test_direct_path_amplitude_and_delay():
    room = [3.0, 4.0, 2.5]
    ps = np.array([[1.0, 1.0, 1.0]])
    pr = np.array([[2.0, 2.0, 1.5]])
    amp, tau, tdp = oracle.amp_tau(room, [0.85] * 6, ps, pr, [3, 3, 3], 16000)
    d = np.sqrt(1 + 1 + 0.25)
    direct = 1 * 9 + 1 * 3 + 1          # n = (1, 1, 1) is k = 0 on every axis
    assert abs(amp[0, 0, direct] - 1 / (4 * np.pi * d)) < 1e-15
    assert abs(tau[0, 0, direct] - d / 343 * 16000) < 1e-12
    assert tdp[0, 0] == tau[0, 0, direct]


def test_first_order_reflections_signs_and_positions():
    """k = +1 mirrors about x = L with -beta_x2; k = -1 mirrors about x = 0 with
    -beta_x1 (src/gpuRIR_cuda.cu:336-353, beta negated at :272-277)."""
    room = [4.0, 5.0, 3.0]
    beta = [0.9, 0.8, 0.7, 0.6, 0.5, 0.4]
    ps = np.array([[1.0, 2.0, 1.5]])
    pr = np.array([[3.0, 2.5, 1.0]])
    amp, tau, _ = oracle.amp_tau(room, beta, ps, pr, [3, 1, 1], 16000)
    # nb_img = [3, 1, 1]: n0 = 0 -> k = -1, n0 = 1 -> k = 0, n0 = 2 -> k = 1
    img_m1 = np.array([-1.0, 2.0, 1.5])          # mirror about x = 0
    img_p1 = np.array([2 * 4.0 - 1.0, 2.0, 1.5])  # mirror about x = L
    f32 = lambda v: float(np.float32(v))   # the oracle, like gpuRIR, takes float32 inputs
    for n, img, b in ((0, img_m1, -f32(0.9)), (2, img_p1, -f32(0.8))):
        d = np.linalg.norm(img - pr[0])
        assert abs(amp[0, 0, n] - b / (4 * np.pi * d)) < 1e-15
        assert abs(tau[0, 0, n] - d / 343 * 16000) < 1e-12


def test_second_order_and_even_counts():
    room = [4.0, 5.0, 3.0]
    beta = [0.9, 0.8, 0.7, 0.6, 0.5, 0.4]
    ps = np.array([[1.0, 2.0, 1.5]])
    pr = np.array([[3.0, 2.5, 1.0]])
    amp, tau, _ = oracle.amp_tau(room, beta, ps, pr, [1, 1, 4], 16000)
    # N = 4: n = 0..3 -> k = -2..1; k = -2: clust -1, refl 0: z = -2L + s, att beta_z1*beta_z2
    z = [-2 * 3.0 + 1.5, -1.5, 1.5, 2 * 3.0 - 1.5]
    f32 = lambda v: float(np.float32(v))
    att = [f32(0.5) * f32(0.4), -f32(0.5), 1.0, -f32(0.4)]
    for n in range(4):
        d = np.linalg.norm(np.array([1.0, 2.0, z[n]]) - pr[0])
        assert abs(amp[0, 0, n] - att[n] / (4 * np.pi * d)) < 1e-15


@pytest.mark.parametrize("pattern,gain", [("homni", lambda c: float(c > 0)),
                                          ("card", lambda c: 0.5 + 0.5 * c),
                                          ("hypcard", lambda c: 0.25 + 0.75 * c),
                                          ("subcard", lambda c: 0.75 + 0.25 * c),
                                          ("bidir", lambda c: c)])
def test_directivity_of_direct_path(pattern, gain):
    room = [4.0, 5.0, 3.0]
    ps = np.array([[1.0, 2.0, 1.5]])
    pr = np.array([[3.0, 2.5, 1.0]])
    orv = np.array([[0.3, -0.2, 0.9]]).astype(np.float32).astype(np.float64)
    v = ps[0] - pr[0]                       # receiver -> source
    d = np.linalg.norm(v)
    c_mic = v @ orv[0] / d / np.linalg.norm(orv[0])
    amp, _, _ = oracle.amp_tau(room, [0.5] * 6, ps, pr, [1, 1, 1], 16000, mic_pattern=pattern,
                               orV_rcv=orv)
    assert abs(amp[0, 0, 0] - gain(c_mic) / (4 * np.pi * d)) < 1e-15
    c_src = -v @ orv[0] / d / np.linalg.norm(orv[0])   # source axis vs source -> receiver
    amp, _, _ = oracle.amp_tau(room, [0.5] * 6, ps, pr, [1, 1, 1], 16000, spkr_pattern=pattern,
                               orV_src=orv)
    assert abs(amp[0, 0, 0] - gain(c_src) / (4 * np.pi * d)) < 1e-15


def test_windowed_sinc_single_image():
    """One image: h[t] = amp * 0.5(1 + cos(2 pi x/Tw)) * sinc(x), x = t - tau, |x| < Tw/2."""
    amp = np.array([[0.37]])
    tau = np.array([[100.3]])
    h = oracle.ism_sum(amp, tau, 300, 16000)[0]
    t = np.arange(300)
    x = t - 100.3
    want = np.where(np.abs(x) < 64, 0.37 * 0.5 * (1 + np.cos(2 * np.pi * x / 128)) * np.sinc(x), 0)
    assert np.abs(h - want).max() < 1e-15
    # on a sample: a single non-zero tap
    h = oracle.ism_sum(amp, np.array([[100.0]]), 300, 16000)[0]
    assert h[100] == 0.37 and np.count_nonzero(np.abs(h) > 1e-15) == 1


def test_sabine_t60_and_envelope():
    room = [6.0, 5.0, 3.0]
    beta = [0.9] * 6
    Sa = 2 * (1 - 0.81) * (5 * 3 + 6 * 3 + 6 * 5)
    assert abs(oracle.sabine_t60(room, beta) - 0.161 * 90 / Sa) < 1e-6
    # envelope: constant early power -> A = P / exp(alpha (w_center - tau_dp))
    n_ism = 1000
    rir = np.zeros((1, n_ism))
    rir[0, 840:] = 0.01
    A, al = oracle.env_pred(rir, np.array([100.0]), n_ism, 16000, room, beta)
    t60 = oracle.sabine_t60(room, beta)
    alpha = -13.8155 / (t60 * 16000)
    assert abs(al[0] - alpha) < 1e-15
    assert abs(A[0] - 1e-4 / np.exp(alpha * (920.0 - 100.0))) < 1e-15


def test_fp32_port_close_to_fp64():
    rng = np.random.default_rng(0)
    room = [3.0, 4.0, 2.5]
    ps = (0.5 + rng.random((1, 3)) * 2).astype(np.float32)
    pr = (0.5 + rng.random((2, 3)) * 1.5).astype(np.float32)
    f32, upd = oracle.ism_f32(room, [0.85] * 6, ps, pr, [11, 9, 13], 0.5, 16000.0)
    f64 = oracle.simulate_rir(room, [0.85] * 6, ps, pr, [11, 9, 13], 0.5, 16000.0)
    # float32 delays (|tau| up to ~1300 samples) bound the port's agreement
    assert rel_l2(f32, f64) < 5e-4
    amp, tau, _ = oracle.amp_tau(room, [0.85] * 6, ps, pr, [11, 9, 13], 16000.0)
    assert upd == oracle.windowed_updates(tau, 8000, 16000.0)


def _curand():
    for p in ("/usr/local/cuda/lib64/libcurand.so", "libcurand.so", "libcurand.so.10"):
        try:
            return ctypes.CDLL(p)
        except OSError:
            continue
    return None


def test_philox_matches_curand_host_generator():
    """cuRAND's host Philox4x32-10 emits block i of a seed from counter
    (0, 0, i, 0) and key (seed_lo, seed_hi); the oracle must reproduce it."""
    L = _curand()
    if L is None:
        pytest.skip("libcurand not available")
    for seed in (0, 1234, 0x123456789ABCDEF, 2**64 - 1):
        gen = ctypes.c_void_p()
        assert L.curandCreateGeneratorHost(ctypes.byref(gen), 161) == 0   # PHILOX4_32_10
        assert L.curandSetPseudoRandomGeneratorSeed(gen, ctypes.c_ulonglong(seed)) == 0
        n = 4 * 257
        out = np.zeros(n, dtype=np.uint32)
        assert L.curandGenerate(gen, out.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(n)) == 0
        L.curandDestroyGenerator(gen)
        key = [seed & 0xFFFFFFFF, seed >> 32]
        want = np.concatenate([oracle.philox4x32_10([0, 0, i, 0], key) for i in range(n // 4)])
        assert np.array_equal(out, want)


def test_philox_counter_words_all_exercised():
    # the tail stream puts the sample block in word 0 and the RIR in word 1
    a = oracle.tail_stream(7, 0, 0, 8)
    assert np.array_equal(a[:4], oracle.philox4x32_10([0, 0, 0, 0], [7, 0]))
    assert np.array_equal(a[4:], oracle.philox4x32_10([1, 0, 0, 0], [7, 0]))
    b = oracle.tail_stream(7, 2**33 + 5, 9, 4)
    assert np.array_equal(b, oracle.philox4x32_10([0, 9, 5, 2], [7, 0]))


def test_tail_statistics():
    """Logistic noise of unit variance (0.551329 = sqrt(3)/pi); Gaussian option."""
    M, n = 1, 200000
    A = np.ones(M)
    al = np.zeros(M)
    tdp = np.zeros(M)
    for kind, kurt in ((0, 4.2), (1, 3.0)):
        out = np.zeros((M, n))
        oracle.lib().orc_tail(oracle.oracle._p(A, ctypes.c_double), oracle.oracle._p(al, ctypes.c_double),
                              oracle.oracle._p(tdp, ctypes.c_double), M, 0, n, 3, 0, None, kind,
                              oracle.oracle._p(out, ctypes.c_double), n)
        z = out[0]
        assert abs(z.mean()) < 0.01
        assert abs(z.var() - 1.0) < 0.02
        k = ((z - z.mean()) ** 4).mean() / z.var() ** 2
        assert abs(k - kurt) < 0.2


def test_torch_fp64_reference_matches_oracle():
    """The differentiable FP64 torch transcription used for the adjoint checks
    agrees with the C oracle."""
    import torch
    from torch_ism_ref import early_part
    rng = np.random.default_rng(7)
    room = np.array([4.0, 3.5, 2.8], dtype=np.float32)
    ps = (0.5 + rng.random((2, 3)) * 2.5).astype(np.float32)
    pr = (0.5 + rng.random((2, 3)) * 2.0).astype(np.float32)
    os_ = rng.standard_normal((2, 3)).astype(np.float32)
    or_ = rng.standard_normal((2, 3)).astype(np.float32)
    beta = rng.uniform(0.6, 0.95, 6).astype(np.float32)
    t = lambda a: torch.tensor(np.asarray(a, dtype=np.float64))
    h = early_part(room, t(beta), t(ps), t(pr), [5, 6, 7], 960, 16000.0, spkr="card", mic="bidir",
                   orV_src=t(os_), orV_rcv=t(or_)).numpy()
    ref = oracle.simulate_rir(room, beta, ps, pr, [5, 6, 7], 0.06, 16000.0, spkr_pattern="card",
                              mic_pattern="bidir", orV_src=os_, orV_rcv=or_)
    assert np.abs(h - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("timestamps,fs", [(None, None), ([0.0, 0.7, 1.9, 3.2], 20.0)])
def test_trajectory_adjoint_is_the_transpose(timestamps, fs):
    """The FP64 adjoint of the trajectory filter satisfies <G, J v> = <J^T G, v>
    for perturbations of the signal and of the RIRs (the filter is bilinear)."""
    rng = np.random.default_rng(3)
    P, R, L, n = 4, 3, 37, 103
    sig = rng.standard_normal(n).astype(np.float32)
    h = rng.standard_normal((P, R, L)).astype(np.float32)
    y = oracle.trajectory(sig, h, timestamps, fs)
    G = rng.standard_normal(y.shape)
    gs, gr = oracle.trajectory_adjoint(sig, h, G, timestamps, fs)
    ds = rng.standard_normal(n).astype(np.float32)
    dh = rng.standard_normal((P, R, L)).astype(np.float32)
    lhs_s = np.sum(G * oracle.trajectory(ds, h, timestamps, fs))
    lhs_h = np.sum(G * oracle.trajectory(sig, dh, timestamps, fs))
    assert abs(lhs_s - np.dot(gs, ds)) <= 1e-10 * max(1.0, abs(lhs_s))
    assert abs(lhs_h - np.sum(gr * dh)) <= 1e-10 * max(1.0, abs(lhs_h))
