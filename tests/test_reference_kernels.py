"""Parity against gpuRIR's own CUDA kernels.

tests/golden/reference_kernels.npz holds the outputs of the reference's kernels
(src/gpuRIR_cuda.cu, compiled from its sources and run on a GB300 by
tests/golden/make_reference_kernels.py) for seeded scenes: image amplitudes and
delays, the early part in FP32 / mixed-precision / lookup-table modes, the
envelope and the diffuse transform of fixed uniforms.

CPU tests pin the oracle to those outputs stage by stage: fed the reference's
own amplitudes and delays, the oracle's windowed sum, lookup-table fetch,
envelope and tail transform agree with the reference to float32 rounding.  The
remaining difference of the full pipeline is the reference's float32 delay
(dist / c * Fs in single precision, up to ~4e-4 samples off at 0.3 s), which
the oracle and the engine compute more accurately.

The engine's reference-delay mode rounds each delay in float32 as the
reference's kernel does (bit for bit, pinned here on every scene); with it the
engine matches the reference's FP32 and LUT outputs within 1e-5 relative L2 and
its half2 output within 2e-3.  GPU tests compare the engine with the same
outputs, and (when oracle/_ref/gpuRIR_ref.cubin is present) with the
reference's kernels run live on random scenes.
"""
import json
import os

import numpy as np
import pytest

import oracle
from oracle import ref_kernels

from conftest import rel_l2

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "reference_kernels.npz")
INV = {v: k for k, v in oracle.PATTERNS.items()}


def _load():
    Z = np.load(FIX)
    meta = json.loads(bytes(Z["meta_json"]).decode())
    scenes = {}
    for name, m in meta.items():
        sc = dict(m)
        for key in ("room_sz", "beta", "pos_src", "pos_rcv", "orV_src", "orV_rcv"):
            k = "%s/in/%s" % (name, key)
            sc[key] = Z[k] if k in Z.files else None
        sc["spkr_pattern"] = int(m.get("spkr_pattern", 0))
        sc["mic_pattern"] = int(m.get("mic_pattern", 0))
        out = {k.split("/", 1)[1]: Z[k] for k in Z.files if k.startswith(name + "/") and "/in/" not in k}
        scenes[name] = (sc, out)
    return scenes


SCENES = _load()


def _amp_tau(sc):
    return oracle.amp_tau(sc["room_sz"], sc["beta"], sc["pos_src"], sc["pos_rcv"], sc["nb_img"], sc["fs"],
                          INV[sc["spkr_pattern"]], INV[sc["mic_pattern"]], sc["orV_src"], sc["orV_rcv"])


def test_fixture_covers_modes_and_patterns():
    names = set(SCENES)
    assert {"plain", "tail", "fs48k", "fs44k1"} <= names
    pats = {(sc["spkr_pattern"], sc["mic_pattern"]) for sc, _ in SCENES.values()}
    assert {p for pair in pats for p in pair} == set(range(6))
    modes = {m for sc, _ in SCENES.values() for m in sc["modes"]}
    assert modes == {"fp32", "mp", "lut"}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_amp_tau_matches_reference_kernel(name):
    """calcAmpTau_kernel (:245-375) vs the FP64 restatement: the reference's
    float32 rounding only."""
    sc, out = SCENES[name]
    amp, tau, tdp = _amp_tau(sc)
    ra, rt = out["amp"].astype(np.float64), out["tau"].astype(np.float64)
    big = np.abs(amp) > 1e-3 * np.abs(amp).max()
    assert np.max(np.abs(ra - amp)[big] / np.abs(amp)[big]) < 2e-4
    assert np.max(np.abs(rt - tau) / tau) < 1e-6
    assert np.max(np.abs(out["tau_dp"] - tdp) / tdp) < 1e-6


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_windowed_sum_matches_reference_kernel(name):
    """generateRIR_kernel + reduceRIR_kernel (:377-413, 618-674) on the
    reference's own amplitudes and delays vs the oracle's FP64 windowed sum."""
    sc, out = SCENES[name]
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    got = oracle.ism_sum(out["amp"], out["tau"], n, sc["fs"])
    assert rel_l2(out["fp32/early"].reshape(got.shape), got) < 1e-6


@pytest.mark.parametrize("name", [n for n in sorted(SCENES) if "lut" in SCENES[n][0]["modes"]])
def test_oracle_lut_matches_reference_kernel(name):
    """generateRIR_kernel_lut (:559-572) with the texture of
    create_sinc_texture_lut (:574-611) vs the oracle's float restatement of
    the fetch and of the texture unit's 8-bit filter weight."""
    sc, out = SCENES[name]
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    got = oracle.ism_sum_lut(out["amp"], out["tau"], n, sc["fs"])
    ref = out["lut/early"].reshape(got.shape)
    assert rel_l2(ref, got) < 5e-7
    assert np.abs(ref - got).max() < 1e-7


def test_reference_mixed_precision_error():
    """The reference's half2 path (:488-553, 676-734) accumulates in half
    precision: ~1e-3 from the exact sum.  Recorded here as the bar that the
    engine's mixed-precision mode (FP32 accumulation) beats."""
    sc, out = SCENES["plain"]
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    exact = oracle.ism_sum(out["amp"], out["tau"], n, sc["fs"])
    err = rel_l2(out["mp/early"].reshape(exact.shape), exact)
    assert 2e-4 < err < 5e-3


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_envelope_matches_reference_kernel(name):
    """envPred_kernel (:415-443) on the reference's early part and tau_dp."""
    sc, out = SCENES[name]
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    early = out["fp32/early"].reshape(-1, n)
    A, al = oracle.env_pred(early, out["tau_dp"].ravel(), n, sc["fs"], sc["room_sz"], sc["beta"])
    rA, ral = out["A"].ravel().astype(np.float64), out["alpha"].ravel().astype(np.float64)
    assert np.all(np.abs(rA - A) <= 5e-6 * np.abs(A) + 1e-30)
    assert np.all(np.abs(ral - al) <= 1e-6 * np.abs(al))


def test_oracle_diffuse_transform_matches_reference_kernel():
    """diffRev_kernel (:445-461) on fixed uniforms (cuRAND is not replayed)."""
    sc, out = SCENES["tail"]
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    d = out["diffuse"]
    u = ref_kernels.hash_uniforms(d.size)
    got = oracle.diffuse_from_uniforms(out["A"], out["alpha"], out["tau_dp"], n, u)
    assert rel_l2(d.reshape(got.shape), got) < 1e-6


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_pipeline_vs_reference_kernels(name):
    """Whole early part from the oracle's own FP64 geometry vs the reference:
    bounded by the reference's float32 delays (the windowed sum alone agrees
    to float32 rounding, above)."""
    sc, out = SCENES[name]
    amp, tau, _ = _amp_tau(sc)
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    got = oracle.ism_sum(amp, tau, n, sc["fs"])
    assert rel_l2(out["fp32/early"].reshape(got.shape), got) < 2e-4


def _tau_ref(sc):
    return oracle.tau_reference_f32(sc["room_sz"], sc["pos_src"], sc["pos_rcv"], sc["nb_img"], sc["fs"],
                                    INV[sc["spkr_pattern"]], INV[sc["mic_pattern"]])


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_reference_delays_bit_exact(name):
    """The float32 delay model (the engine's reference-delay mode) reproduces
    every delay and direct-path delay calcAmpTau_kernel wrote, bit for bit."""
    sc, out = SCENES[name]
    tau, tdp = _tau_ref(sc)
    assert np.array_equal(tau, out["tau"].reshape(tau.shape))
    assert np.array_equal(tdp, out["tau_dp"].reshape(tdp.shape))


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_with_reference_delays_matches_reference(name):
    """FP64 amplitudes with the float32 delays: the whole early part agrees
    with the reference's FP32 and LUT outputs to float32 rounding, and with its
    half2 path to the error of its half-precision accumulation."""
    sc, out = SCENES[name]
    amp, _, _ = _amp_tau(sc)
    tau, _ = _tau_ref(sc)
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    got = oracle.ism_sum(amp, tau.astype(np.float64), n, sc["fs"])
    assert rel_l2(out["fp32/early"].reshape(got.shape), got) < 1e-6
    if "lut" in sc["modes"]:
        lut = oracle.ism_sum_lut(amp, tau.astype(np.float64), n, sc["fs"])
        assert rel_l2(out["lut/early"].reshape(lut.shape), lut) < 5e-7
    if "mp" in sc["modes"]:
        assert rel_l2(out["mp/early"].reshape(got.shape), got) < 2e-3


# ---------------------------------------------------------------------------------- GPU


def _engine(sc, mode="fp32", reference_delays=False):
    import gpurir_gb300 as G
    sim = G.Simulator(seed=1, mixed_precision=(mode == "mp"), lut=(mode == "lut"),
                      reference_delays=reference_delays)
    r = sim.simulate_rir(sc["room_sz"], sc["beta"], sc["pos_src"], sc["pos_rcv"], sc["orV_src"],
                         sc["orV_rcv"], sc["spkr_pattern"], sc["mic_pattern"], sc["nb_img"], sc["Tdiff"],
                         sc["Tmax"], sc["fs"])
    return sim, r


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SCENES))
def test_engine_reference_delays_match_reference_kernels(built, name):
    """Reference-delay mode against gpuRIR's own kernels: FP32 and LUT within
    1e-5 relative L2, mixed precision within 2e-3 (the reference accumulates
    in half precision), and each mode within float32 rounding of the oracle
    fed the same delays."""
    sc, out = SCENES[name]
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    amp, _, _ = _amp_tau(sc)
    tau, _ = _tau_ref(sc)
    for mode in sc["modes"]:
        _, r = _engine(sc, mode, reference_delays=True)
        ref = out["%s/early" % mode]
        e_ref = rel_l2(r[..., :n], ref)
        if mode == "lut":
            want = oracle.ism_sum_lut(amp, tau.astype(np.float64), n, sc["fs"]).reshape(ref.shape)
        else:
            want = oracle.ism_sum(amp, tau.astype(np.float64), n, sc["fs"]).reshape(ref.shape)
        e_orc = rel_l2(r[..., :n], want)
        print("%s %s: vs reference %.2e, vs oracle %.2e" % (name, mode, e_ref, e_orc))
        assert e_ref < (2e-3 if mode == "mp" else 1e-5)
        assert e_orc < (5e-4 if mode == "mp" else 1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SCENES))
def test_engine_matches_reference_kernels(built, name):
    """Default (exact-delay) mode against the reference: bounded by the
    reference's float32 delays, and closer to the exact sum than it."""
    sc, out = SCENES[name]
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    sim, r = _engine(sc)
    ref = out["fp32/early"]
    print("%s: default mode vs reference %.2e" % (name, rel_l2(r[..., :n], ref)))
    assert rel_l2(r[..., :n], ref) < 2e-4
    amp, tau, _ = _amp_tau(sc)
    exact = oracle.ism_sum(amp, tau, n, sc["fs"]).reshape(ref.shape)
    # closer to the exact sum than the reference is
    assert rel_l2(r[..., :n], exact) < 1e-6 < rel_l2(ref, exact)


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in sorted(SCENES) if "lut" in SCENES[n][0]["modes"]])
def test_engine_lut_matches_reference_kernels(built, name):
    sc, out = SCENES[name]
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    _, r = _engine(sc, "lut")
    amp, tau, _ = _amp_tau(sc)
    want = oracle.ism_sum_lut(amp, tau, n, sc["fs"]).reshape(r[..., :n].shape)
    assert rel_l2(r[..., :n], want) < 1e-5
    # vs the reference itself: its float32 delays move the fetch coordinates
    assert rel_l2(r[..., :n], out["lut/early"]) < 5e-4


@pytest.mark.gpu
def test_engine_mixed_precision_beats_reference(built):
    sc, out = SCENES["plain"]
    n = oracle.n_samples(sc["Tdiff"], sc["fs"])
    _, r = _engine(sc, "mp")
    amp, tau, _ = _amp_tau(sc)
    exact = oracle.ism_sum(amp, tau, n, sc["fs"]).reshape(r[..., :n].shape)
    assert rel_l2(r[..., :n], exact) < 0.25 * rel_l2(out["mp/early"], exact)


@pytest.mark.gpu
def test_engine_envelope_matches_reference_kernels(built):
    """envPred on the engine's own early part (the scene with a diffuse tail)."""
    sc, out = SCENES["tail"]
    sim, r = _engine(sc)
    env = sim.last_envelope(r.shape[0] * r.shape[1]).astype(np.float64)   # [M, 3]: A, alpha, tau_dp
    rA, ral, rtd = (out[k].ravel().astype(np.float64) for k in ("A", "alpha", "tau_dp"))
    assert np.all(np.abs(env[:, 0] - rA) <= 1e-3 * np.abs(rA) + 1e-30)
    assert np.all(np.abs(env[:, 1] - ral) <= 1e-6 * np.abs(ral))
    assert np.all(np.abs(env[:, 2] - rtd) <= 1e-6 * rtd)


@pytest.mark.gpu
def test_engine_envelope_reference_delays(built):
    """With reference delays the direct-path delay is the reference's bit for
    bit, and A follows its early part to float32 rounding."""
    sc, out = SCENES["tail"]
    sim, r = _engine(sc, reference_delays=True)
    env = sim.last_envelope(r.shape[0] * r.shape[1])
    assert np.array_equal(env[:, 2], out["tau_dp"].ravel())
    rA = out["A"].ravel().astype(np.float64)
    assert np.all(np.abs(env[:, 0] - rA) <= 1e-5 * np.abs(rA) + 1e-30)
    ral = out["alpha"].ravel().astype(np.float64)
    assert np.all(np.abs(env[:, 1] - ral) <= 1e-6 * np.abs(ral))


def _random_scene(rng):
    fs = float(rng.choice([8000.0, 16000.0, 22050.0, 44100.0, 48000.0]))
    room = rng.uniform([3, 3, 2.5], [9, 7, 4]).astype(np.float32)
    ms, mr = int(rng.integers(1, 4)), int(rng.integers(1, 5))
    sp, mp = int(rng.integers(0, 6)), int(rng.integers(0, 6))
    ps = (0.4 + rng.random((ms, 3)) * (room - 0.8)).astype(np.float32)
    pr = (0.4 + rng.random((mr, 3)) * (room - 0.8)).astype(np.float32)
    unit = lambda n: (lambda v: (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32))(
        rng.standard_normal((n, 3)))
    T = float(rng.uniform(0.03, 0.12))
    return dict(room_sz=room, beta=rng.uniform(0.5, 0.97, 6).astype(np.float32), pos_src=ps, pos_rcv=pr,
                orV_src=unit(ms), orV_rcv=unit(mr), spkr_pattern=sp, mic_pattern=mp,
                nb_img=[int(x) for x in rng.integers(3, 10, 3)], Tdiff=T, Tmax=T, fs=fs)


@pytest.mark.gpu
@pytest.mark.skipif(not ref_kernels.available(), reason="reference kernels not built (oracle/_ref)")
def test_live_reference_kernels_random_scenes(built):
    """The reference's kernels run now on random scenes (sampling rates 8-48
    kHz, every polar pattern): the oracle fed their amplitudes and delays
    reproduces their FP32 and LUT outputs, and the engine agrees with them up
    to their float32 delays."""
    rk = ref_kernels.RefKernels()
    rng = np.random.default_rng(2024)
    for _ in range(12):
        sc = _random_scene(rng)
        kw = {k: sc[k] for k in ("room_sz", "beta", "pos_src", "pos_rcv", "orV_src", "orV_rcv",
                                 "spkr_pattern", "mic_pattern", "nb_img", "Tmax", "Tdiff", "fs")}
        ref = rk.simulate(mode="fp32", **kw)
        lut = rk.simulate(mode="lut", **kw)
        n = ref["n_ism"]
        fed = oracle.ism_sum(ref["amp"], ref["tau"], n, sc["fs"]).reshape(ref["early"].shape)
        assert rel_l2(ref["early"], fed) < 1e-6
        fed_lut = oracle.ism_sum_lut(ref["amp"], ref["tau"], n, sc["fs"]).reshape(ref["early"].shape)
        assert rel_l2(lut["early"], fed_lut) < 5e-7
        _, r = _engine(sc)
        assert rel_l2(r[..., :n], ref["early"]) < 3e-4
        # the float32 delay model is the reference's, bit for bit, on every pattern pair
        inv = {v: k for k, v in oracle.PATTERNS.items()}
        tau, tdp = oracle.tau_reference_f32(sc["room_sz"], sc["pos_src"], sc["pos_rcv"], sc["nb_img"],
                                            sc["fs"], inv[sc["spkr_pattern"]], inv[sc["mic_pattern"]])
        assert np.array_equal(tau, ref["tau"].reshape(tau.shape))
        assert np.array_equal(tdp, ref["tau_dp"].reshape(tdp.shape))
        _, rr = _engine(sc, reference_delays=True)
        assert rel_l2(rr[..., :n], ref["early"]) < 1e-5
        _, rl = _engine(sc, "lut", reference_delays=True)
        assert rel_l2(rl[..., :n], lut["early"]) < 1e-5
        mp = rk.simulate(mode="mp", **kw)
        _, rm = _engine(sc, "mp", reference_delays=True)
        assert rel_l2(rm[..., :n], mp["early"]) < 2e-3
    rk.close()


@pytest.mark.gpu
@pytest.mark.skipif(not ref_kernels.available(), reason="reference kernels not built (oracle/_ref)")
def test_tail_energy_decay_matches_reference_kernels(built):
    """The engine's diffuse tail (Philox, logistic transform) against the reference's
    own tail: its envPred_kernel and diffRev_kernel run live (src/gpuRIR_cuda.cu:
    415-461) on uniforms standing in for its cuRAND stream (a closed library).  The
    noise differs, the statistics must not: the energy-decay curve (Schroeder
    integral) averaged over the 16 RIRs agrees within 0.5 dB down to -60 dB, up to
    2 / |alpha| samples before the end (where a few samples decide the integral)."""
    import torch
    import gpurir_gb300 as G
    rng = np.random.default_rng(5)
    room = [6.0, 5.0, 3.0]
    beta = G.beta_SabineEstimation(room, 1.0)
    ps = (0.5 + rng.random((4, 3)) * (np.array(room) - 1)).astype(np.float32)
    pr = (0.5 + rng.random((4, 3)) * (np.array(room) - 1)).astype(np.float32)
    nb, fs, Tdiff, Tmax = G.t2n(0.1, room), 16000.0, 0.1, 1.0
    rk = ref_kernels.RefKernels()
    n_ism, n = oracle.n_samples(Tdiff, fs), oracle.n_samples(Tmax, fs)
    g = torch.Generator(device="cuda").manual_seed(3)
    u = torch.rand((16 * (n - n_ism),), device="cuda", generator=g).clamp_(1e-7, 1 - 1e-7)
    ref = rk.simulate(room, beta, ps, pr, nb, Tmax, fs, Tdiff=Tdiff, mode="fp32", uniforms=u)
    rk.close()
    ref_rir = np.concatenate([ref["early"], ref["diffuse"]], axis=-1).reshape(16, n).astype(np.float64)
    sim = G.Simulator(seed=8, reference_delays=True)
    got = sim.simulate_rir(room, beta, ps, pr, None, None, 0, 0, nb, Tdiff, Tmax, fs).reshape(16, n)
    edc = lambda x: np.mean([np.cumsum((r.astype(np.float64) ** 2)[::-1])[::-1] for r in x], axis=0)
    ea, eb = edc(got), edc(ref_rir)
    alpha = abs(float(ref["alpha"].ravel()[0]))
    keep = (eb > eb[0] * 1e-6) & (np.arange(n) < n - int(2 / alpha))
    d = 10 * np.log10(ea[keep] / eb[keep])
    print("EDC max difference %.3f dB over %d samples" % (np.abs(d).max(), keep.sum()))
    assert np.abs(d).max() < 0.5
