"""GPU parity of the fused ISM forward kernel against the FP64 oracle.

Tolerance (FP32 mode): relative L2 error <= 1e-5 of the early part against
the FP64 restatement of src/gpuRIR_cuda.cu, and max-abs error <= 1e-5 of the
RIR's peak.  All calls go through the C ABI (gpurir_simulate_rir).
"""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL_REL_L2 = 1e-5
TOL_MAXABS = 1e-5


def _sim():
    import gpurir_gb300 as G
    return G.Simulator(mixed_precision=False, lut=False, seed=1234)


def _rand_inside(rng, n, room, margin):
    room = np.asarray(room, dtype=np.float64)
    return (margin + rng.random((n, 3)) * (room - 2 * margin)).astype(np.float32)


def _unit(rng, n):
    v = rng.standard_normal((n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def _run(sim, room, beta, ps, pr, nb, Tmax, fs, Tdiff=None, spkr="omni", mic="omni",
         os_=None, or_=None, c=343.0):
    import gpurir_gb300 as G
    Tdiff = Tmax if Tdiff is None else Tdiff
    out = sim.simulate_rir(room, beta, ps, pr, os_, or_, G.polar_patterns[spkr],
                           G.polar_patterns[mic], nb, Tdiff, Tmax, fs, c)
    ref, parts = oracle.simulate_rir(room, beta, ps, pr, nb, Tmax, fs, Tdiff, spkr, mic, os_, or_,
                                     c, return_parts=True)
    return out, ref, parts


def _check_ism(out, ref, n_ism, label=""):
    a = out[..., :n_ism].reshape(-1, n_ism)
    b = ref[..., :n_ism].reshape(-1, n_ism)
    e = rel_l2(a, b)
    mx = np.abs(a - b).max() / np.abs(b).max()
    assert e <= TOL_REL_L2, "%s rel-L2 %.3g" % (label, e)
    assert mx <= TOL_MAXABS, "%s max-abs/peak %.3g" % (label, mx)
    return e, mx


def test_plain_single_room(built):
    """1 source x 2 receivers, full ISM, nb_img [11, 9, 13], 0.5 s at 16 kHz (omni)."""
    rng = np.random.default_rng(0)
    room = [3.0, 4.0, 2.5]
    ps = _rand_inside(rng, 1, room, 0.5)
    pr = _rand_inside(rng, 2, room, 0.5)
    out, ref, p = _run(_sim(), room, [0.85] * 6, ps, pr, [11, 9, 13], 0.5, 16000.0)
    assert out.shape == (1, 2, 8000) and out.dtype == np.float32
    _check_ism(out, ref, p["n_ism"], "plain")


@pytest.mark.parametrize("spkr", list(range(6)))
@pytest.mark.parametrize("mic", list(range(6)))
def test_polar_patterns(built, spkr, mic):
    names = ["omni", "homni", "card", "hypcard", "subcard", "bidir"]
    rng = np.random.default_rng(100 + 6 * spkr + mic)
    room = [5.0, 4.0, 3.0]
    ps = _rand_inside(rng, 2, room, 0.4)
    pr = _rand_inside(rng, 3, room, 0.4)
    out, ref, p = _run(_sim(), room, [0.9, 0.8, 0.7, 0.75, 0.6, 0.95], ps, pr, [5, 6, 7], 0.12,
                       16000.0, spkr=names[spkr], mic=names[mic], os_=_unit(rng, 2),
                       or_=_unit(rng, 3))
    _check_ism(out, ref, p["n_ism"], "patterns %d %d" % (spkr, mic))


@pytest.mark.parametrize("fs", [8000.0, 16000.0, 22050.0, 44100.0, 48000.0])
def test_sample_rates(built, fs):
    rng = np.random.default_rng(7)
    room = [4.0, 3.5, 2.8]
    ps = _rand_inside(rng, 2, room, 0.3)
    pr = _rand_inside(rng, 2, room, 0.3)
    out, ref, p = _run(_sim(), room, [0.8] * 6, ps, pr, [7, 7, 7], 0.1, fs)
    _check_ism(out, ref, p["n_ism"], "fs %g" % fs)


def test_many_rirs_single_segment(built):
    """Enough RIRs that each one is a single work item."""
    rng = np.random.default_rng(1)
    room = [6.0, 5.0, 3.0]
    ps = _rand_inside(rng, 24, room, 0.5)
    pr = _rand_inside(rng, 32, room, 0.5)
    out, ref, p = _run(_sim(), room, [0.9407] * 6, ps, pr, [6, 7, 12], 0.15, 16000.0)
    _check_ism(out, ref, p["n_ism"], "many")


def test_long_rir_many_segments(built):
    """A few long RIRs are split into many segments; images land on segment edges."""
    rng = np.random.default_rng(3)
    room = [3.0, 4.0, 2.5]
    ps = _rand_inside(rng, 1, room, 0.5)
    pr = _rand_inside(rng, 1, room, 0.5)
    out, ref, p = _run(_sim(), room, [0.9] * 6, ps, pr, [25, 19, 31], 1.1, 16000.0)
    _check_ism(out, ref, p["n_ism"], "long")


def test_image_exactly_on_sample(built):
    """Direct path of exactly 50 samples (c = 320 m/s, fs = 16 kHz, 1 m apart)."""
    room = [4.0, 4.0, 3.0]
    ps = np.array([[1.0, 2.0, 1.5]], dtype=np.float32)
    pr = np.array([[2.0, 2.0, 1.5]], dtype=np.float32)
    out, ref, p = _run(_sim(), room, [0.7] * 6, ps, pr, [3, 3, 3], 0.05, 16000.0, c=320.0)
    assert abs(p["tau_dp"][0, 0] - 50.0) < 1e-12
    _check_ism(out, ref, p["n_ism"], "on-sample")
    # the direct path contributes exactly its amplitude at t = 50 and ~0 at other integers
    assert abs(out[0, 0, 50] - ref[0, 0, 50]) < 1e-6


def test_zero_and_negative_walls(built):
    """beta = 0 (anechoic walls) and mixed signs of odd reflection orders."""
    rng = np.random.default_rng(5)
    room = [3.5, 3.0, 2.7]
    ps = _rand_inside(rng, 1, room, 0.4)
    pr = _rand_inside(rng, 2, room, 0.4)
    out, ref, p = _run(_sim(), room, [0.0, 0.9, 0.5, 0.0, 1.0, 0.3], ps, pr, [9, 9, 9], 0.2,
                       16000.0)
    _check_ism(out, ref, p["n_ism"], "walls")


def test_even_nb_img_and_single_image(built):
    rng = np.random.default_rng(6)
    room = [3.0, 3.0, 3.0]
    ps = _rand_inside(rng, 1, room, 0.5)
    pr = _rand_inside(rng, 1, room, 0.5)
    for nb in ([1, 1, 1], [2, 4, 6], [1, 8, 3]):
        out, ref, p = _run(_sim(), room, [0.8] * 6, ps, pr, nb, 0.08, 16000.0)
        _check_ism(out, ref, p["n_ism"], "nb %s" % nb)


def test_repeat_calls_bitwise_identical(built):
    """Deterministic summation order: two calls give identical bits."""
    rng = np.random.default_rng(8)
    room = [6.0, 5.0, 3.0]
    ps = _rand_inside(rng, 4, room, 0.5)
    pr = _rand_inside(rng, 4, room, 0.5)
    sim = _sim()
    import gpurir_gb300 as G
    a = sim.simulate_rir(room, [0.9] * 6, ps, pr, None, None, 0, 0, [10, 10, 10], 0.3, 0.3, 16000.0)
    b = sim.simulate_rir(room, [0.9] * 6, ps, pr, None, None, 0, 0, [10, 10, 10], 0.3, 0.3, 16000.0)
    assert np.array_equal(a, b)


def test_dropin_simulateRIR(built):
    """The gpuRIR-named entry point: shape, dtype, Tdiff default and asserts."""
    import gpurir_gb300 as G
    rng = np.random.default_rng(9)
    room = [3.0, 4.0, 2.5]
    ps = _rand_inside(rng, 2, room, 0.5).astype(np.float64)
    pr = _rand_inside(rng, 3, room, 0.5)
    r = G.simulateRIR(room, [0.85] * 6, ps, pr, [5, 5, 5], 0.1, 16000)
    assert r.shape == (2, 3, 1600) and r.dtype == np.float32
    ref = oracle.simulate_rir(room, [0.85] * 6, ps, pr, [5, 5, 5], 0.1, 16000)
    assert rel_l2(r, ref) <= TOL_REL_L2
    with pytest.raises(AssertionError):
        G.simulateRIR(room, [0.85] * 6, ps + 10, pr, [5, 5, 5], 0.1, 16000)
    with pytest.raises(AssertionError):
        G.simulateRIR(room, [0.85] * 6, ps, pr, [5, 5, 5], 0.1, 16000, Tdiff=0.2)
    with pytest.raises(AssertionError):
        G.simulateRIR(room, [0.85] * 6, ps, pr, [5, 5, 5], 0.1, 16000, mic_pattern="card")


def test_device_entry_matches_host_entry(built):
    """gpurir_simulate_rir_device on torch-owned memory equals the host entry."""
    import ctypes
    import torch
    import gpurir_gb300 as G
    from gpurir_gb300 import _lib
    rng = np.random.default_rng(10)
    room = np.array([6.0, 5.0, 3.0], dtype=np.float32)
    beta = np.full(6, 0.9, dtype=np.float32)
    ps = _rand_inside(rng, 3, room, 0.5)
    pr = _rand_inside(rng, 5, room, 0.5)
    nb = np.array([6, 6, 6], dtype=np.int32)
    sim = _sim()
    host = sim.simulate_rir(room, beta, ps, pr, None, None, 0, 0, nb, 0.1, 0.25, 16000.0)
    dps = torch.from_numpy(ps).cuda()
    dpr = torch.from_numpy(pr).cuda()
    out = torch.empty(host.shape, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    sim.set_seed(1234, 0)
    L = _lib.load()
    _lib.check(L.gpurir_simulate_rir_device(
        sim.handle, room.ctypes.data_as(_lib.fptr), beta.ctypes.data_as(_lib.fptr), dps.data_ptr(), 3,
        dpr.data_ptr(), None, None, 0, 0, 5, nb.ctypes.data_as(_lib.iptr), 0.1, 0.25, 16000.0,
        343.0, out.data_ptr(), ctypes.c_void_p(st)), "device")
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), host)


def test_invalid_arguments_raise(built):
    import gpurir_gb300 as G
    sim = _sim()
    ps = np.array([[1, 1, 1]], dtype=np.float32)
    with pytest.raises(G.GpuRirError):
        sim.simulate_rir([3, 3, 3], [0.5] * 6, ps, ps, None, None, 0, 0, [0, 3, 3], 0.1, 0.1, 16000.0)
    with pytest.raises(G.GpuRirError):
        sim.simulate_rir([3, 3, 3], [0.5] * 6, ps, ps, None, None, 0, 2, [3, 3, 3], 0.1, 0.1, 16000.0)
    with pytest.raises(G.GpuRirError):
        sim.simulate_rir([3, 3, 3], [0.5] * 6, ps, ps, None, None, 0, 0, [3, 3, 3], 0.2, 0.1, 16000.0)


@pytest.mark.parametrize("fs", [96000.0, 11025.0])
def test_high_and_odd_sample_rates(built, fs):
    """96 kHz: a 768-tap window (24 taps per lane, the large shared-memory layout);
    11.025 kHz: an odd 88-tap window (half-integer half width, clamped taps)."""
    rng = np.random.default_rng(11)
    room = [3.5, 3.0, 2.6]
    ps = _rand_inside(rng, 1, room, 0.4)
    pr = _rand_inside(rng, 2, room, 0.4)
    out, ref, p = _run(_sim(), room, [0.75] * 6, ps, pr, [5, 5, 5], 0.03, fs)
    _check_ism(out, ref, p["n_ism"], "fs %g" % fs)


def test_window_beyond_supported_rate_is_an_error(built):
    """Above ~190 kHz the window exceeds 24 taps per lane: refused, not truncated."""
    import gpurir_gb300 as G
    ps = np.array([[1, 1, 1]], dtype=np.float32)
    pr = np.array([[2, 2, 1]], dtype=np.float32)
    with pytest.raises(G.GpuRirError):
        _sim().simulate_rir([3, 3, 3], [0.5] * 6, ps, pr, None, None, 0, 0, [3, 3, 3], 0.01, 0.01, 192000.0)


def test_zero_lengths(built):
    """Tmax = 0: an empty time axis; Tdiff = 0: no early part, and an empty envelope
    window gives a silent tail (gpuRIR divides by <= 0 there)."""
    sim = _sim()
    ps = np.array([[1, 1, 1]], dtype=np.float32)
    pr = np.array([[2, 2, 1.5], [2.5, 1.0, 1.0]], dtype=np.float32)
    a = sim.simulate_rir([3, 3, 3], [0.8] * 6, ps, pr, None, None, 0, 0, [3, 3, 3], 0.0, 0.0, 16000.0)
    assert a.shape == (1, 2, 0)
    b = sim.simulate_rir([3, 3, 3], [0.8] * 6, ps, pr, None, None, 0, 0, [3, 3, 3], 0.0, 0.05, 16000.0)
    assert b.shape == (1, 2, 800) and np.all(b == 0.0)


def test_too_many_images_is_an_error(built):
    import gpurir_gb300 as G
    ps = np.array([[1, 1, 1]], dtype=np.float32)
    with pytest.raises(G.GpuRirError):
        _sim().simulate_rir([3, 3, 3], [0.5] * 6, ps, ps + 0.5, None, None, 0, 0, [300, 300, 300],
                            0.01, 0.01, 16000.0)


def test_rirs_split_by_images_with_tail(built):
    """Few RIRs with many images: each RIR's images are split into parts whose partial
    early parts a reduction adds up; the tail kernel then reads the finished early part."""
    rng = np.random.default_rng(17)
    room = [5.0, 4.0, 3.0]
    ps = _rand_inside(rng, 1, room, 0.5)
    pr = _rand_inside(rng, 2, room, 0.5)
    out, ref, p = _run(_sim(), room, [0.85] * 6, ps, pr, [21, 21, 21], 0.3, 16000.0, Tdiff=0.08)
    _check_ism(out, ref, p["n_ism"], "split")
    n = p["n_ism"]
    assert np.all(p["A"] > 0)
    assert rel_l2(out[..., n:], ref[..., n:]) <= 1e-4


def test_segments_past_the_last_image(built):
    """A short image set in a long RIR: the planner cuts it into many segments, most of
    them past every image's window; the device flags those from the actual positions.
    One source lies outside the room (its images reach further than the in-room bound
    the planner uses), so a wrong skip would drop its late images."""
    rng = np.random.default_rng(11)
    room = [3.0, 4.0, 2.5]
    ps = np.concatenate([_rand_inside(rng, 1, room, 0.5), np.array([[9.5, 2.0, 1.0]], np.float32)])
    pr = _rand_inside(rng, 2, room, 0.5)
    out, ref, parts = _run(_sim(), room, [0.8] * 6, ps, pr, [5, 5, 5], 0.3, 16000.0)
    n = parts["n_ism"]
    _check_ism(out, ref, n, "segments past the images")
    # the far source's windows reach past sample 900 (the in-room delay bound of this room
    # is ~850 samples): that energy must be there, and everything after it is zero
    late = slice(850, 1000)
    assert np.abs(ref[1, :, late]).max() > 1e-4 * np.abs(ref).max()
    assert np.abs(out[1, :, late] - ref[1, :, late]).max() <= 1e-5 * np.abs(ref).max()
    assert not np.any(out[:, :, 1000:n])


def _one_shot_adjoint(sim, rooms, g, fs=16000.0):
    """gpurir_ism_backward_batch_device on torch tensors: gradients of sum(h * g)."""
    import ctypes
    import torch
    from gpurir_gb300 import _lib
    from gpurir_gb300.batch import _room_struct
    dev = torch.device("cuda")
    ps = torch.tensor(np.concatenate([r["pos_src"] for r in rooms]), device=dev)
    pr = torch.tensor(np.concatenate([r["pos_rcv"] for r in rooms]), device=dev)
    gr = torch.tensor(g, dtype=torch.float32, device=dev)
    gb = torch.empty((len(rooms), 6), device=dev)
    gs, gq = torch.empty_like(ps), torch.empty_like(pr)
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.load().gpurir_ism_backward_batch_device(
        sim.handle, len(rooms), _room_struct(rooms), fs, 343.0, ps.data_ptr(), pr.data_ptr(), None, None,
        gr.data_ptr(), gb.data_ptr(), gs.data_ptr(), gq.data_ptr(), None, None, ctypes.c_void_p(st)),
        "gpurir_ism_backward_batch_device")
    torch.cuda.synchronize()
    return gb.cpu().numpy(), gs.cpu().numpy(), gq.cpu().numpy()


def test_plan_reuse_across_calls_and_other_uploads(built):
    """Calls with the same room shapes reuse the plan and the work items already on the
    device; new positions and walls must still take effect, and an upload by another
    entry (the one-shot adjoint) in between must not leave stale items behind."""
    rng = np.random.default_rng(21)
    room, nb, T = [5.0, 4.0, 3.0], [7, 8, 9], 0.12
    sim = _sim()

    def check(ps, pr, beta, nb_=nb, label=""):
        out, ref, parts = _run(sim, room, beta, ps, pr, nb_, T, 16000.0)
        _check_ism(out, ref, parts["n_ism"], label)
        return out

    shapes = lambda: (_rand_inside(rng, 3, room, 0.5), _rand_inside(rng, 5, room, 0.5),
                      rng.uniform(0.5, 0.95, 6).astype(np.float32))
    a = check(*shapes(), label="first call")
    b = check(*shapes(), label="same shapes, new positions and walls")
    assert not np.array_equal(a, b)
    ps, pr, beta = shapes()
    n = oracle.n_samples(T, 16000.0)
    _one_shot_adjoint(sim, [dict(room_sz=np.float32(room), beta=beta, pos_src=ps, pos_rcv=pr, nb_img=[5, 5, 5],
                                 Tmax=0.05, Tdiff=0.05)],
                      rng.standard_normal(3 * 5 * oracle.n_samples(0.05, 16000.0)))
    check(*shapes(), label="after another entry's upload")
    check(*shapes(), nb_=[6, 6, 6], label="new shapes")
    check(*shapes(), label="back to the first shapes")
    assert n > 0


def test_one_shot_adjoint_matches_torch_batch(built):
    """gpurir_ism_backward_batch_device gives the gradients of the prepared-batch path."""
    import torch
    from gpurir_gb300.autograd import TorchBatch
    rng = np.random.default_rng(23)
    rooms = []
    for i in range(3):
        room = rng.uniform([3, 3, 2.5], [6, 5, 3.5]).astype(np.float32)
        rooms.append(dict(room_sz=room, beta=rng.uniform(0.6, 0.9, 6).astype(np.float32),
                          pos_src=_rand_inside(rng, 2, room, 0.5), pos_rcv=_rand_inside(rng, 3, room, 0.5),
                          nb_img=[5, 6, 7], Tmax=0.05 + 0.01 * i, Tdiff=0.05 + 0.01 * i))
    sim = _sim()
    model = TorchBatch(rooms, 16000.0, sim=sim)
    g = rng.standard_normal(model.total)
    t = lambda a: torch.tensor(a, device="cuda", requires_grad=True)
    beta = t(np.stack([r["beta"] for r in rooms]))
    ps, pr = t(np.concatenate([r["pos_src"] for r in rooms])), t(np.concatenate([r["pos_rcv"] for r in rooms]))
    (model(beta, ps, pr) * torch.tensor(g, dtype=torch.float32, device="cuda")).sum().backward()
    gb, gs, gq = _one_shot_adjoint(sim, rooms, g)
    for ours, ref in ((gb, beta.grad), (gs, ps.grad), (gq, pr.grad)):
        ref = ref.cpu().numpy()
        assert rel_l2(ours, ref) < 1e-6, rel_l2(ours, ref)


def test_plan_reuse_across_mode_switches(built):
    """Same shapes, the evaluation mode switched between calls on one simulator: each call
    matches a fresh simulator in that mode (the reused plan is keyed by the mode)."""
    import gpurir_gb300 as G
    rng = np.random.default_rng(29)
    room, nb, T = [4.0, 5.0, 3.0], [6, 6, 6], 0.1
    ps, pr = _rand_inside(rng, 2, room, 0.5), _rand_inside(rng, 3, room, 0.5)
    args = (room, [0.8] * 6, ps, pr, None, None, 0, 0, nb, T, T, 16000.0)
    sim = _sim()
    fresh = {m: G.Simulator(mixed_precision=(m == "mp"), lut=(m == "lut"), seed=1234) for m in ("fp32", "mp", "lut")}
    for mode in ("fp32", "lut", "fp32", "mp", "lut"):
        sim.activate_lut(mode == "lut")
        sim.activate_mixed_precision(mode == "mp")
        got = sim.simulate_rir(*args)
        want = fresh[mode].simulate_rir(*args)
        assert np.array_equal(got, want), mode
