"""Tuned launch shapes on the GPU: every candidate of every knob gives the default
launch's result bit for bit (the knobs lay work out differently, they do not
change the arithmetic), and the autotuner measures, picks and caches."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def knobs(built):
    from gpurir_gb300 import tune
    tune.reset()
    yield tune
    tune.reset()


def test_conv_rows_identical_bits(knobs):
    import torch
    from gpurir_gb300.trajectory import gpu_conv
    rng = np.random.default_rng(0)
    seg = rng.standard_normal((5, 300)).astype(np.float32)
    rir = rng.standard_normal((5, 3, 3000)).astype(np.float32)
    outs = []
    for v in (1, 2):
        knobs.set_knobs({"conv_rows": v})
        outs.append(gpu_conv(seg, rir))
    assert np.array_equal(outs[0], outs[1])


def test_ism_and_adjoint_blocks_identical_bits(knobs):
    import torch
    import gpurir_gb300 as G
    from gpurir_gb300.autograd import TorchBatch
    from gpurir_gb300 import workloads
    rooms = workloads.inverse_problem()[:3]
    dev = torch.device("cuda")
    t = lambda a, g=True: torch.tensor(a, device=dev, requires_grad=g)
    res = []
    for ism, adj in ((0, 0), (1, 1), (0, 2)):
        knobs.set_knobs({"ism_blocks_per_sm": ism, "adjoint_blocks_per_sm": adj})
        sim = G.Simulator(seed=3)
        sc = workloads.plain_room()
        r1 = sim.simulate_rir(sc["room_sz"], sc["beta"], sc["pos_src"], sc["pos_rcv"], None, None, 0, 0,
                              sc["nb_img"], sc["Tdiff"], sc["Tmax"], sc["fs"]).copy()
        model = TorchBatch(rooms, 16000.0, sim=sim)
        beta = t(np.stack([r["beta"] for r in rooms]))
        ps = t(np.concatenate([r["pos_src"] for r in rooms]))
        pr = t(np.concatenate([r["pos_rcv"] for r in rooms]))
        orv = t(np.concatenate([r["orV_rcv"] for r in rooms]), False)
        target = model(beta.detach() * 0.98, ps.detach(), pr.detach(), None, orv).detach()
        model.l2_step(beta, ps, pr, None, orv, target)
        torch.cuda.synchronize()
        res.append((r1, model.last_rirs.clone(), beta.grad.clone(), ps.grad.clone(), pr.grad.clone()))
    for other in res[1:]:
        assert np.array_equal(res[0][0], other[0])
        for a, b in zip(res[0][1:], other[1:]):
            assert torch.equal(a, b)


def test_traj_adjoint_blocks_identical_bits(knobs):
    import torch
    from gpurir_gb300.trajectory import simulate_trajectory_torch
    rng = np.random.default_rng(1)
    dev = torch.device("cuda")
    grads = []
    for v in (1, 2):
        knobs.set_knobs({"traj_adjoint_blocks_per_sm": v})
        sig = torch.tensor(rng.standard_normal(3000).astype(np.float32) if not grads else sig0,
                           device=dev, requires_grad=True)
        rir = torch.tensor(rng.standard_normal((10, 2, 1500)).astype(np.float32) if not grads else rir0,
                           device=dev, requires_grad=True)
        sig0, rir0 = sig.detach().cpu().numpy(), rir.detach().cpu().numpy()
        simulate_trajectory_torch(sig, rir).sum().backward()
        grads.append((sig.grad.clone(), rir.grad.clone()))
    assert torch.equal(grads[0][0], grads[1][0]) and torch.equal(grads[0][1], grads[1][1])


def test_autotuner_measures_and_caches(knobs, tmp_path):
    path = str(tmp_path / "tuning.json")
    entry = knobs.tune(reps=2, warmup=1, path=path)
    for k, cands in knobs.KNOBS.items():
        assert entry["knobs"][k] in cands
        assert set(entry["timings_ms"][k]) == {str(v) for v in cands}
    assert knobs.get_knobs() == entry["knobs"]
    knobs.reset()
    assert knobs.apply_cached(path=path) == entry["knobs"]
