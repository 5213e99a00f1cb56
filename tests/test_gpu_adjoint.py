"""GPU checks of the adjoint kernel behind torch.autograd: gradients with respect
to beta, source/receiver positions and orientations against FP64 torch autograd
of the same formulas (tests/torch_ism_ref.py) and against FP64 central
differences of the C oracle (step 1e-5).

Tolerance: relative L2 error of each gradient <= 2e-4 against FP64 autograd
(FP32 forward quantities, FP32 accumulation over ~1e5 taps)."""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 2e-4


def _setup(seed, spkr="card", mic="hypcard", ns=2, nr=3, nb=(5, 6, 7), T=0.06, room=(4.0, 3.5, 2.8), fs=16000.0):
    rng = np.random.default_rng(seed)
    room = np.array(room)
    ps = (0.5 + rng.random((ns, 3)) * (room - 1.0)).astype(np.float32)
    pr = (0.5 + rng.random((nr, 3)) * (room - 1.0)).astype(np.float32)
    os_ = rng.standard_normal((ns, 3)).astype(np.float32)
    or_ = rng.standard_normal((nr, 3)).astype(np.float32)
    beta = rng.uniform(0.6, 0.95, 6).astype(np.float32)
    n = oracle.n_samples(T, fs)
    g = rng.standard_normal((ns, nr, n))
    return dict(room=room.astype(np.float32), ps=ps, pr=pr, os=os_, orv=or_, beta=beta, nb=list(nb),
                T=T, n=n, g=g, spkr=spkr, mic=mic, fs=fs)


def _ours(c):
    import torch
    from gpurir_gb300.autograd import simulate_rir_torch
    t = lambda a: torch.tensor(a, device="cuda", requires_grad=True)
    beta, ps, pr = t(c["beta"]), t(c["ps"]), t(c["pr"])
    os_ = t(c["os"]) if c["spkr"] != "omni" else None
    or_ = t(c["orv"]) if c["mic"] != "omni" else None
    h = simulate_rir_torch(c["room"], beta, ps, pr, c["nb"], c["T"], c["fs"], spkr_pattern=c["spkr"],
                           mic_pattern=c["mic"], orV_src=os_, orV_rcv=or_)
    loss = (h.double() * torch.tensor(c["g"], device="cuda")).sum()
    loss.backward()
    grads = dict(beta=beta.grad, ps=ps.grad, pr=pr.grad)
    if os_ is not None:
        grads["os"] = os_.grad
    if or_ is not None:
        grads["orv"] = or_.grad
    return {k: v.detach().cpu().numpy().astype(np.float64) for k, v in grads.items()}, h


def _ref(c):
    import torch
    from torch_ism_ref import early_part
    t = lambda a: torch.tensor(np.asarray(a, dtype=np.float64), requires_grad=True)
    beta, ps, pr, os_, or_ = t(c["beta"]), t(c["ps"]), t(c["pr"]), t(c["os"]), t(c["orv"])
    h = early_part(c["room"], beta, ps, pr, c["nb"], c["n"], c["fs"], spkr=c["spkr"], mic=c["mic"],
                   orV_src=os_, orV_rcv=or_)
    loss = (h * torch.tensor(c["g"])).sum()
    loss.backward()
    out = dict(beta=beta.grad, ps=ps.grad, pr=pr.grad, os=os_.grad, orv=or_.grad)
    return {k: v.numpy() for k, v in out.items() if v is not None}, h.detach().numpy()


@pytest.mark.parametrize("spkr,mic", [("omni", "omni"), ("card", "hypcard"), ("subcard", "bidir"),
                                      ("hypcard", "card")])
def test_gradients_match_fp64_autograd(built, spkr, mic):
    c = _setup(31, spkr, mic)
    ours, h = _ours(c)
    ref, href = _ref(c)
    assert rel_l2(h.detach().cpu().numpy(), href) < 1e-5
    for k in ours:
        e = rel_l2(ours[k], ref[k])
        assert e < TOL, (k, e)


def test_beta_gradient_matches_central_differences(built):
    """dL/dbeta against FP64 central differences of the C oracle (step 1e-5)."""
    c = _setup(32, "omni", "card", ns=1, nr=2, nb=(4, 5, 6), T=0.05)
    ours, _ = _ours(c)

    def L(beta):
        h = oracle.simulate_rir(c["room"], beta, c["ps"], c["pr"], c["nb"], c["T"], 16000.0,
                                mic_pattern=c["mic"], orV_rcv=c["orv"])
        return float((h * c["g"]).sum())

    fd = np.zeros(6)
    for w in range(6):
        e = np.zeros(6)
        e[w] = 1e-5
        # the oracle reads beta as float32: difference quotient over the float32 step actually taken
        bp = (c["beta"].astype(np.float64) + e).astype(np.float32)
        bm = (c["beta"].astype(np.float64) - e).astype(np.float32)
        fd[w] = (L(bp) - L(bm)) / (float(bp[w]) - float(bm[w]))
    assert rel_l2(ours["beta"], fd) < 1e-3


def test_position_gradient_matches_central_differences(built):
    c = _setup(33, "omni", "omni", ns=1, nr=1, nb=(3, 3, 3), T=0.04)
    ours, _ = _ours(c)
    fd = np.zeros(3)
    for d in range(3):
        hs = []
        for sgn in (1, -1):
            ps = c["ps"].astype(np.float64)
            ps[0, d] += sgn * 1e-4
            ps32 = ps.astype(np.float32)
            h = oracle.simulate_rir(c["room"], c["beta"], ps32, c["pr"], c["nb"], c["T"], 16000.0)
            hs.append(((h * c["g"]).sum(), float(ps32[0, d])))
        fd[d] = (hs[0][0] - hs[1][0]) / (hs[0][1] - hs[1][1])
    assert rel_l2(ours["ps"][0], fd) < 2e-3


def test_batched_gradients(built):
    """Several rooms in one launch: per-room beta, per-source and per-receiver gradients."""
    import torch
    from torch_ism_ref import early_part
    from gpurir_gb300.autograd import simulate_batch_torch
    from gpurir_gb300 import batch as B
    rng = np.random.default_rng(34)
    rooms, betas, ps_all, pr_all, or_all = [], [], [], [], []
    for i in range(3):
        cc = _setup(40 + i, "omni", "hypcard", ns=1 + i % 2, nr=2 + i, nb=(4, 5, 5), T=0.05,
                    room=(4.0 + i, 3.5, 2.8))
        rooms.append(dict(room_sz=cc["room"], beta=cc["beta"], pos_src=cc["ps"], pos_rcv=cc["pr"],
                          nb_img=cc["nb"], Tmax=cc["T"], Tdiff=cc["T"], spkr_pattern="omni",
                          mic_pattern="hypcard", orV_rcv=cc["orv"]))
        betas.append(cc["beta"]); ps_all.append(cc["ps"]); pr_all.append(cc["pr"]); or_all.append(cc["orv"])
    t = lambda a: torch.tensor(np.concatenate(a) if isinstance(a, list) else a, device="cuda",
                               requires_grad=True)
    beta, ps, pr, orv = t(np.stack(betas)), t(ps_all), t(pr_all), t(or_all)
    out = simulate_batch_torch(rooms, 16000.0, beta, ps, pr, None, orv)
    g = torch.tensor(rng.standard_normal(out.shape[0]), device="cuda")
    (out.double() * g).sum().backward()
    views = B.unpack(g.cpu().numpy(), rooms, 16000.0)
    s0 = r0 = 0
    for i, r in enumerate(rooms):
        ns, nr = r["pos_src"].shape[0], r["pos_rcv"].shape[0]
        tt = lambda a: torch.tensor(np.asarray(a, dtype=np.float64), requires_grad=True)
        b64, p64, q64, o64 = tt(r["beta"]), tt(r["pos_src"]), tt(r["pos_rcv"]), tt(r["orV_rcv"])
        h = early_part(r["room_sz"], b64, p64, q64, r["nb_img"], oracle.n_samples(r["Tmax"], 16000.0),
                       16000.0, mic="hypcard", orV_rcv=o64)
        (h * torch.tensor(views[i])).sum().backward()
        assert rel_l2(beta.grad[i].cpu().numpy(), b64.grad.numpy()) < TOL
        assert rel_l2(ps.grad[s0:s0 + ns].cpu().numpy(), p64.grad.numpy()) < TOL
        assert rel_l2(pr.grad[r0:r0 + nr].cpu().numpy(), q64.grad.numpy()) < TOL
        assert rel_l2(orv.grad[r0:r0 + nr].cpu().numpy(), o64.grad.numpy()) < TOL
        s0 += ns
        r0 += nr


def test_inverse_problem_recovers_walls(built):
    """A few Adam steps from beta = 0.8 move toward the walls that made the target."""
    import torch
    from gpurir_gb300.autograd import simulate_rir_torch
    c = _setup(35, "omni", "omni", ns=2, nr=4, nb=(5, 5, 5), T=0.05)
    ps, pr = torch.tensor(c["ps"], device="cuda"), torch.tensor(c["pr"], device="cuda")
    true = torch.tensor(c["beta"], device="cuda")
    with torch.no_grad():
        target = simulate_rir_torch(c["room"], true, ps, pr, c["nb"], c["T"], 16000.0)
    beta = torch.full((6,), 0.8, device="cuda", requires_grad=True)
    opt = torch.optim.Adam([beta], lr=0.01)
    first = None
    for step in range(60):
        opt.zero_grad()
        loss = ((simulate_rir_torch(c["room"], beta, ps, pr, c["nb"], c["T"], 16000.0) - target) ** 2).sum()
        loss.backward()
        opt.step()
        with torch.no_grad():
            beta.clamp_(0.05, 0.999)
        first = first if first is not None else float(loss.detach())
    assert float(loss.detach()) < 0.05 * first
    assert float((beta.detach() - true).abs().max()) < float((0.8 - true).abs().max())


def test_device_beta_forward_matches_host_tables(built):
    """TorchBatch refreshes the rooms' power tables from the device beta; the RIRs
    are those of the batch entry that builds the tables on the host (the same FP64
    products, the same bits)."""
    import torch
    from gpurir_gb300 import batch as B
    from gpurir_gb300.autograd import TorchBatch
    from gpurir_gb300 import workloads
    rooms = workloads.inverse_problem()[:4]
    fs = 16000.0
    host, _ = B.simulate_batch(rooms, fs)
    dev = torch.device("cuda")
    beta = torch.tensor(np.stack([r["beta"] for r in rooms]), device=dev)
    ps = torch.tensor(np.concatenate([r["pos_src"] for r in rooms]), device=dev)
    pr = torch.tensor(np.concatenate([r["pos_rcv"] for r in rooms]), device=dev)
    orv = torch.tensor(np.concatenate([r["orV_rcv"] for r in rooms]), device=dev)
    got = TorchBatch(rooms, fs)(beta, ps, pr, None, orv)
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy(), host.cpu().numpy())


def test_training_step_in_a_cuda_graph(built):
    """TorchBatch only enqueues kernels: forward, loss and adjoint record into one CUDA
    graph, and replays give the eager step's gradients."""
    import torch
    from gpurir_gb300.autograd import TorchBatch
    from gpurir_gb300 import workloads
    rooms = workloads.inverse_problem()[:3]
    fs = 16000.0
    dev = torch.device("cuda")
    model = TorchBatch(rooms, fs)
    beta0 = np.stack([r["beta"] for r in rooms])
    beta = torch.tensor(beta0, device=dev, requires_grad=True)
    ps = torch.tensor(np.concatenate([r["pos_src"] for r in rooms]), device=dev, requires_grad=True)
    pr = torch.tensor(np.concatenate([r["pos_rcv"] for r in rooms]), device=dev)
    orv = torch.tensor(np.concatenate([r["orV_rcv"] for r in rooms]), device=dev)
    target = model(beta.detach() * 0.98, ps.detach(), pr, None, orv).detach()

    def step():
        loss = ((model(beta, ps, pr, None, orv) - target) ** 2).sum()
        loss.backward()

    step()
    eager = (beta.grad.clone(), ps.grad.clone())
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            beta.grad = ps.grad = None
            step()
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    beta.grad = ps.grad = None
    with torch.cuda.graph(graph):
        step()
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(beta.grad, eager[0]) and torch.equal(ps.grad, eager[1])
    assert model.status() == 0


def test_gradients_with_rirs_split_by_images(built):
    """A small launch with many images (1 x 2 RIRs, 17^3 images): the planner splits
    each RIR's images into parts; forward and adjoint still match FP64 autograd."""
    c = _setup(41, "card", "omni", ns=1, nr=2, nb=(17, 17, 17), T=0.05)
    ours, h = _ours(c)
    ref, href = _ref(c)
    assert rel_l2(h.detach().cpu().numpy(), href) < 1e-5
    for k in ours:
        assert rel_l2(ours[k], ref[k]) < TOL, k


def test_gradients_with_segments_past_the_images(built):
    """A long RIR over a small image set: most segments lie past every image's window
    and the adjoint skips them from the actual positions.  One source is outside the
    room (its images reach beyond the in-room delay bound), so a wrong skip would lose
    part of its gradient."""
    c = _setup(37, "card", "omni", ns=2, nr=3, nb=(5, 6, 7), T=0.3)
    c["ps"][1] = np.array([9.0, 1.5, 1.2], np.float32)
    ours, h = _ours(c)
    ref, href = _ref(c)
    assert rel_l2(h.detach().cpu().numpy(), href) < 1e-5
    for k in ours:
        e = rel_l2(ours[k], ref[k])
        assert e < TOL, (k, e)


def test_backward_after_two_forwards_uses_each_calls_beta(built):
    """The backward reuses the room tables of the forward only when no other forward
    ran on the batch in between: two calls with different beta, then one backward,
    give the same gradients as the two calls differentiated one at a time."""
    import torch
    from gpurir_gb300.autograd import TorchBatch
    c = _setup(41, "omni", "card", ns=1, nr=2, nb=(5, 5, 5), T=0.05)
    room = dict(room_sz=c["room"], beta=c["beta"], pos_src=c["ps"], pos_rcv=c["pr"], nb_img=c["nb"],
                Tmax=c["T"], Tdiff=c["T"], spkr_pattern="omni", mic_pattern="card")
    model = TorchBatch([room], 16000.0)
    rng = np.random.default_rng(5)
    b1 = torch.tensor(c["beta"][None], device="cuda")
    b2 = torch.tensor(np.clip(c["beta"][None] - 0.1, 0.0, 1.0), device="cuda")
    ps, pr = torch.tensor(c["ps"], device="cuda"), torch.tensor(c["pr"], device="cuda")
    orv = torch.tensor(c["orv"], device="cuda")
    g1 = torch.tensor(rng.standard_normal(model.total), dtype=torch.float32, device="cuda")
    g2 = torch.tensor(rng.standard_normal(model.total), dtype=torch.float32, device="cuda")

    def grads(pairs):
        out = []
        for b, g in pairs:
            x = b.clone().requires_grad_(True)
            out.append((x, (model(x, ps, pr, None, orv) * g).sum()))
        sum(l for _, l in out).backward()
        return [x.grad.cpu().numpy() for x, _ in out]

    both = grads([(b1, g1), (b2, g2)])
    one1, = grads([(b1, g1)])
    one2, = grads([(b2, g2)])
    assert np.array_equal(both[0], one1) and np.array_equal(both[1], one2)
    assert not np.allclose(one1, one2)


@pytest.mark.parametrize("fs", [22050.0, 48000.0])
def test_gradients_at_other_sample_rates(built, fs):
    """Windows that do not fill the lanes exactly (Tw = 176 and 384 samples: 8 and 12 taps
    per lane, taps beyond |x| < Tw/2 masked) against the FP64 reference."""
    c = _setup(43, "card", "hypcard", nb=(4, 5, 6), T=0.05, fs=fs)
    ours, h = _ours(c)
    ref, href = _ref(c)
    assert rel_l2(h.detach().cpu().numpy(), href) < 1e-5
    for k in ours:
        e = rel_l2(ours[k], ref[k])
        assert e < TOL, (fs, k, e)


def test_fused_l2_step_matches_composed_step(built):
    """TorchBatch.l2_loss and TorchBatch.l2_step (forward, loss, its gradient and the
    adjoint in one call) give the gradients of the autograd-composed step bit for
    bit (the same 2 (y - t) and the same deterministic adjoint) and the same loss
    to float rounding; reduction "mean" scales both by 1 / n."""
    import torch
    from gpurir_gb300.autograd import TorchBatch
    from gpurir_gb300 import workloads
    rooms = workloads.inverse_problem()[:4]
    fs = 16000.0
    dev = torch.device("cuda")
    model = TorchBatch(rooms, fs)
    t = lambda a: torch.tensor(a, device=dev, requires_grad=True)
    beta = t(np.stack([r["beta"] for r in rooms]))
    ps = t(np.concatenate([r["pos_src"] for r in rooms]))
    pr = t(np.concatenate([r["pos_rcv"] for r in rooms]))
    orv = t(np.concatenate([r["orV_rcv"] for r in rooms]))
    params = (beta, ps, pr, orv)
    target = model(beta.detach() * 0.97, ps.detach(), pr.detach(), None, orv.detach()).detach()
    loss_c = ((model(beta, ps, pr, None, orv) - target) ** 2).sum()
    loss_c.backward()
    comp = [x.grad.clone() for x in params]
    for x in params:
        x.grad = None
    loss_f = model.l2_loss(beta, ps, pr, None, orv, target)
    loss_f.backward()
    for a, x in zip(comp, params):
        assert torch.equal(a, x.grad)
    assert abs(float(loss_f.detach()) - float(loss_c.detach())) <= 1e-5 * float(loss_c.detach())
    assert torch.equal(model.last_rirs, model(beta, ps, pr, None, orv).detach())
    # the graph-free step overwrites .grad with the same values
    loss_s = model.l2_step(beta, ps, pr, None, orv, target)
    for a, x in zip(comp, params):
        assert torch.equal(a, x.grad)
    assert float(loss_s) == float(loss_f)
    for x in params:
        x.grad = None
    loss_m = model.l2_loss(beta, ps, pr, None, orv, target, reduction="mean")
    loss_m.backward()
    assert abs(float(loss_m) * model.total - float(loss_c)) <= 1e-5 * float(loss_c)
    assert torch.allclose(beta.grad * model.total, comp[0], rtol=1e-5, atol=0)
    assert model.status() == 0


def test_inverse_problem_200_adam_steps(built):
    """The inverse-problem workload at full size (16 rooms x 4 sources x 8
    hypercardioid receivers, 0.4 s, nb_img [9, 11, 13]): 200 Adam steps on beta
    from 0.8 through the fused L2 step.  The loss falls by orders of magnitude
    and every wall moves to the one that made the target."""
    import torch
    from gpurir_gb300.autograd import TorchBatch
    from gpurir_gb300 import workloads
    rooms = workloads.inverse_problem()
    fs = 16000.0
    dev = torch.device("cuda")
    model = TorchBatch(rooms, fs)
    true = torch.tensor(np.stack([r["beta"] for r in rooms]), device=dev)
    ps = torch.tensor(np.concatenate([r["pos_src"] for r in rooms]), device=dev)
    pr = torch.tensor(np.concatenate([r["pos_rcv"] for r in rooms]), device=dev)
    orv = torch.tensor(np.concatenate([r["orV_rcv"] for r in rooms]), device=dev)
    with torch.no_grad():
        target = model(true, ps, pr, None, orv).clone()
    beta = torch.full((16, 6), 0.8, device=dev, requires_grad=True)
    opt = torch.optim.Adam([beta], lr=0.01)
    losses = []
    for step in range(200):
        loss = model.l2_step(beta, ps, pr, None, orv, target)
        losses.append(loss.clone())
        opt.step()
        with torch.no_grad():
            beta.clamp_(0.05, 0.999)
    losses = [float(x) for x in losses]
    err0 = float((0.8 - true).abs().max())
    err = float((beta.detach() - true).abs().max())
    print("loss %.3e -> %.3e, max |beta - true| %.3f -> %.4f" % (losses[0], losses[-1], err0, err))
    assert losses[-1] < 1e-3 * losses[0]
    assert err < 0.1 * err0
    assert model.status() == 0
