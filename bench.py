#!/usr/bin/env python3
"""Throughput benchmark of the gpurir_gb300 forward path on one or more GB300s.

One step = one simulateRIR of the mic_array workload: 64 omni sources x 32
cardioid receivers in a 6 x 5 x 3 m room, Sabine beta at T60 = 1 s, early part
by the ISM up to Tdiff = 0.3 s (nb_img [12, 14, 24]), Gaussian diffuse tail up
to Tmax = 1 s, fs = 16 kHz, FP32: 2048 RIRs of 16000 samples per step.

  value  RIRs/s with inputs resident in HBM (device entry of the C ABI),
         device time from CUDA events on the launch stream, L2 flushed
         (256 MiB write) before every timed step, max over ranks.
  e2e    the same metric through the host entry of the C ABI
         (gpurir_simulate_rir): positions from host memory, RIRs returned into
         pinned host memory, both copies inside the timed region.

--impl reference times the CPU restatement of the path (FP32, all host
threads) on a bounded sample of the same workload: the reference library has
no CPU implementation and its CUDA build cannot run here.
Multi-GPU: every rank simulates its own copy of the workload (independent
RIRs, no collective on the data path): weak scaling.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = ("RIRs/s & image-sample updates/s, batched vs plain fwd; fwd+adjoint step time, 1 GB300")
WORKLOAD = "mic_array"
WORKLOAD_DESC = ("mic_array: room 6x5x3 m, Sabine beta (T60 1.0 s), 64 omni src x 32 cardioid rcv, "
                 "nb_img [12,14,24], Tdiff 0.3 s, Tmax 1.0 s, fs 16 kHz, Gaussian tail, FP32")
FLOPS_PER_UPDATE = 8      # FP32 ops per windowed update of the reference formula
SFU_PER_UPDATE = 3        # transcendental ops (sin, cos, reciprocal) per update


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=300)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the batched / adjoint / trajectory measurements")
    p.add_argument("--extras", default="batched,inverse,trajectory,tuning,modes",
                   help="comma list of the extra measurements to run (batched, inverse, trajectory, tuning, "
                        "modes)")
    return p.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def _cpu_port_sample(scene, n_src, threads):
    """(RIRs, windowed updates, seconds) of the FP32 CPU restatement of the whole
    per-RIR work (early part, envelope, diffuse tail: every sample of every RIR)
    on the first `n_src` sources and all receivers."""
    import oracle
    t = time.perf_counter()
    out, upd = oracle.rir_f32(scene["room_sz"], scene["beta"], scene["pos_src"][:n_src],
                              scene["pos_rcv"], scene["nb_img"], scene["Tmax"], scene["fs"],
                              scene["Tdiff"], scene["spkr_pattern"], scene["mic_pattern"], None,
                              scene["orV_rcv"], scene["c"], noise=scene["noise"], n_threads=threads)
    dt = time.perf_counter() - t
    return n_src * scene["pos_rcv"].shape[0], upd, dt


def _accuracy(G, scene, d_out, seed, offset):
    """Max-abs and relative-L2 error of an output of the mic_array workload against
    the FP64 oracle, on 64 RIRs spread over the sources and receivers (every 8th
    source x every 4th receiver), early part and tail separately."""
    import oracle
    ms, mr = scene["pos_src"].shape[0], scene["pos_rcv"].shape[0]
    src_i, rcv_i = np.arange(0, ms, 8), np.arange(0, mr, 4)
    got = d_out[src_i][:, rcv_i].cpu().numpy().astype(np.float64)
    want = np.zeros_like(got)
    n_ism = None
    for a, s_idx in enumerate(src_i):
        ref, parts = oracle.simulate_rir(
            scene["room_sz"], scene["beta"], scene["pos_src"][s_idx:s_idx + 1], scene["pos_rcv"][rcv_i],
            scene["nb_img"], scene["Tmax"], scene["fs"], scene["Tdiff"], scene["spkr_pattern"],
            scene["mic_pattern"], None, scene["orV_rcv"][rcv_i], scene["c"], seed=seed, offset=offset,
            noise=scene["noise"], return_parts=True, rir_index=s_idx * mr + rcv_i)
        want[a] = ref[0]
        n_ism = parts["n_ism"]

    def stats(x, y):
        n = float(np.linalg.norm(y))
        return {"rel_l2": float(np.linalg.norm(x - y)) / n if n > 0 else None,
                "max_abs": float(np.abs(x - y).max()), "ref_max_abs": float(np.abs(y).max())}

    return {"vs": "fp64 oracle (oracle/ism_oracle.c)", "rirs_checked": int(got.shape[0] * got.shape[1]),
            "which": "timed output of the last step: sources 0,8,..,56 x receivers 0,4,..,28",
            "early": stats(got[..., :n_ism], want[..., :n_ism]),
            "tail": stats(got[..., n_ism:], want[..., n_ism:]),
            "note": "the tail of this workload is silent: its images end before the 10 ms envelope "
                    "window at Tdiff (nb_img [12,14,24] reaches ~0.18 s), so A = 0 in both"}


def run_reference(a):
    rank, world, _ = _dist()
    if rank != 0:
        return
    from gpurir_gb300 import workloads
    scene = workloads.mic_array()
    threads = os.cpu_count() or 1
    n_src = 4
    for _ in range(min(max(a.warmup, 1), 3)):
        _cpu_port_sample(scene, n_src, threads)
    times, n_rir, upd = [], 0, 0
    for _ in range(a.steps):
        n_rir, upd, dt = _cpu_port_sample(scene, n_src, threads)
        times.append(dt)
    step_s = sum(times) / len(times)
    value = n_rir / step_s
    sample = ("%d of 64 sources x 32 receivers (%d RIRs) per step, every sample of each RIR (early "
              "part, envelope, diffuse tail): the same per-RIR work as the GPU arm" % (n_src, n_rir))
    line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "RIRs/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": step_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": {"workload": WORKLOAD_DESC},
            "updates_per_s": upd / step_s,
            "cpu_baseline": {"value": value, "unit": "RIRs/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "RIRs/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "same_config": True,
            "note": "runs on the host cores: the reference has no CPU implementation of the path, "
                    "so its FP32 restatement (OpenMP, windowed, early part + envelope + tail) is "
                    "timed; gpuRIR's own CUDA kernels on the same GPU are timed by "
                    "oracle/time_reference_kernels.py"}
    print(json.dumps(line), flush=True)


def _traffic(workload):
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get(workload)
    except (OSError, ValueError):
        return None


def _measured_hbm_gbs():
    """HBM copy bandwidth measured on this machine's GPUs (MEASURED_PEAKS.json), or None."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, ValueError, KeyError, TypeError):
        return None


def _timed(fn, steps, stream, flush=None):
    """Median device time (ms) of fn() over `steps` runs, CUDA events on `stream`."""
    import torch
    ts = []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    ts.sort()
    return ts[len(ts) // 2]


def run_extras(G, flush, stream, which=("batched", "inverse", "trajectory", "tuning", "modes")):
    """The metric's other parts: batched vs plain forward (512 uneven rooms), forward +
    adjoint step vs forward (16 rooms x 32 RIRs), trajectory filtering (400 points)."""
    import torch
    from gpurir_gb300 import batch as B, workloads
    out = {}
    fs = 16000.0
    dev = stream.device
    sim = G.Simulator(seed=7)
    if "batched" in which:
        out.update(_extra_batched(G, B, workloads, sim, flush, stream, fs, dev))
    if "inverse" in which:
        out.update(_extra_inverse(workloads, sim, flush, stream, fs, dev))
    if "trajectory" in which:
        out.update(_extra_trajectory(workloads, sim, flush, stream, fs, dev))
    if "tuning" in which:
        out.update(_extra_tuning(G, B, workloads, flush, stream, fs, dev))
    if "modes" in which:
        out.update(_extra_modes(G, workloads, flush, stream, dev))
    return out


def _extra_modes(G, workloads, flush, stream, dev):
    """The main workload (mic_array) in gpuRIR's two other evaluation modes, mixed
    precision and lookup table: kernel time and the error of the timed output against
    the FP64 oracle, as for the FP32 line."""
    import torch
    scene = workloads.mic_array()
    sp, mp = G.polar_patterns[scene["spkr_pattern"]], G.polar_patterns[scene["mic_pattern"]]
    ms, mr = scene["pos_src"].shape[0], scene["pos_rcv"].shape[0]
    ns = workloads.n_samples(scene["Tmax"], scene["fs"])
    d_ps = torch.from_numpy(scene["pos_src"]).to(dev)
    d_pr = torch.from_numpy(scene["pos_rcv"]).to(dev)
    d_or = torch.from_numpy(scene["orV_rcv"]).to(dev)
    d_out = torch.empty((ms, mr, ns), dtype=torch.float32, device=dev)
    res = {}
    for name in ("mixed_precision", "lut"):
        sim = G.Simulator(mixed_precision=name == "mixed_precision", lut=name == "lut", seed=1234)
        sim.set_noise(scene["noise"])

        def step():
            sim.simulate_rir_device(scene["room_sz"], scene["beta"], d_ps, d_pr, None, d_or, sp, mp,
                                    scene["nb_img"], scene["Tdiff"], scene["Tmax"], scene["fs"],
                                    scene["c"], d_out, stream.cuda_stream)

        for _ in range(3):
            step()
        t = _timed(step, 20, stream, flush)
        seed_used, calls_after = sim.get_seed()
        acc = _accuracy(G, scene, d_out, seed_used, calls_after - 1)
        res[name] = {"ms_per_step": t, "rirs_per_s": ms * mr / (t * 1e-3), "accuracy": acc["early"],
                     "rirs_checked": acc["rirs_checked"]}
    return {"modes": dict(res, note="mic_array in each mode, device-resident, L2 flushed; accuracy of the "
                                    "early part of 64 timed RIRs against the FP64 oracle (exact sinc "
                                    "sum); FP32 is the main line")}


def _extra_tuning(G, B, workloads, flush, stream, fs, dev):
    """The autotuner on this GPU, then the batched-rooms replay and the fused
    inverse-problem step with the default and with the tuned launch shapes."""
    import torch
    from gpurir_gb300 import tune
    from gpurir_gb300.autograd import TorchBatch
    entry = tune.tune(reps=5, warmup=2, write=False)
    rooms = workloads.batched_rooms()
    inv = workloads.inverse_problem()
    t = lambda a, g=False: torch.tensor(a, device=dev, requires_grad=g)
    beta = t(np.stack([r["beta"] for r in inv]), True)
    ps = t(np.concatenate([r["pos_src"] for r in inv]))
    pr = t(np.concatenate([r["pos_rcv"] for r in inv]))
    orv = t(np.concatenate([r["orV_rcv"] for r in inv]))
    res = {}
    for label, knobs in (("default", None), ("tuned", entry["knobs"])):
        tune.reset()
        if knobs:
            tune.set_knobs(knobs)
        sim = G.Simulator(seed=9)
        plan = B.BatchPlan(rooms, fs, sim=sim)
        for _ in range(2):
            plan.launch(stream.cuda_stream)
        tb = _timed(lambda: plan.launch(stream.cuda_stream), 10, stream, flush)
        model = TorchBatch(inv, fs, sim=sim)
        target = model(beta.detach() * 0.99, ps, pr, None, orv).detach()
        for _ in range(3):
            model.l2_step(beta, ps, pr, None, orv, target)
        ti = _timed(lambda: model.l2_step(beta, ps, pr, None, orv, target), 20, stream, flush)
        res[label] = {"batched_ms": tb, "inverse_l2_step_ms": ti}
        del plan, model
    tune.reset()
    return {"tuning": {"knobs": entry["knobs"], "candidates_ms": entry["timings_ms"], "tuned_s": entry["tuned_s"],
                       "default": res["default"], "tuned": res["tuned"],
                       "note": "launch-shape knobs only (results bitwise equal for every candidate); "
                               "batched = 512-room graph replay, inverse = fused L2 step"}}


def _extra_batched(G, B, workloads, sim, flush, stream, fs, dev):
    import torch
    out = {}
    # -- batched rooms: one captured launch vs one call per room
    rooms = workloads.batched_rooms()
    n_rir = sum(r["pos_src"].shape[0] * r["pos_rcv"].shape[0] for r in rooms)
    plan = B.BatchPlan(rooms, fs, sim=sim)
    for _ in range(2):
        plan.launch(stream.cuda_stream)
    t_batch = _timed(lambda: plan.launch(stream.cuda_stream), 10, stream, flush)
    per_room = []
    for r in rooms:
        d = lambda x: torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(dev)
        o = torch.empty((r["pos_src"].shape[0], r["pos_rcv"].shape[0],
                         workloads.n_samples(r["Tmax"], fs)), device=dev)
        per_room.append((r, d(r["pos_src"]), d(r["pos_rcv"]), o))

    def plain():
        for r, ps, pr, o in per_room:
            sim.simulate_rir_device(r["room_sz"], r["beta"], ps, pr, None, None, 0, 0, r["nb_img"],
                                    r["Tdiff"], r["Tmax"], fs, 343.0, o, stream.cuda_stream)

    plain()
    t_plain = _timed(plain, 3, stream, flush)
    upd = sum(workloads.windowed_updates_torch(dict(r, fs=fs)) for r in rooms)
    # the plain single-room configuration (2 RIRs, 0.5 s, full ISM) through the same entry
    pr_scene = workloads.plain_room()
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(dev)
    p_ps, p_pr = d(pr_scene["pos_src"]), d(pr_scene["pos_rcv"])
    p_out = torch.empty((p_ps.shape[0], p_pr.shape[0], workloads.n_samples(pr_scene["Tmax"], fs)), device=dev)

    def single():
        sim.simulate_rir_device(pr_scene["room_sz"], pr_scene["beta"], p_ps, p_pr, None, None, 0, 0,
                                pr_scene["nb_img"], pr_scene["Tdiff"], pr_scene["Tmax"], fs, 343.0, p_out,
                                stream.cuda_stream)

    single()
    t_single = _timed(single, 20, stream, flush)
    n_single = p_ps.shape[0] * p_pr.shape[0]
    upd_single = workloads.windowed_updates_torch(dict(pr_scene, fs=fs))
    out["batched_rooms"] = {
        "rooms": len(rooms), "rirs": n_rir, "windowed_updates": upd,
        "batched_ms": t_batch, "batched_rirs_per_s": n_rir / (t_batch * 1e-3),
        "batched_updates_per_s": upd / (t_batch * 1e-3),
        "plain_loop_ms": t_plain, "plain_loop_rirs_per_s": n_rir / (t_plain * 1e-3),
        "batched_over_plain": t_plain / t_batch,
        "plain_room_ms": t_single, "plain_room_rirs_per_s": n_single / (t_single * 1e-3),
        "plain_room_updates_per_s": upd_single / (t_single * 1e-3),
        "batched_over_plain_room_updates": (upd / t_batch) / (upd_single / t_single),
        "note": "batched = one CUDA-graph replay of all 512 rooms; plain = one device-API call "
                "per room on the same stream; plain_room = the plain single-room configuration "
                "(2 RIRs, 0.5 s, full ISM) per device-API call"}
    return out


def _extra_inverse(workloads, sim, flush, stream, fs, dev):
    import torch
    out = {}
    # -- forward + adjoint step of the inverse problem
    from gpurir_gb300.autograd import TorchBatch
    inv = workloads.inverse_problem()
    model = TorchBatch(inv, fs, sim=sim)
    beta = torch.tensor(np.stack([r["beta"] for r in inv]), device=dev, requires_grad=True)
    ps = torch.tensor(np.concatenate([r["pos_src"] for r in inv]), device=dev, requires_grad=True)
    pr = torch.tensor(np.concatenate([r["pos_rcv"] for r in inv]), device=dev, requires_grad=True)
    orv = torch.tensor(np.concatenate([r["orV_rcv"] for r in inv]), device=dev)
    target = model(beta.detach() * 0.99, ps.detach(), pr.detach(), None, orv).detach()

    def fwd():
        with torch.no_grad():
            model(beta, ps, pr, None, orv)

    def fwd_bwd():
        loss = torch.nn.functional.mse_loss(model(beta, ps, pr, None, orv), target, reduction="sum")
        loss.backward()

    for _ in range(3):
        fwd(); fwd_bwd()
    t_f = _timed(fwd, 20, stream, flush)
    t_fb = _timed(fwd_bwd, 20, stream, flush)
    # the same step recorded once in a CUDA graph (our calls only enqueue kernels) and
    # replayed: what the GPU spends on it without PyTorch's per-op host overhead
    side = torch.cuda.Stream(device=dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(side):
        for _ in range(3):
            beta.grad = ps.grad = pr.grad = None
            fwd_bwd()
            fwd()
    torch.cuda.current_stream(dev).wait_stream(side)
    g_f, g_fb = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
    with torch.cuda.graph(g_f):
        fwd()
    beta.grad = ps.grad = pr.grad = None
    with torch.cuda.graph(g_fb):
        fwd_bwd()
    t_gf = _timed(g_f.replay, 20, stream, flush)
    t_gfb = _timed(g_fb.replay, 20, stream, flush)

    # the same step through the fused L2 entry: forward, loss, its gradient and the adjoint
    # in one C call that writes the parameters' .grad (no autograd graph)
    def fused_step():
        model.l2_step(beta, ps, pr, None, orv, target)

    for _ in range(3):
        fused_step()
    t_fused = _timed(fused_step, 20, stream, flush)

    # what one backward() call costs PyTorch itself on this host, whatever the graph:
    # a trivial loss of a leaf tensor of the same size (host-bound, no kernel of ours)
    leaf = torch.zeros(model.total, device=dev, requires_grad=True)

    def trivial_bwd():
        (leaf * 2.0).sum().backward()

    for _ in range(3):
        trivial_bwd()
    t_triv = _timed(trivial_bwd, 20, stream, flush)
    out["inverse_problem"] = {"rirs": 16 * 32, "forward_ms": t_f, "forward_adjoint_ms": t_fb,
                              "adjoint_over_forward": t_fb / t_f,
                              "graph_forward_ms": t_gf, "graph_forward_adjoint_ms": t_gfb,
                              "graph_adjoint_over_forward": t_gfb / t_gf,
                              "fused_l2_step_ms": t_fused, "fused_l2_step_over_forward": t_fused / t_f,
                              "torch_trivial_backward_ms": t_triv,
                              "note": "grads of an L2 loss w.r.t. beta[16,6], pos_src[64,3], "
                                      "pos_rcv[128,3]; beta stays on the device (TorchBatch). "
                                      "forward_adjoint_ms is the eager autograd step (model, "
                                      "mse_loss, backward()): host-bound, and "
                                      "torch_trivial_backward_ms, one backward() of (x * 2).sum() "
                                      "on a leaf, is what PyTorch alone spends per backward() "
                                      "call on this host"}
    return out


def _extra_trajectory(workloads, sim, flush, stream, fs, dev):
    import torch
    out = {}
    # -- trajectory: RIRs simulated on the device, then convolution + overlap-add
    tr = workloads.trajectory()
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(dev)
    tps, tpr = d(tr["pos_src"]), d(tr["pos_rcv"])
    rirs = torch.empty((400, 8, 12800), device=dev)
    from gpurir_gb300.trajectory import simulate_trajectory
    sim.simulate_rir_device(tr["room_sz"], tr["beta"], tps, tpr, None, None, 0, 0, tr["nb_img"],
                            tr["Tdiff"], tr["Tmax"], fs, 343.0, rirs, stream.cuda_stream)
    simulate_trajectory(tr["signal"], rirs, sim=sim)
    t_rir = _timed(lambda: sim.simulate_rir_device(tr["room_sz"], tr["beta"], tps, tpr, None, None, 0, 0,
                                                   tr["nb_img"], tr["Tdiff"], tr["Tmax"], fs, 343.0,
                                                   rirs, stream.cuda_stream), 10, stream, flush)
    t_conv = _timed(lambda: simulate_trajectory(tr["signal"], rirs, sim=sim), 10, stream, flush)
    conv_bytes = 4 * (400 * 8 * 12800 + 400 * 400 + 2 * 400 * 8 * (400 + 12799)) + 8 * 8 * (160000 + 12799)
    out["trajectory"] = {"rir_ms": t_rir, "convolution_ola_ms": t_conv,
                         "conv_hbm_gbs": conv_bytes / (t_conv * 1e-3) / 1e9,
                         "note": "400 points x 8 mics, 12800-sample RIRs, 10 s signal; segments "
                                 "uploaded from host memory inside the timed call"}
    # forward + adjoint: RIRs from the differentiable batch (beta on the device), the filtered
    # signal, an L2 loss against a target, gradients w.r.t. the signal and beta
    from gpurir_gb300.autograd import TorchBatch
    from gpurir_gb300.trajectory import simulate_trajectory_torch
    model = TorchBatch([dict(tr, spkr_pattern="omni", mic_pattern="omni")], fs, sim=sim)
    beta = torch.tensor(np.asarray(tr["beta"], np.float32), device=dev).reshape(1, 6).requires_grad_(True)
    sig = torch.from_numpy(tr["signal"]).to(dev).requires_grad_(True)
    with torch.no_grad():
        target = simulate_trajectory_torch(sig, model(beta * 0.99, tps, tpr).view(400, 8, 12800), sim=sim)

    def t_fwd():
        with torch.no_grad():
            simulate_trajectory_torch(sig, model(beta, tps, tpr).view(400, 8, 12800), sim=sim)

    def t_fwd_bwd():
        y = simulate_trajectory_torch(sig, model(beta, tps, tpr).view(400, 8, 12800), sim=sim)
        ((y - target) ** 2).sum().backward()

    for _ in range(3):
        t_fwd(); t_fwd_bwd()
    tf = _timed(t_fwd, 10, stream, flush)
    tfb = _timed(t_fwd_bwd, 10, stream, flush)
    out["trajectory"].update({"forward_ms": tf, "forward_adjoint_ms": tfb, "adjoint_over_forward": tfb / tf,
                              "adjoint_note": "RIRs (early part + tail) and the filtered signal; then "
                                              "dL/dsignal [160000] and dL/dbeta [6] of an L2 loss, through "
                                              "the trajectory adjoint (FFT correlations) and the "
                                              "image-source adjoint"})
    return out


def run_gpu(a):
    import torch
    rank, world, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import gpurir_gb300 as G
    from gpurir_gb300 import workloads
    scene = workloads.mic_array()
    sp, mp = G.polar_patterns[scene["spkr_pattern"]], G.polar_patterns[scene["mic_pattern"]]
    ms, mr = scene["pos_src"].shape[0], scene["pos_rcv"].shape[0]
    M = ms * mr
    ns = workloads.n_samples(scene["Tmax"], scene["fs"])
    sim = G.Simulator(seed=1234 + rank)
    sim.set_noise(scene["noise"])
    sim.set_profiling(True)
    dev = torch.device("cuda", local)
    d_ps = torch.from_numpy(scene["pos_src"]).to(dev)
    d_pr = torch.from_numpy(scene["pos_rcv"]).to(dev)
    d_or = torch.from_numpy(scene["orV_rcv"]).to(dev)
    d_out = torch.empty((ms, mr, ns), dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        sim.simulate_rir_device(scene["room_sz"], scene["beta"], d_ps, d_pr, None, d_or, sp, mp,
                                scene["nb_img"], scene["Tdiff"], scene["Tmax"], scene["fs"],
                                scene["c"], d_out, stream.cuda_stream)

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    fp32_flops, mufu_ops = G.probe_peaks()
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    total_ms, ism_ms, tail_ms, launches = 0.0, [], [], 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(a.steps):
        flush.zero_()
        ev0.record(stream)
        step()
        ev1.record(stream)
        ev1.synchronize()
        total_ms += ev0.elapsed_time(ev1)
        i_ms, t_ms = sim.last_timing()
        launches += sim.last_launch_count()
        ism_ms.append(i_ms)
        tail_ms.append(t_ms)
    torch.cuda.synchronize()
    if world > 1:
        from gpurir_gb300.replicas import max_over_ranks
        torch.distributed.barrier()
        total_ms = max_over_ranks(total_ms)
    clk = clocks.stop()
    # accuracy of the timed output (outside the timed region): the last step drew the
    # tail of call counter calls - 1
    seed_used, calls_after = sim.get_seed()
    accuracy = _accuracy(G, scene, d_out, seed_used, calls_after - 1) if rank == 0 else None
    ms_per_step = total_ms / a.steps
    value = world * M * a.steps / (total_ms * 1e-3)

    # end to end through the host entry (positions from host memory, RIRs to pinned memory)
    h_out = torch.empty((ms, mr, ns), dtype=torch.float32, pin_memory=True).numpy()

    def host_step():
        sim.simulate_rir(scene["room_sz"], scene["beta"], scene["pos_src"], scene["pos_rcv"],
                         None, scene["orV_rcv"], sp, mp, scene["nb_img"], scene["Tdiff"],
                         scene["Tmax"], scene["fs"], scene["c"], out=h_out)

    for _ in range(max(2, a.warmup // 2)):
        host_step()
    e2e_s, e2e_kernel_ms = 0.0, 0.0
    for _ in range(a.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_step()
        e2e_s += time.perf_counter() - t0
        e2e_kernel_ms += sim.last_timing()[0]
    h2d, d2h = sim.last_transfer_bytes()
    direct = sim.last_output_direct()
    if world > 1:
        from gpurir_gb300.replicas import max_over_ranks
        e2e_s = max_over_ranks(e2e_s)
    e2e_value = world * M * a.steps / e2e_s

    if rank != 0:
        return
    updates, brute = workloads.windowed_updates(scene)
    ism_avg = sum(ism_ms) / len(ism_ms)
    upd_per_s = updates / (ism_avg * 1e-3)
    sfu_ach = upd_per_s * SFU_PER_UPDATE
    fp32_ach = upd_per_s * FLOPS_PER_UPDATE
    frac_sfu = sfu_ach / mufu_ops
    frac_fp32 = fp32_ach / (fp32_flops / 2.0)
    use_sfu = frac_sfu >= frac_fp32
    traffic = _traffic(WORKLOAD)
    roofline = {
        "bound": "sfu" if use_sfu else "fp32",
        "achieved": (sfu_ach if use_sfu else fp32_ach) / 1e12,
        "peak": (mufu_ops if use_sfu else fp32_flops / 2.0) / 1e12,
        "unit": "Tops/s",
        "frac": frac_sfu if use_sfu else frac_fp32,
        "traffic": traffic,
        "kernel": "ism_forward_kernel<4, 0> (diffuse tail fused into its epilogue)",
        "basis": "%d transcendental + %d FP32 ops per windowed image-sample update; %d updates "
                 "per launch; peaks measured on this device (MUFU rcp, FP32 FMA)" %
                 (SFU_PER_UPDATE, FLOPS_PER_UPDATE, updates),
        "frac_fp32": frac_fp32, "frac_sfu": frac_sfu,
        "peak_fp32_tflops_measured": fp32_flops / 1e12, "peak_mufu_tops_measured": mufu_ops / 1e12,
        "ism_ms": ism_avg,
        "why_not_hbm_or_tensor": "no dense contraction (no tensor-core work) and ~71 MB of DRAM "
                                 "traffic per 0.5 ms launch: the kernel is bound by special-function "
                                 "and issue throughput, so its fraction is taken against the MUFU "
                                 "and FP32 peaks measured on the device",
    }
    hbm_peak = _measured_hbm_gbs()
    if traffic and hbm_peak:
        hbm_ach = traffic / (ism_avg * 1e-3) / 1e9
        roofline["hbm"] = {"achieved": hbm_ach, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_ach / hbm_peak,
                           "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
    line = {"metric": METRIC, "value": value, "unit": "RIRs/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD_DESC, "rirs_per_step": M, "samples_per_rir": ns,
                       "windowed_updates_per_step": updates, "brute_force_evaluations": brute,
                       "l2": "flushed (256 MiB write) before every timed step",
                       "parallelism": "replicas" if world > 1 else "single"},
            "updates_per_s": updates * world * a.steps / (total_ms * 1e-3),
            "kernel_ms": {"ism_forward": ism_avg, "tail": sum(tail_ms) / len(tail_ms)},
            "e2e": {"value": e2e_value, "unit": "RIRs/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s / a.steps * 1e3,
                    "kernel_ms": e2e_kernel_ms / a.steps,
                    "d2h": ("the kernel stores the RIRs into the pinned host buffer over the host "
                            "link; tails silent by geometry are streamed there meanwhile by a copy "
                            "engine from a device zero buffer (kernel_ms: the kernel alone)") if direct
                           else "cudaMemcpyAsync after the kernels"},
            "roofline": roofline, "clocks": clk, "gpu_launches": launches, "accuracy": accuracy}
    if world == 1 and not a.no_extras:
        line["workloads"] = run_extras(G, flush, stream, tuple(a.extras.split(",")))
    if world == 1 and not a.no_cpu_baseline:
        scene_cpu = workloads.mic_array()
        threads = os.cpu_count() or 1
        n_rir, upd, dt = _cpu_port_sample(scene_cpu, 16, threads)
        line["cpu_baseline"] = {"value": n_rir / dt, "unit": "RIRs/s", "cores": threads,
                                "kind": "port", "updates_per_s": upd / dt,
                                "sample": "16 of 64 sources x 32 receivers (%d RIRs), every sample "
                                          "(early part, envelope, tail), FP32 OpenMP restatement" % n_rir}
    print(json.dumps(line), flush=True)


def main():
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_gpu(a)
    if int(os.environ.get("WORLD_SIZE", "1")) > 1 and a.impl != "reference":
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
