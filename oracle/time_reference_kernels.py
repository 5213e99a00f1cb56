"""Times gpuRIR's own CUDA kernels on this GPU beside this engine, on the
benchmark workloads.  Measurement infrastructure: it runs the reference's
kernels (oracle/_ref/gpuRIR_ref.cubin, built by oracle.ref_kernels.build_ref
from the reference sources) through the host replay of oracle.ref_kernels, the
way cuda_simulateRIR (src/gpuRIR_cuda.cu:766-931) drives them: one synchronised
kernel after another, outputs copied to pageable host memory at the end.

Per simulateRIR call it reports
  device_ms  CUDA-event time of the reference's kernel sequence (calcAmpTau,
             generateRIR or its MP / LUT variant, the reduceRIR ladder, envPred,
             the uniform fill, diffRev).  The uniform fill is torch.rand of the
             same size standing in for curandGenerateUniform; buffers come from
             torch's caching allocator, cheaper than the reference's per-call
             cudaMalloc / cudaFree.
  call_ms    wall time of the call including the copies of the early part and
             the tail to host memory.
and the same call through this engine's public API (host arrays in and out).

    python oracle/time_reference_kernels.py [--out FILE]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import ref_kernels  # noqa: E402

_PAT = {"omni": 0, "homni": 1, "card": 2, "hypcard": 3, "subcard": 4, "bidir": 5}


def _ref_call(rk, torch, sc, mode):
    kw = dict(room_sz=sc["room_sz"], beta=sc["beta"], pos_src=sc["pos_src"], pos_rcv=sc["pos_rcv"],
              nb_img=sc["nb_img"], Tmax=sc["Tmax"], fs=sc["fs"], Tdiff=sc.get("Tdiff"),
              spkr_pattern=_PAT[sc.get("spkr_pattern", "omni")], mic_pattern=_PAT[sc.get("mic_pattern", "omni")],
              orV_src=sc.get("orV_src"), orV_rcv=sc.get("orV_rcv"), c=sc.get("c", 343.0))
    ms, mr = len(sc["pos_src"]), len(sc["pos_rcv"])
    n_ism = ref_kernels._n_samples(sc.get("Tdiff") or sc["Tmax"], sc["fs"])
    n_diff = ref_kernels._n_samples(sc["Tmax"], sc["fs"]) - n_ism
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    u = torch.rand(ms * mr * n_diff, device="cuda") if n_diff > 0 else None
    r = rk.simulate(mode=mode, uniforms=u, host=False, **kw)
    e1.record()
    early = r["early"].cpu().numpy()
    if n_diff > 0:
        diff = r["diffuse"].cpu().numpy()
        del diff
    t1 = time.perf_counter()
    torch.cuda.synchronize()
    del early
    return e0.elapsed_time(e1), (t1 - t0) * 1e3


def _engine_call(sim, sc):
    t0 = time.perf_counter()
    sim.simulate_rir(sc["room_sz"], sc["beta"], sc["pos_src"], sc["pos_rcv"], sc.get("orV_src"),
                     sc.get("orV_rcv"), _PAT[sc.get("spkr_pattern", "omni")], _PAT[sc.get("mic_pattern", "omni")],
                     sc["nb_img"], sc.get("Tdiff") or sc["Tmax"], sc["Tmax"], sc["fs"])
    return (time.perf_counter() - t0) * 1e3


def _time(fn, reps, warm=1):
    for _ in range(warm):
        fn()
    out = [fn() for _ in range(reps)]
    return out


def main():
    import torch
    import gpurir_gb300 as G
    from gpurir_gb300 import workloads as W
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    ap.add_argument("--skip-batched", action="store_true")
    args = ap.parse_args()
    rk = ref_kernels.RefKernels()
    res = {"gpu": torch.cuda.get_device_name(0)}

    single = {"plain_room": (W.plain_room(), 5), "mic_array": (W.mic_array(), 3)}
    traj = W.trajectory()
    single["trajectory_rirs"] = ({k: v for k, v in traj.items() if k != "signal"}, 2)
    for name, (sc, reps) in single.items():
        modes = ("fp32", "mp", "lut") if name == "mic_array" else ("fp32",)
        entry = {}
        for mode in modes:
            t = _time(lambda: _ref_call(rk, torch, sc, mode), reps)
            entry["reference_" + mode] = {"device_ms": float(np.median([a for a, _ in t])),
                                          "call_ms": float(np.median([b for _, b in t]))}
            sim = G.Simulator(seed=1, mixed_precision=(mode == "mp"), lut=(mode == "lut"))
            te = _time(lambda: _engine_call(sim, sc), max(reps, 5), warm=2)
            entry["engine_" + mode] = {"call_ms": float(np.median(te))}
            entry["speedup_call_" + mode] = entry["reference_" + mode]["call_ms"] / entry["engine_" + mode]["call_ms"]
            print(name, mode, json.dumps(entry), flush=True)
        res[name] = entry

    for name, rooms, reps in (("inverse_problem", W.inverse_problem(), 2),
                              ("batched_rooms", None if args.skip_batched else W.batched_rooms(), 1)):
        if rooms is None:
            continue
        sim = G.Simulator(seed=1)
        rl = []
        for _ in range(reps):
            dev = wall = 0.0
            for sc in rooms:
                a, b = _ref_call(rk, torch, sc, "fp32")
                dev += a
                wall += b
            rl.append((dev, wall))
        el = []
        for _ in range(reps + 1):
            t0 = time.perf_counter()
            for sc in rooms:
                _engine_call(sim, sc)
            el.append((time.perf_counter() - t0) * 1e3)
        entry = {"rooms": len(rooms), "reference_loop_device_ms": float(np.median([a for a, _ in rl])),
                 "reference_loop_call_ms": float(np.median([b for _, b in rl])),
                 "engine_loop_call_ms": float(np.median(el[1:])),
                 "note": "one simulateRIR call per room (the reference has no batched call)"}
        entry["speedup_loop"] = entry["reference_loop_call_ms"] / entry["engine_loop_call_ms"]
        print(name, json.dumps(entry), flush=True)
        res[name] = entry
    rk.close()
    txt = json.dumps(res, indent=1)
    print(txt)
    if args.out:
        with open(args.out, "w") as f:
            f.write(txt)


if __name__ == "__main__":
    main()
