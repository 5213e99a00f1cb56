"""Golden vectors from gpuRIR's own CUDA kernels (reference_kernels.npz).

Runs the reference's kernels, compiled from its sources into
oracle/_ref/gpuRIR_ref.cubin (oracle.ref_kernels.build_ref), on a GB300 through
oracle.ref_kernels.RefKernels, on small seeded scenes, and stores the inputs
with every stage's output: image amplitudes and delays (calcAmpTau_kernel),
the early part in the three modes (FP32, mixed precision, lookup table), the
envelope (envPred_kernel) and the diffuse tail of deterministic uniforms
(diffRev_kernel).

    python tests/golden/make_reference_kernels.py --out tests/golden/reference_kernels.npz

Needs a GPU and the cubin; the committed .npz is what the tests read.
"""
import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_kernels  # noqa: E402


def _inside(rng, n, room, margin):
    room = np.asarray(room, dtype=np.float64)
    return (margin + rng.random((n, 3)) * (room - 2 * margin)).astype(np.float32)


def _unit(rng, n):
    v = rng.standard_normal((n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def scenes():
    """Seeded scenes: name -> (kwargs of RefKernels.simulate, modes)."""
    out = {}
    rng = np.random.default_rng(0)
    room = [3.0, 4.0, 2.5]
    # the 2-RIR room of the simplest example, full ISM over 0.5 s
    out["plain"] = (dict(room_sz=room, beta=[0.85] * 6, pos_src=_inside(rng, 1, room, 0.5),
                         pos_rcv=_inside(rng, 2, room, 0.5), nb_img=[11, 9, 13], Tmax=0.5,
                         Tdiff=0.5, fs=16000.0), ("fp32", "mp", "lut"))
    rng = np.random.default_rng(21)
    room = [4.0, 5.0, 3.0]
    for sp in range(6):
        mp = (sp + 2) % 6
        out["pattern_%d_%d" % (sp, mp)] = (
            dict(room_sz=room, beta=rng.uniform(0.6, 0.95, 6).astype(np.float32),
                 pos_src=_inside(rng, 2, room, 0.5), pos_rcv=_inside(rng, 3, room, 0.5),
                 orV_src=_unit(rng, 2), orV_rcv=_unit(rng, 3), spkr_pattern=sp, mic_pattern=mp,
                 nb_img=[5, 5, 5], Tmax=0.05, Tdiff=0.05, fs=16000.0), ("fp32",))
    rng = np.random.default_rng(22)
    room = [6.0, 5.0, 3.0]
    # early part + envelope + diffuse tail (2 sources x 4 receivers)
    out["tail"] = (dict(room_sz=room, beta=[0.93, 0.94, 0.92, 0.95, 0.9, 0.91],
                        pos_src=_inside(rng, 2, room, 0.5), pos_rcv=_inside(rng, 4, room, 0.5),
                        nb_img=[12, 14, 24], Tmax=0.2, Tdiff=0.1, fs=16000.0), ("fp32",))
    rng = np.random.default_rng(23)
    room = [5.0, 4.0, 3.0]
    # 48 kHz: 384-sample window; 44.1 kHz: odd 353-sample window (half-integer half width)
    out["fs48k"] = (dict(room_sz=room, beta=[0.8] * 6, pos_src=_inside(rng, 1, room, 0.5),
                         pos_rcv=_inside(rng, 2, room, 0.5), nb_img=[7, 7, 7], Tmax=0.05,
                         Tdiff=0.05, fs=48000.0), ("fp32", "lut"))
    out["fs44k1"] = (dict(room_sz=room, beta=[0.8] * 6, pos_src=_inside(rng, 1, room, 0.5),
                          pos_rcv=_inside(rng, 2, room, 0.5), nb_img=[7, 7, 7], Tmax=0.04,
                          Tdiff=0.04, fs=44100.0), ("fp32", "lut"))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                  "reference_kernels.npz"))
    args = ap.parse_args()
    rk = ref_kernels.RefKernels()
    arrays, meta = {}, {}
    for name, (kw, modes) in scenes().items():
        for key in ("room_sz", "beta", "pos_src", "pos_rcv", "orV_src", "orV_rcv"):
            if kw.get(key) is not None:
                arrays["%s/in/%s" % (name, key)] = np.asarray(kw[key], dtype=np.float32)
        meta[name] = {k: (list(map(int, v)) if k == "nb_img" else v) for k, v in kw.items()
                      if k in ("nb_img", "Tmax", "Tdiff", "fs", "spkr_pattern", "mic_pattern")}
        meta[name]["modes"] = list(modes)
        for mode in modes:
            n_diff = ref_kernels._n_samples(kw["Tmax"], kw["fs"]) - ref_kernels._n_samples(kw["Tdiff"], kw["fs"])
            ms, mr = len(kw["pos_src"]), len(kw["pos_rcv"])
            u = ref_kernels.hash_uniforms(ms * mr * n_diff) if (mode == "fp32" and n_diff > 0) else None
            r = rk.simulate(mode=mode, uniforms=u, **kw)
            arrays["%s/%s/early" % (name, mode)] = r["early"]
            if mode == "fp32":
                for key in ("amp", "tau", "tau_dp", "A", "alpha"):
                    arrays["%s/%s" % (name, key)] = r[key]
                if "diffuse" in r:
                    arrays["%s/diffuse" % name] = r["diffuse"]
            print(name, mode, r["early"].shape, float(np.abs(r["early"]).max()))
    arrays["meta_json"] = np.frombuffer(json.dumps(meta, sort_keys=True).encode(), dtype=np.uint8)
    np.savez_compressed(args.out, **arrays)
    print("wrote", args.out, os.path.getsize(args.out), "bytes")


if __name__ == "__main__":
    main()
