"""Generate golden vectors from the reference's own Python package.

Run in the build container, where the reference checkout exists:

    python tests/golden/make_golden.py <path of the gpuRIR checkout>

gpuRIR/__init__.py imports a compiled module ``gpuRIR_bind`` whose constructor
needs a GPU; a stub module stands in for it here.  The stub only records the
arguments the reference passes to the binding and, for ``gpu_conv``, returns an
FP64 direct convolution, so the goldens capture the reference's own host-side
Python: the Sabine/T60 helpers, the argument marshalling of ``simulateRIR``
and the segmentation + FP64 overlap-add of ``simulateTrajectory``.

Output: tests/golden/reference_python.npz (small; committed).
"""
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class _StubBind:
    """Records what gpuRIR/__init__.py hands to the compiled binding."""

    def __init__(self, mixed_precision=False):
        self.calls = []

    def simulateRIR_bind(self, room_sz, beta, pos_src, pos_rcv, orV_src, orV_rcv, spkr_pattern,
                         mic_pattern, nb_img, Tdiff, Tmax, fs, c):
        self.calls.append(dict(room_sz=room_sz, beta=beta, pos_src=pos_src, pos_rcv=pos_rcv,
                               orV_src=orV_src, orV_rcv=orV_rcv, spkr_pattern=spkr_pattern,
                               mic_pattern=mic_pattern, nb_img=nb_img, Tdiff=Tdiff, Tmax=Tmax,
                               fs=fs, c=c))
        return np.zeros((len(pos_src), len(pos_rcv), 2), dtype=np.float32)

    def gpu_conv(self, segments, RIRs):
        P, S = segments.shape
        _, R, L = RIRs.shape
        out = np.zeros((P, R, S + L - 1))
        for p in range(P):
            for r in range(R):
                out[p, r] = np.convolve(segments[p].astype(np.float64),
                                        RIRs[p, r].astype(np.float64))
        self.calls.append(dict(segments=segments.copy()))
        return out

    def activate_mixed_precision_bind(self, a):
        return a

    def activate_lut_bind(self, a):
        return a


def load_reference(ref_root):
    mod = types.ModuleType("gpuRIR_bind")
    mod.gpuRIR_bind = _StubBind
    sys.modules["gpuRIR_bind"] = mod
    sys.path.insert(0, ref_root)
    import gpuRIR  # noqa: E402  (the reference package)
    return gpuRIR


def main(ref_root):
    g = load_reference(ref_root)
    rng = np.random.default_rng(20261203)
    out = {}
    meta = {}

    # --- beta_SabineEstimation (gpuRIR/__init__.py:22-54) -------------------
    cases = [([6.0, 5.0, 3.0], 1.0, [1.0] * 6), ([8.0, 6.0, 3.0], 0.8, [1.0] * 6),
             ([3.0, 4.0, 2.5], 0.7, [1.0] * 6), ([5.0, 4.0, 3.0], 0.3, [1.0] * 6),
             ([3.0, 4.0, 2.5], 0.05, [1.0] * 6),          # clamps to total absorption
             ([3.0, 4.0, 2.5], 30.0, [1.0] * 6),          # nearly rigid walls
             ([6.0, 5.0, 3.0], 1.0, [0.5, 1.0, 1.0, 2.0, 1.0, 0.25])]
    for _ in range(24):
        room = [float(rng.uniform(3, 10)), float(rng.uniform(3, 8)), float(rng.uniform(2.5, 4.5))]
        cases.append((room, float(rng.uniform(0.2, 1.2)), [1.0] * 6))
    rooms = np.array([c[0] for c in cases])
    t60s = np.array([c[1] for c in cases])
    wts = np.array([c[2] for c in cases])
    betas = np.array([g.beta_SabineEstimation(list(r), t, list(w)) for r, t, w in cases])
    out["sabine_room"], out["sabine_t60"], out["sabine_weights"] = rooms, t60s, wts
    out["sabine_beta"] = betas.astype(np.float32)

    # --- t2n, att2t_SabineEstimator (gpuRIR/__init__.py:56-93) ---------------
    t2n_T = np.array([0.3, 0.5, 0.25, 0.4, 1.0, 0.123])
    t2n_room = np.array([[6, 5, 3], [3, 4, 2.5], [8, 6, 3], [5, 4, 3], [10, 8, 4.5], [3, 3, 2.5]],
                        dtype=np.float64)
    out["t2n_T"], out["t2n_room"] = t2n_T, t2n_room
    out["t2n"] = np.array([g.t2n(T, r) for T, r in zip(t2n_T, t2n_room)], dtype=np.int64)
    out["t2n_c"] = np.array([g.t2n(0.3, [6, 5, 3], c=300.0)], dtype=np.int64)
    out["att2t"] = np.array([g.att2t_SabineEstimator(a, t) for a, t in
                             [(13.0, 0.7), (50.0, 0.7), (15.0, 0.6), (60.0, 1.2)]])

    # --- simulateRIR argument marshalling (gpuRIR/__init__.py:154-175) -------
    stub = g.gpuRIR_bind_simulator
    ps = rng.uniform(0.5, 2.5, (3, 3))
    pr = rng.uniform(0.5, 2.0, (2, 3))
    orv = rng.standard_normal((2, 3))
    g.simulateRIR([3.0, 4.0, 2.5], [0.85] * 6, ps, pr, [11, 9, 13], 0.5, 16000.0)
    g.simulateRIR([3.0, 4.0, 2.5], [0.85] * 6, ps, pr, [5, 5, 5], 0.5, 16000.0, Tdiff=0.2,
                  mic_pattern="card", orV_rcv=orv)
    g.simulateRIR(np.array([3.0, 4.0, 2.5]), np.full(6, 0.7), ps.astype(np.float32), pr,
                  [4, 6, 8], 0.3, 8000, spkr_pattern="hypcard", orV_src=ps, c=340.0)
    marsh = []
    for call in stub.calls:
        rec = {}
        for k, v in call.items():
            if isinstance(v, np.ndarray):
                rec[k] = dict(dtype=str(v.dtype), c_contig=bool(v.flags.c_contiguous),
                              value=v.tolist())
            else:
                rec[k] = v if not isinstance(v, np.ndarray) else v.tolist()
                if isinstance(v, (np.floating, np.integer)):
                    rec[k] = v.item()
                elif isinstance(v, np.ndarray):
                    rec[k] = v.tolist()
                elif isinstance(v, list):
                    rec[k] = [x.item() if hasattr(x, "item") else x for x in v]
        marsh.append(rec)
    meta["simulateRIR_calls"] = marsh
    meta["simulateRIR_inputs"] = dict(ps=ps.tolist(), pr=pr.tolist(), orv=orv.tolist())
    stub.calls.clear()

    # --- simulateTrajectory (gpuRIR/__init__.py:177-221) ---------------------
    sig = rng.standard_normal(3001).astype(np.float32)
    rirs = (rng.standard_normal((7, 3, 257)) * np.exp(-np.arange(257) / 60.0)).astype(np.float32)
    out["traj_signal"], out["traj_rirs"] = sig, rirs
    out["traj_default"] = g.simulateTrajectory(sig, rirs)
    out["traj_default_segments"] = stub.calls[-1]["segments"]
    ts = np.array([0.0, 0.01, 0.05, 0.06, 0.11, 0.15, 0.17])
    out["traj_custom_ts"] = ts
    out["traj_custom"] = g.simulateTrajectory(sig, rirs, timestamps=ts, fs=16000)
    out["traj_custom_segments"] = stub.calls[-1]["segments"]
    stub.calls.clear()

    # --- polar_patterns dict and the exported names ---------------------------
    meta["polar_patterns"] = dict(g.polar_patterns)
    meta["__all__"] = list(g.__all__)

    np.savez_compressed(os.path.join(HERE, "reference_python.npz"), **out)
    with open(os.path.join(HERE, "reference_python.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote", sorted(out), sorted(meta))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the gpuRIR checkout>")
    main(sys.argv[1])
