"""Autotuner of the launch shapes (tuning knobs of the C ABI, gpurir_set_tuning).

gpuRIR fixes its launch shapes as compile-time constants
(src/gpuRIR_cuda.cu:20-45).  Here the shapes that do not change any result bit
-- rows per block of the convolution, resident blocks per SM of the forward and
adjoint image-source kernels and of the trajectory adjoint -- are measured on
the current GPU with the benchmark workloads' shapes, and the fastest are stored
in a JSON cache keyed by the GPU's name (and the library version):

    $GPURIR_TUNE_CACHE, default ~/.cache/gpurir_gb300/tuning.json

The package applies a cached entry when it creates its first simulator
(``apply_cached``; GPURIR_TUNE=0 turns that off).  ``tune()`` measures and writes
the entry; every candidate's output is checked to be bitwise equal to the
default's before its time counts.

    python -m gpurir_gb300.tune          # measure on this GPU, write the cache
"""
import ctypes
import json
import os
import time

import numpy as np

from . import _lib

KNOBS = {
    "conv_rows": (1, 2),
    "ism_blocks_per_sm": (0, 1),
    "adjoint_blocks_per_sm": (0, 1, 2),
    "traj_adjoint_blocks_per_sm": (0, 1, 2),
}
CACHE_VERSION = 1
_applied = False


def cache_path():
    return os.environ.get("GPURIR_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "gpurir_gb300",
                                                               "tuning.json")


def device_name():
    buf = ctypes.create_string_buffer(256)
    _lib.check(_lib.load().gpurir_device_name(buf, 256), "gpurir_device_name")
    return buf.value.decode()


def library_version():
    return _lib.load().gpurir_version().decode()


def set_knobs(knobs):
    L = _lib.load()
    for k, v in knobs.items():
        _lib.check(L.gpurir_set_tuning(k.encode(), int(v)), "gpurir_set_tuning(%s)" % k)


def get_knobs():
    L = _lib.load()
    out = {}
    for k in KNOBS:
        v = ctypes.c_int()
        _lib.check(L.gpurir_get_tuning(k.encode(), ctypes.byref(v)), "gpurir_get_tuning")
        out[k] = v.value
    return out


def reset():
    _lib.check(_lib.load().gpurir_reset_tuning(), "gpurir_reset_tuning")


def load_cache(path=None):
    try:
        with open(path or cache_path()) as f:
            c = json.load(f)
        return c if c.get("version") == CACHE_VERSION else {"version": CACHE_VERSION, "devices": {}}
    except (OSError, ValueError):
        return {"version": CACHE_VERSION, "devices": {}}


def save_entry(name, entry, path=None):
    path = path or cache_path()
    c = load_cache(path)
    c.setdefault("devices", {})[name] = entry
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = "%s.tmp%d" % (path, os.getpid())
    with open(tmp, "w") as f:
        json.dump(c, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply_cached(name=None, path=None):
    """Set the knobs of the cache entry for this GPU (and this library version).
    Returns the knobs applied, or None when there is no matching entry."""
    name = name or device_name()
    e = load_cache(path).get("devices", {}).get(name)
    if not e or e.get("library") != library_version():
        return None
    knobs = {k: v for k, v in e.get("knobs", {}).items() if k in KNOBS and v in KNOBS[k]}
    set_knobs(knobs)
    return knobs


def apply_cached_once():
    """apply_cached() the first time the package needs the GPU (GPURIR_TUNE=0: never)."""
    global _applied
    if _applied:
        return
    _applied = True
    if os.environ.get("GPURIR_TUNE", "1") == "0":
        return
    try:
        apply_cached()
    except Exception:   # no device yet, unreadable cache: keep the defaults
        pass


# --------------------------------------------------------------------------- measurement
def _timer(fn, reps, flush):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ts = []
    for _ in range(reps):
        flush.zero_()
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    ts.sort()
    return ts[len(ts) // 2]


def _case_conv(sim, dev):
    import torch
    g = torch.Generator(device=dev).manual_seed(4)
    rir = torch.randn((400, 8, 12800), device=dev, generator=g) * 0.01
    seg = torch.randn((400, 400), device=dev, generator=g)
    out = torch.empty((400, 8, 13199), device=dev)
    L = _lib.load()

    def run():
        _lib.check(L.gpurir_convolutions_device(sim.handle, seg.data_ptr(), 400, 400, rir.data_ptr(), 8, 12800,
                                                out.data_ptr(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                   "gpurir_convolutions_device")
        return out
    return run


def _case_ism(sim, dev):
    import torch
    from . import polar_patterns, workloads
    sc = workloads.mic_array()
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)
    ps, pr, orv = d(sc["pos_src"]), d(sc["pos_rcv"]), d(sc["orV_rcv"])
    out = torch.empty((64, 32, 16000), device=dev)

    def run():
        sim.simulate_rir_device(sc["room_sz"], sc["beta"], ps, pr, None, orv, 0, polar_patterns["card"],
                                sc["nb_img"], sc["Tdiff"], sc["Tmax"], sc["fs"], sc["c"], out)
        return out[..., :4800]   # the ISM part (the tail's noise advances per call)
    return run


def _case_adjoint(sim, dev):
    import torch
    from .autograd import TorchBatch
    from . import workloads
    rooms = workloads.inverse_problem()
    state = {}

    def run():
        knob = get_knobs()["adjoint_blocks_per_sm"]
        if state.get("knob") != knob:   # the adjoint handle fixes its grid at creation
            state["knob"] = knob
            state["model"] = TorchBatch(rooms, 16000.0, sim=sim)
            t = lambda a, g: torch.tensor(a, device=dev, requires_grad=g)
            state["args"] = (t(np.stack([r["beta"] for r in rooms]), True),
                             t(np.concatenate([r["pos_src"] for r in rooms]), True),
                             t(np.concatenate([r["pos_rcv"] for r in rooms]), True), None,
                             t(np.concatenate([r["orV_rcv"] for r in rooms]), False))
            m = state["model"]
            state["target"] = m(state["args"][0].detach() * 0.99, *[a.detach() if a is not None else None
                                                                   for a in state["args"][1:]]).detach()
        m, a = state["model"], state["args"]
        m.l2_step(*a, target=state["target"])
        return torch.cat([a[0].grad.ravel(), a[1].grad.ravel(), a[2].grad.ravel()])
    return run


def _case_traj_adjoint(sim, dev):
    import torch
    g = torch.Generator(device=dev).manual_seed(5)
    rir = torch.randn((400, 8, 12800), device=dev, generator=g) * 0.01
    seg = torch.randn((400, 400), device=dev, generator=g)
    gout = torch.randn((160000 + 12799, 8), device=dev, dtype=torch.float64, generator=g)
    gs = torch.empty(160000, device=dev)
    gr = torch.empty_like(rir)
    w = np.ascontiguousarray((np.arange(401) * 400).astype(np.int32))
    L = _lib.load()

    def run():
        _lib.check(L.gpurir_trajectory_adjoint_device(
            sim.handle, seg.data_ptr(), 400, 400, w.ctypes.data_as(_lib.iptr), rir.data_ptr(), 8, 12800,
            gout.data_ptr(), gs.data_ptr(), gr.data_ptr(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
            "gpurir_trajectory_adjoint_device")
        return torch.cat([gs, gr.ravel()])
    return run


CASES = {"conv_rows": _case_conv, "ism_blocks_per_sm": _case_ism, "adjoint_blocks_per_sm": _case_adjoint,
         "traj_adjoint_blocks_per_sm": _case_traj_adjoint}


def tune(reps=10, warmup=3, path=None, write=True, knobs=None):
    """Measure every candidate of every knob (the others at their defaults) and keep
    the fastest; returns the cache entry (and writes it unless write=False)."""
    import torch
    from . import Simulator
    dev = torch.device("cuda", torch.cuda.current_device())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    reset()
    sim = Simulator(seed=11)
    best, timings = {}, {}
    t0 = time.time()
    for knob in (knobs or KNOBS):
        run = CASES[knob](sim, dev)
        ref, times = None, {}
        for v in KNOBS[knob]:
            set_knobs({knob: v})
            for _ in range(warmup):
                out = run()
            torch.cuda.synchronize()
            out = run().clone()
            torch.cuda.synchronize()
            if ref is None:
                ref = out
            elif not torch.equal(out, ref):
                raise RuntimeError("tuning knob %s=%d changed the results" % (knob, v))
            times[v] = _timer(run, reps, flush)
        reset()
        best[knob] = min(times, key=times.get)
        timings[knob] = {str(v): t for v, t in times.items()}
    reset()
    set_knobs(best)
    entry = {"knobs": best, "timings_ms": timings, "library": library_version(),
             "tuned_s": round(time.time() - t0, 2)}
    if write:
        save_entry(device_name(), entry, path)
    return entry


if __name__ == "__main__":
    print(json.dumps(tune(), indent=1))
