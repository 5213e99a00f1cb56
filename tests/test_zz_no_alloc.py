"""gpurir_simulate_ism_noalloc: the image-source entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc while they run -- a
real-time audio thread (an allocation can block on a device-wide
synchronisation), a host application that fixes the device-memory budget of
its plugins, work recorded under global stream capture.  Its scratch is a
fixed array inside the library shared by every call.  This file checks, through
the C ABI, that two calls in a row give the same RIRs as the allocating entry
point gpurir_simulate_rir_device (Tdiff = Tmax), within the early-part
tolerance of the other GPU tests (relative L2 <= 1e-5), and that a repeated
call is unaffected by what the previous call left in the shared scratch.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL_REL_L2 = 1e-5


def _scene(seed, ns, nr, room, nb, T, spkr, mic):
    rng = np.random.default_rng(seed)
    room = np.asarray(room, dtype=np.float32)
    ps = (0.4 + rng.random((ns, 3)) * (room - 0.8)).astype(np.float32)
    pr = (0.4 + rng.random((nr, 3)) * (room - 0.8)).astype(np.float32)
    os_ = rng.standard_normal((ns, 3)).astype(np.float32)
    or_ = rng.standard_normal((nr, 3)).astype(np.float32)
    beta = rng.uniform(0.7, 0.95, 6).astype(np.float32)
    return dict(room=room, beta=beta, ps=ps, pr=pr, os=os_, orv=or_, nb=np.array(nb, np.int32), T=T,
                spkr=spkr, mic=mic)


def _noalloc(L, lib, c, d, out, stream):
    lib.check(L.gpurir_simulate_ism_noalloc(
        c["room"].ctypes.data_as(lib.fptr), c["beta"].ctypes.data_as(lib.fptr), d["ps"].data_ptr(),
        c["ps"].shape[0], d["pr"].data_ptr(), d["os"].data_ptr(), d["or"].data_ptr(), c["spkr"],
        c["mic"], c["pr"].shape[0], c["nb"].ctypes.data_as(lib.iptr), c["T"], 16000.0, 343.0,
        out.data_ptr(), ctypes.c_void_p(stream)), "gpurir_simulate_ism_noalloc")


def test_noalloc_matches_allocating_entry_two_calls_in_a_row(built):
    import torch
    import gpurir_gb300 as G
    from gpurir_gb300 import _lib
    L = _lib.load()
    scenes = [_scene(1, 64, 32, [6.0, 5.0, 3.0], [12, 14, 24], 0.3, 0, 2),   # 2048 RIRs
              _scene(2, 3, 4, [4.0, 3.5, 2.8], [9, 9, 9], 0.12, 3, 5)]       # directional, long split
    dev = torch.device("cuda")
    bufs = []
    for c in scenes:
        d = {k: torch.from_numpy(c[v]).to(dev) for k, v in (("ps", "ps"), ("pr", "pr"), ("os", "os"),
                                                            ("or", "orv"))}
        n = G._lib.load().gpurir_n_samples(c["T"], 16000.0)
        bufs.append((d, torch.full((c["ps"].shape[0], c["pr"].shape[0], n), float("nan"), device=dev)))
    st = torch.cuda.current_stream().cuda_stream
    # two no-allocation calls back to back on one stream, sharing the scratch
    for c, (d, out) in zip(scenes, bufs):
        _noalloc(L, _lib, c, d, out, st)
    torch.cuda.synchronize()
    sim = G.Simulator()
    for c, (d, out) in zip(scenes, bufs):
        ref = torch.empty_like(out)
        sim.simulate_rir_device(c["room"], c["beta"], d["ps"], d["pr"], d["os"], d["or"], c["spkr"],
                                c["mic"], c["nb"], c["T"], c["T"], 16000.0, 343.0, ref)
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert np.all(np.isfinite(a))
        assert rel_l2(a, b) <= TOL_REL_L2
    # a repeat of the first scene after the second is unaffected by the scratch's contents
    d, out = bufs[0]
    again = torch.full_like(out, float("nan"))
    _noalloc(L, _lib, scenes[0], d, again, st)
    torch.cuda.synchronize()
    assert np.array_equal(again.cpu().numpy(), out.cpu().numpy())


def test_noalloc_rejects_sizes_beyond_the_scratch(built):
    import torch
    from gpurir_gb300 import _lib
    L = _lib.load()
    c = _scene(3, 128, 65, [6.0, 5.0, 3.0], [3, 3, 3], 0.05, 0, 0)   # 8320 RIRs > 8192
    dev = torch.device("cuda")
    d = {k: torch.from_numpy(c[v]).to(dev) for k, v in (("ps", "ps"), ("pr", "pr"), ("os", "os"),
                                                        ("or", "orv"))}
    out = torch.empty(1, device=dev)
    rc = L.gpurir_simulate_ism_noalloc(
        c["room"].ctypes.data_as(_lib.fptr), c["beta"].ctypes.data_as(_lib.fptr), d["ps"].data_ptr(),
        128, d["pr"].data_ptr(), None, None, 0, 0, 65, c["nb"].ctypes.data_as(_lib.iptr), c["T"],
        16000.0, 343.0, out.data_ptr(), None)
    assert rc == -1
    assert b"8192" in L.gpurir_last_error()


def test_noalloc_limit_counts_segments_of_long_rirs(built):
    """The 8192-item scratch holds RIRs x segments: at 16 kHz a 2 s RIR is cut
    into 7 segments of at most 5120 samples, so 1170 RIRs fit and 1600 do not
    (rejected on the host before anything is enqueued)."""
    import torch
    from gpurir_gb300 import _lib
    L = _lib.load()
    dev = torch.device("cuda")
    room = np.array([6.0, 5.0, 3.0], np.float32)
    beta = np.full(6, 0.8, np.float32)
    nb = np.array([3, 3, 3], np.int32)
    n = L.gpurir_n_samples(2.0, 16000.0)
    for ns, nr, ok in ((39, 30, True), (40, 40, False)):
        rng = np.random.default_rng(ns)
        ps = torch.from_numpy((0.5 + rng.random((ns, 3)) * (room - 1.0)).astype(np.float32)).to(dev)
        pr = torch.from_numpy((0.5 + rng.random((nr, 3)) * (room - 1.0)).astype(np.float32)).to(dev)
        out = torch.full((ns, nr, n) if ok else (1,), float("nan"), device=dev)
        rc = L.gpurir_simulate_ism_noalloc(
            room.ctypes.data_as(_lib.fptr), beta.ctypes.data_as(_lib.fptr), ps.data_ptr(), ns, pr.data_ptr(),
            None, None, 0, 0, nr, nb.ctypes.data_as(_lib.iptr), 2.0, 16000.0, 343.0, out.data_ptr(),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        if ok:
            assert rc == 0, L.gpurir_last_error()
            assert bool(torch.isfinite(out).all())
        else:
            assert rc == -1
            assert b"segments" in L.gpurir_last_error()
