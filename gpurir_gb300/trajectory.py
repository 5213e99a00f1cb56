"""Moving-source filtering: simulateTrajectory (gpuRIR/__init__.py:177-221).

The signal is cut into one segment per trajectory point, each segment is
convolved with the RIRs of its point, and the convolutions are overlap-added.
gpuRIR does the convolutions with cuFFT (src/gpuRIR_cuda.cu:933-1023) and the
overlap-add as a Python double loop in float64; here both run on the GPU in
hand-written FFT kernels behind the C ABI (gpurir_trajectory_*).
"""
import numpy as np


def segment_bounds(n, n_pts, timestamps=None, fs=None):
    """First sample of every segment and the signal length, w_ini int [n_pts + 1], as
    gpuRIR/__init__.py:198-205 forms them."""
    assert timestamps is None or fs is not None, "fs must be indicated for custom timestamps"
    assert timestamps is None or timestamps[0] == 0, "The first timestamp must be 0"
    if timestamps is None:
        fs = n / n_pts
        timestamps = np.arange(n_pts)
    return np.append((np.asarray(timestamps) * fs).astype(int), n)


def segment_signal(source_signal, n_pts, timestamps=None, fs=None):
    """Segmentation of gpuRIR/__init__.py:198-213.

    Returns (segments float32 [n_pts, max_len], w_ini int [n_pts + 1], w_len int [n_pts]).
    """
    n = len(source_signal)
    w_ini = segment_bounds(n, n_pts, timestamps, fs)
    w_len = np.diff(w_ini)
    width = int(w_len.max())
    sig = np.asarray(source_signal)
    if np.all(w_len == width) and np.array_equal(w_ini[:-1], width * np.arange(n_pts)):
        # back to back: a view of a float32 signal, no copy
        segments = sig[:n_pts * width].reshape(n_pts, width).astype(np.float32, copy=False)
    else:
        segments = np.zeros((n_pts, width), dtype=np.float32)
        for p in range(n_pts):
            segments[p, 0:w_len[p]] = sig[w_ini[p]:w_ini[p + 1]]
    return np.ascontiguousarray(segments), w_ini, w_len


def gpu_conv(source_segments, RIRs, sim=None):
    """Batched convolutions of gpuRIR_bind.gpu_conv (src/python_bind.cpp:90-119):
    float32 [P, S] x float32 [P, R, L] -> float32 [P, R, S + L - 1]."""
    from . import _lib, simulator
    sim = sim or simulator()
    seg = np.ascontiguousarray(np.asarray(source_segments, dtype=np.float32))
    rir = np.ascontiguousarray(np.asarray(RIRs, dtype=np.float32))
    if seg.ndim != 2 or rir.ndim != 3 or seg.shape[0] != rir.shape[0]:
        raise ValueError("source_segments [P, S] and RIRs [P, R, L] with the same P")
    P, S = seg.shape
    _, R, L = rir.shape
    out = np.empty((P, R, S + L - 1), dtype=np.float32)
    _lib.check(_lib.load().gpurir_convolutions(sim.handle, seg.ctypes.data, P, S, rir.ctypes.data, R, L,
                                               out.ctypes.data), "gpurir_convolutions")
    return out


def simulate_trajectory(source_signal, RIRs, timestamps=None, fs=None, sim=None):
    """simulateTrajectory: float64 [len(signal) + L - 1, R] (numpy), or a float64
    CUDA tensor when RIRs is a CUDA tensor (then everything stays on the device)."""
    from . import _lib, simulator
    sim = sim or simulator()
    n_pts = RIRs.shape[0]
    seg, w_ini, w_len = segment_signal(source_signal, n_pts, timestamps, fs)
    w = np.ascontiguousarray(w_ini.astype(np.int32))
    L = _lib.load()
    if hasattr(RIRs, "is_cuda") and RIRs.is_cuda:
        import torch
        rir = RIRs.to(torch.float32).contiguous()
        dseg = torch.from_numpy(seg).to(rir.device)
        _, R, Lr = rir.shape
        out = torch.empty((int(w[-1]) + Lr - 1, R), dtype=torch.float64, device=rir.device)
        st = torch.cuda.current_stream(rir.device).cuda_stream
        import ctypes
        _lib.check(L.gpurir_trajectory_device(sim.handle, dseg.data_ptr(), n_pts, seg.shape[1],
                                              w.ctypes.data_as(_lib.iptr), rir.data_ptr(), R, Lr,
                                              out.data_ptr(), ctypes.c_void_p(st)),
                   "gpurir_trajectory_device")
        return out
    rir = np.ascontiguousarray(np.asarray(RIRs, dtype=np.float32))
    _, R, Lr = rir.shape
    out = np.empty((int(w[-1]) + Lr - 1, R), dtype=np.float64)
    _lib.check(L.gpurir_trajectory(sim.handle, seg.ctypes.data, n_pts, seg.shape[1],
                                   w.ctypes.data_as(_lib.iptr), rir.ctypes.data, R, Lr,
                                   out.ctypes.data), "gpurir_trajectory")
    return out


class _Trajectory:
    """torch.autograd.Function of simulateTrajectory on device tensors (built lazily:
    importing this module does not import torch)."""
    fn = None

    @classmethod
    def get(cls):
        if cls.fn is None:
            import torch

            class Fn(torch.autograd.Function):
                @staticmethod
                def forward(ctx, signal, rirs, w_ini, seg_len, sim):
                    from . import _lib
                    import ctypes
                    dseg = _segments_device(signal, w_ini, seg_len)
                    P, R, Lr = rirs.shape
                    out = torch.empty((int(w_ini[-1]) + Lr - 1, R), dtype=torch.float64, device=rirs.device)
                    st = torch.cuda.current_stream(rirs.device).cuda_stream
                    _lib.check(_lib.load().gpurir_trajectory_device(
                        sim.handle, dseg.data_ptr(), P, seg_len, w_ini.ctypes.data_as(_lib.iptr), rirs.data_ptr(),
                        R, Lr, out.data_ptr(), ctypes.c_void_p(st)), "gpurir_trajectory_device")
                    ctx.save_for_backward(dseg, rirs)
                    ctx.w_ini, ctx.seg_len, ctx.sim, ctx.n_sig = w_ini, seg_len, sim, signal.shape[0]
                    return out

                @staticmethod
                def backward(ctx, grad_out):
                    from . import _lib
                    import ctypes
                    dseg, rirs = ctx.saved_tensors
                    P, R, Lr = rirs.shape
                    g = grad_out.to(torch.float64).contiguous()
                    gs = torch.zeros(ctx.n_sig, dtype=torch.float32, device=rirs.device) \
                        if ctx.needs_input_grad[0] else None
                    gr = torch.empty_like(rirs) if ctx.needs_input_grad[1] else None
                    st = torch.cuda.current_stream(rirs.device).cuda_stream
                    _lib.check(_lib.load().gpurir_trajectory_adjoint_device(
                        ctx.sim.handle, dseg.data_ptr(), P, ctx.seg_len, ctx.w_ini.ctypes.data_as(_lib.iptr),
                        rirs.data_ptr(), R, Lr, g.data_ptr(), gs.data_ptr() if gs is not None else None,
                        gr.data_ptr() if gr is not None else None, ctypes.c_void_p(st)),
                        "gpurir_trajectory_adjoint_device")
                    return gs, gr, None, None, None

            cls.fn = Fn
        return cls.fn


def _segments_device(signal, w_ini, seg_len):
    """Segments [n_pts, seg_len] of a device signal (zero-padded), as segment_signal cuts them."""
    import torch
    n_pts = len(w_ini) - 1
    w_len = np.diff(w_ini)
    if np.all(w_len == seg_len) and np.array_equal(w_ini[:-1], seg_len * np.arange(n_pts)):
        return signal[:n_pts * seg_len].reshape(n_pts, seg_len).contiguous()
    # one gather: destination (p, t) <- signal[w_ini[p] + t] for t < w_len[p]
    t = np.arange(seg_len)
    keep = t[None, :] < w_len[:, None]
    dst = np.nonzero(keep.ravel())[0]
    src = (w_ini[:-1, None] + t[None, :]).ravel()[dst]
    seg = torch.zeros(n_pts * seg_len, dtype=torch.float32, device=signal.device)
    seg[torch.from_numpy(dst).to(signal.device)] = signal[torch.from_numpy(src).to(signal.device)]
    return seg.view(n_pts, seg_len)


def simulate_trajectory_torch(source_signal, RIRs, timestamps=None, fs=None, sim=None):
    """simulateTrajectory on float32 CUDA tensors with autograd: returns the float64
    [len(signal) + L - 1, R] tensor; its backward gives dL/dsignal and dL/dRIRs
    (FFT correlations on the device, gpurir_trajectory_adjoint_device).  Chain RIRs
    from gpurir_gb300.autograd to reach the wall coefficients and positions."""
    import torch
    from . import simulator
    sim = sim or simulator()
    if not (source_signal.is_cuda and RIRs.is_cuda):
        raise ValueError("source_signal and RIRs must be CUDA tensors")
    sig = source_signal.to(torch.float32).contiguous()
    rirs = RIRs.to(torch.float32).contiguous()
    n_pts = rirs.shape[0]
    n = sig.shape[0]
    assert timestamps is None or fs is not None, "fs must be indicated for custom timestamps"
    if timestamps is None:
        w_ini = np.append((np.arange(n_pts) * (n / n_pts)).astype(int), n)
    else:
        assert timestamps[0] == 0, "The first timestamp must be 0"
        w_ini = np.append((np.asarray(timestamps) * fs).astype(int), n)
    w_ini = np.ascontiguousarray(w_ini.astype(np.int32))
    seg_len = int(np.diff(w_ini).max())
    return _Trajectory.get().apply(sig, rirs, w_ini, seg_len, sim)
