"""gpurir_gb300 -- room impulse responses by the image-source method on one GB300.

Drop-in for the Python API of gpuRIR (gpuRIR/__init__.py): the same function
names, argument order, defaults, shapes and dtypes.  ``import gpurir_gb300 as
gpuRIR`` runs existing gpuRIR scripts.  The compute path is the CUDA library
libgpurir_gb300.so (hand-written sm_103a kernels behind a C ABI, see
include/gpurir_gb300.h); there is no CPU fallback.

Differences from gpuRIR, all deliberate:
  * FP32 exact evaluation is the default mode (gpuRIR defaults to its lookup
    table, src/python_bind.cpp:15); activateLUT()/activateMixedPrecision()
    select the other modes and exclude each other as in gpuRIR.
  * Errors raise Python exceptions instead of terminating the process.
  * The diffuse-tail noise comes from a Philox stream keyed by ``seed()``
    instead of cuRAND's stateful generator; it is reproducible.
  * ``__all__`` lists the functions that exist (gpuRIR's names two that do not,
    gpuRIR/__init__.py:11).
"""
import ctypes

import numpy as np

from . import _hostmem, _lib
from ._lib import GpuRirError

__all__ = ["polar_patterns", "beta_SabineEstimation", "att2t_SabineEstimator", "t2n",
           "simulateRIR", "simulateTrajectory", "activateMixedPrecision", "activateLUT",
           "activateReferenceDelays", "seed", "set_noise", "GpuRirError"]

# gpuRIR/__init__.py:13-20 (numbering of src/gpuRIR_cuda.h:2-8)
polar_patterns = {
    "omni": 0,
    "homni": 1,
    "card": 2,
    "hypcard": 3,
    "subcard": 4,
    "bidir": 5,
}


# ---------------------------------------------------------------------------
# Host helpers (FP64), gpuRIR/__init__.py:22-93
# ---------------------------------------------------------------------------
def beta_SabineEstimation(room_sz, T60, abs_weights=[1.0] * 6):
    """Reflection coefficients of the six walls for a wanted reverberation time.

    Same estimator as gpuRIR/__init__.py:22-54: minimise |T60 - 0.161 V / Sa|
    over the absorption scale x in [0, 1] with L-BFGS-B started at 0.5, then
    beta = sqrt(1 - x * weights).  The optimiser is run exactly as gpuRIR runs
    it, so results match gpuRIR bit for bit (including where L-BFGS-B stops
    short of the optimum); ``beta_sabine_closed_form`` gives the exact optimum.
    Unlike gpuRIR, a caller's ``abs_weights`` array is not modified in place.
    """
    from scipy.optimize import minimize

    w = np.asarray(abs_weights, dtype=np.float64)
    w = w / w.max()
    room = room_sz

    def t60error(x, T60, room_sz, abs_weights):
        alpha = x * abs_weights
        Sa = (alpha[0] + alpha[1]) * room_sz[1] * room_sz[2] + \
             (alpha[2] + alpha[3]) * room_sz[0] * room_sz[2] + \
             (alpha[4] + alpha[5]) * room_sz[0] * room_sz[1]
        V = np.prod(room_sz)
        if Sa == 0:
            return T60 - 0
        return abs(T60 - 0.161 * V / Sa)

    res = minimize(t60error, 0.5, args=(T60, room, w), bounds=[[0, 1]])
    return np.sqrt(1 - res.x * w).astype(np.float32)


def beta_sabine_closed_form(room_sz, T60, abs_weights=None):
    """Exact minimiser of the Sabine fit, vectorised over rooms.

    room_sz [..., 3], T60 [...], abs_weights [..., 6] (default all ones).
    x = 0.161 V / (T60 * sum_w area_w), clipped to [0, 1];
    beta = sqrt(1 - x * w) as float32 [..., 6].
    """
    L = np.asarray(room_sz, dtype=np.float64)
    T = np.asarray(T60, dtype=np.float64)
    w = np.ones(L.shape[:-1] + (6,)) if abs_weights is None else \
        np.broadcast_to(np.asarray(abs_weights, dtype=np.float64), L.shape[:-1] + (6,))
    w = w / w.max(axis=-1, keepdims=True)
    Lx, Ly, Lz = L[..., 0], L[..., 1], L[..., 2]
    Sw = (w[..., 0] + w[..., 1]) * Ly * Lz + (w[..., 2] + w[..., 3]) * Lx * Lz + \
         (w[..., 4] + w[..., 5]) * Lx * Ly
    x = np.clip(0.161 * Lx * Ly * Lz / (T * Sw), 0.0, 1.0)
    return np.sqrt(1 - x[..., None] * w).astype(np.float32)


def att2t_SabineEstimator(att_dB, T60):
    """Time for the RIR to decay by att_dB under the Sabine model (gpuRIR/__init__.py:56-72)."""
    return att_dB / 60.0 * T60


def t2n(T, rooms_sz, c=343.0):
    """Images per axis needed to cover T seconds (gpuRIR/__init__.py:74-93)."""
    nb_img = 2 * T / (np.array(rooms_sz) / c)
    return [int(n) for n in np.ceil(nb_img)]


# ---------------------------------------------------------------------------
# Simulator handle (module singleton, like gpuRIR_bind_simulator)
# ---------------------------------------------------------------------------
class Simulator:
    """Owns one gpurir_sim handle of the C ABI (one CUDA stream + workspace)."""

    def __init__(self, mixed_precision=False, lut=False, seed=1234, reference_delays=False):
        self._L = _lib.load()
        from . import tune
        tune.apply_cached_once()   # launch shapes measured on this GPU, if cached
        h = ctypes.c_void_p()
        _lib.check(self._L.gpurir_create(int(mixed_precision), int(lut), int(seed),
                                         ctypes.byref(h)), "gpurir_create")
        self._h = h
        if reference_delays:
            self.activate_reference_delays(True)

    def __del__(self):
        L = getattr(self, "_L", None)
        h = getattr(self, "_h", None)
        if L is not None and h:
            L.gpurir_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def activate_mixed_precision(self, activate):
        st = ctypes.c_int()
        _lib.check(self._L.gpurir_activate_mixed_precision(self._h, int(bool(activate)),
                                                           ctypes.byref(st)), "activate_mp")
        return bool(st.value)

    def activate_lut(self, activate):
        st = ctypes.c_int()
        _lib.check(self._L.gpurir_activate_lut(self._h, int(bool(activate)), ctypes.byref(st)),
                   "activate_lut")
        return bool(st.value)

    def activate_reference_delays(self, activate):
        """Round image delays in float32 as gpuRIR's calcAmpTau_kernel does
        (src/gpuRIR_cuda.cu:336-369) instead of computing them exactly."""
        st = ctypes.c_int()
        _lib.check(self._L.gpurir_set_reference_delays(self._h, int(bool(activate)), ctypes.byref(st)),
                   "reference_delays")
        return bool(st.value)

    def set_compensation(self, policy):
        """Compensated accumulation: 0 never, 1 long RIRs in lookup-table mode (default),
        2 always in mixed-precision and lookup-table modes (gpurir_set_compensation)."""
        _lib.check(self._L.gpurir_set_compensation(self._h, int(policy)), "set_compensation")

    def modes(self):
        mp, lut, rd = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(self._L.gpurir_get_modes(self._h, ctypes.byref(mp), ctypes.byref(lut)), "modes")
        _lib.check(self._L.gpurir_get_reference_delays(self._h, ctypes.byref(rd)), "modes")
        return dict(mixed_precision=bool(mp.value), lut=bool(lut.value), reference_delays=bool(rd.value))

    def set_seed(self, seed, call_counter=0):
        _lib.check(self._L.gpurir_set_seed(self._h, int(seed), int(call_counter)), "set_seed")

    def get_seed(self):
        s, c = ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(self._L.gpurir_get_seed(self._h, ctypes.byref(s), ctypes.byref(c)), "get_seed")
        return s.value, c.value

    def set_noise(self, kind):
        _lib.check(self._L.gpurir_set_noise(self._h, {"logistic": 0, "gaussian": 1}[kind]),
                   "set_noise")

    def simulate_rir(self, room_sz, beta, pos_src, pos_rcv, orV_src, orV_rcv, spkr, mic, nb_img,
                     Tdiff, Tmax, fs, c=343.0, out=None):
        """float32 host arrays in, float32 [M_src, M_rcv, nSamples] out (C ABI host entry)."""
        room = np.ascontiguousarray(np.asarray(room_sz, dtype=np.float32).reshape(3))
        b = np.ascontiguousarray(np.asarray(beta, dtype=np.float32).reshape(6))
        nb = np.ascontiguousarray(np.asarray(nb_img, dtype=np.int32).reshape(3))
        f32 = lambda a: None if a is None else \
            np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, 3))
        pos_src, pos_rcv, orV_src, orV_rcv = f32(pos_src), f32(pos_rcv), f32(orV_src), f32(orV_rcv)
        ms, mr = pos_src.shape[0], pos_rcv.shape[0]
        if (orV_src is not None and orV_src.shape[0] != ms) or \
                (orV_rcv is not None and orV_rcv.shape[0] != mr):
            raise ValueError("orientations must have the shape of the positions")
        ns = self._L.gpurir_n_samples(float(Tmax), float(fs))
        if out is None:
            # page-locked and reused across calls: the kernels store into it directly
            out = _hostmem.pool().empty((ms, mr, ns), np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.shape == (ms, mr, ns)
        _lib.check(self._L.gpurir_simulate_rir(
            self._h, room.ctypes.data_as(_lib.fptr), b.ctypes.data_as(_lib.fptr),
            pos_src.ctypes.data, ms, pos_rcv.ctypes.data,
            orV_src.ctypes.data if orV_src is not None else None,
            orV_rcv.ctypes.data if orV_rcv is not None else None,
            int(spkr), int(mic), mr, nb.ctypes.data_as(_lib.iptr), float(Tdiff), float(Tmax),
            float(fs), float(c), out.ctypes.data), "gpurir_simulate_rir")
        return out

    def simulate_rir_device(self, room_sz, beta, d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv, spkr,
                            mic, nb_img, Tdiff, Tmax, fs, c, d_out, stream=None):
        """Stream-ordered call on device memory (torch CUDA tensors, float32, C order)."""
        room = np.ascontiguousarray(np.asarray(room_sz, dtype=np.float32).reshape(3))
        b = np.ascontiguousarray(np.asarray(beta, dtype=np.float32).reshape(6))
        nb = np.ascontiguousarray(np.asarray(nb_img, dtype=np.int32).reshape(3))
        for t in (d_pos_src, d_pos_rcv, d_orV_src, d_orV_rcv, d_out):
            if t is not None and (not t.is_cuda or not t.is_contiguous() or t.dtype != _torch().float32):
                raise ValueError("device arrays must be contiguous float32 CUDA tensors")
        if stream is None:
            stream = _torch().cuda.current_stream().cuda_stream
        _lib.check(self._L.gpurir_simulate_rir_device(
            self._h, room.ctypes.data_as(_lib.fptr), b.ctypes.data_as(_lib.fptr),
            d_pos_src.data_ptr(), d_pos_src.shape[0], d_pos_rcv.data_ptr(),
            d_orV_src.data_ptr() if d_orV_src is not None else None,
            d_orV_rcv.data_ptr() if d_orV_rcv is not None else None, int(spkr), int(mic),
            d_pos_rcv.shape[0], nb.ctypes.data_as(_lib.iptr), float(Tdiff), float(Tmax), float(fs),
            float(c), d_out.data_ptr(), ctypes.c_void_p(stream)), "gpurir_simulate_rir_device")
        return d_out

    def last_output_direct(self):
        """True when the last host-buffer call stored its RIRs from the kernels (no copy)."""
        v = ctypes.c_int()
        _lib.check(self._L.gpurir_last_output_direct(self._h, ctypes.byref(v)), "last_output_direct")
        return bool(v.value)

    def last_launch_count(self):
        """Kernels launched by the last simulate call (1 when the tail is fused)."""
        v = ctypes.c_int()
        _lib.check(self._L.gpurir_last_launch_count(self._h, ctypes.byref(v)), "last_launch_count")
        return v.value

    def set_profiling(self, on=True):
        _lib.check(self._L.gpurir_set_profiling(self._h, int(bool(on))), "set_profiling")

    def last_timing(self):
        """(ism_ms, tail_ms) of the last call, from CUDA events on its stream."""
        a, b = ctypes.c_float(), ctypes.c_float()
        _lib.check(self._L.gpurir_last_timing(self._h, ctypes.byref(a), ctypes.byref(b)), "timing")
        return a.value, b.value

    def last_transfer_bytes(self):
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(self._L.gpurir_last_transfer_bytes(self._h, ctypes.byref(a), ctypes.byref(b)),
                   "transfer_bytes")
        return a.value, b.value

    def last_envelope(self, n):
        out = np.zeros((n, 3), dtype=np.float32)
        _lib.check(self._L.gpurir_last_envelope(self._h, out.ctypes.data_as(_lib.fptr), n),
                   "last_envelope")
        return out


def _torch():
    import torch
    return torch


def probe_peaks():
    """Measured FP32 FLOP/s and MUFU op/s of the current device."""
    L = _lib.load()
    a, b = ctypes.c_double(), ctypes.c_double()
    _lib.check(L.gpurir_probe_peaks(ctypes.byref(a), ctypes.byref(b)), "probe_peaks")
    return a.value, b.value


_sim = None


def simulator():
    """The module's simulator (created on first use, like gpuRIR's import-time one)."""
    global _sim
    if _sim is None:
        _sim = Simulator()
    return _sim


def seed(value, call_counter=0):
    """Key of the diffuse-tail noise: (seed, call counter); the counter advances per call."""
    simulator().set_seed(value, call_counter)


def set_noise(kind):
    """'logistic' (gpuRIR's transform, default) or 'gaussian' tail noise."""
    simulator().set_noise(kind)


def activateMixedPrecision(activate=True):
    """Half-precision sinc evaluation with FP32 accumulation (gpuRIR/__init__.py:223-232).
    Turns the lookup table off."""
    simulator().activate_mixed_precision(activate)


def activateLUT(activate=True):
    """Lookup-table sinc evaluation (gpuRIR/__init__.py:234-243).  Turns mixed precision off."""
    simulator().activate_lut(activate)


def activateReferenceDelays(activate=True):
    """Image delays rounded in float32 step by step as gpuRIR's kernel rounds them
    (src/gpuRIR_cuda.cu:336-369), so that outputs match gpuRIR's own build instead
    of the exact sum (gpuRIR's delays are up to ~4e-4 samples off at 0.3 s).  Off
    by default; independent of the mixed-precision and lookup-table switches.
    gpuRIR has no such switch: its delays are always the float32 ones."""
    simulator().activate_reference_delays(activate)


def _marshal_simulate_args(room_sz, beta, pos_src, pos_rcv, nb_img, Tmax, fs, Tdiff=None,
                           spkr_pattern="omni", mic_pattern="omni", orV_src=None, orV_rcv=None,
                           c=343.0):
    """Checks and conversions of gpuRIR/__init__.py:154-172, returning the
    arguments of the binding call (gpuRIR_bind.simulateRIR_bind order)."""
    pos_src = np.asarray(pos_src)
    pos_rcv = np.asarray(pos_rcv)
    assert not ((pos_src >= room_sz).any() or (pos_src <= 0).any()), "The sources must be inside the room"
    assert not ((pos_rcv >= room_sz).any() or (pos_rcv <= 0).any()), "The receivers must be inside the room"
    assert Tdiff is None or Tdiff <= Tmax, "Tmax must be equal or greater than Tdiff"
    assert mic_pattern in polar_patterns, "mic_pattern must be omni, homni, card, hypcard, subcard or bidir"
    assert mic_pattern == "omni" or orV_rcv is not None, "the mics are not omni but their orientation is undefined"
    assert spkr_pattern in polar_patterns, "spkr_pattern must be omni, homni, card, hypcard, subcard or bidir"
    assert spkr_pattern == "omni" or orV_src is not None, "the sources are not omni but their orientation is undefined"
    pos_src = pos_src.astype('float32', order='C', copy=False)
    pos_rcv = pos_rcv.astype('float32', order='C', copy=False)
    if Tdiff is None:
        Tdiff = Tmax
    if orV_rcv is None:
        orV_rcv = np.zeros_like(pos_rcv)
    else:
        orV_rcv = np.asarray(orV_rcv).astype('float32', order='C', copy=False)
    if orV_src is None:
        orV_src = np.zeros_like(pos_src)
    else:
        orV_src = np.asarray(orV_src).astype('float32', order='C', copy=False)
    return (room_sz, beta, pos_src, pos_rcv, orV_src, orV_rcv, polar_patterns[spkr_pattern],
            polar_patterns[mic_pattern], nb_img, Tdiff, Tmax, fs, c)


def simulateRIR(room_sz, beta, pos_src, pos_rcv, nb_img, Tmax, fs, Tdiff=None, spkr_pattern="omni",
                mic_pattern="omni", orV_src=None, orV_rcv=None, c=343.0):
    """Room impulse responses by the image-source method (gpuRIR/__init__.py:95-175).

    Returns float32 [M_src, M_rcv, nSamples], nSamples = ceil(Tmax*fs) rounded up
    to even.  Samples before Tdiff (default Tmax) come from the ISM, the rest
    from the diffuse-reverberation model.
    """
    a = _marshal_simulate_args(room_sz, beta, pos_src, pos_rcv, nb_img, Tmax, fs, Tdiff,
                               spkr_pattern, mic_pattern, orV_src, orV_rcv, c)
    (room_sz, beta, pos_src, pos_rcv, orV_src, orV_rcv, sp, mp, nb_img, Tdiff, Tmax, fs, c) = a
    if pos_src.ndim != 2 or pos_src.shape[1] != 3 or pos_rcv.ndim != 2 or pos_rcv.shape[1] != 3:
        raise ValueError("pos_src and pos_rcv must be [M, 3] arrays")
    if orV_src.shape != pos_src.shape or orV_rcv.shape != pos_rcv.shape:
        raise ValueError("orientations must have the shape of the positions")
    return simulator().simulate_rir(room_sz, beta, pos_src, pos_rcv, orV_src, orV_rcv, sp, mp,
                                    nb_img, Tdiff, Tmax, fs, c)


def simulateTrajectory(source_signal, RIRs, timestamps=None, fs=None):
    """Filter a moving source's signal through the RIRs of its trajectory
    (gpuRIR/__init__.py:177-221).  Returns float64 [len(signal) + L - 1, M_rcv]."""
    from .trajectory import simulate_trajectory
    return simulate_trajectory(source_signal, RIRs, timestamps, fs)
