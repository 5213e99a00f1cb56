"""ctypes wrapper around ism_oracle.c plus numpy restatements of gpuRIR's
host-side Python (gpuRIR/__init__.py).  Test infrastructure only.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "ism_oracle.c")
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None
_lock = threading.Lock()

PATTERNS = {"omni": 0, "homni": 1, "card": 2, "hypcard": 3, "subcard": 4, "bidir": 5}


def build(force=False):
    """Compile ism_oracle.c into oracle/liboracle.so (gcc, OpenMP, -O2).

    No -march flags: the same recipe builds on x86_64 and aarch64 hosts.
    """
    if not force and os.path.exists(_LIB_PATH) and \
            os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC):
        return _LIB_PATH
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-fno-fast-math",
           _SRC, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            dp = ctypes.POINTER(ctypes.c_double)
            fp = ctypes.POINTER(ctypes.c_float)
            ip = ctypes.POINTER(ctypes.c_int)
            up = ctypes.POINTER(ctypes.c_uint32)
            L.orc_n_samples.argtypes = [ctypes.c_float, ctypes.c_float]
            L.orc_n_samples.restype = ctypes.c_int
            L.orc_window_len.argtypes = [ctypes.c_float]
            L.orc_window_len.restype = ctypes.c_int
            L.orc_amp_tau.argtypes = [fp, fp, fp, ctypes.c_int, fp, ctypes.c_int, fp, fp,
                                      ctypes.c_int, ctypes.c_int, ip, ctypes.c_float,
                                      ctypes.c_float, dp, dp, dp]
            L.orc_amp_tau.restype = None
            L.orc_tau_ref_f32.argtypes = [fp, fp, ctypes.c_int, fp, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ip, ctypes.c_float, ctypes.c_float, fp, fp]
            L.orc_tau_ref_f32.restype = None
            L.orc_ism_sum.argtypes = [dp, dp, ctypes.c_long, ctypes.c_long, ctypes.c_int,
                                      ctypes.c_float, dp, ctypes.c_long]
            L.orc_ism_sum.restype = None
            L.orc_ism_sum_lut.argtypes = L.orc_ism_sum.argtypes
            L.orc_ism_sum_lut.restype = None
            L.orc_lut_len.argtypes = [ctypes.c_float]
            L.orc_lut_len.restype = ctypes.c_int
            L.orc_lut_table.argtypes = [ctypes.c_float, fp]
            L.orc_lut_table.restype = None
            L.orc_sabine_t60.argtypes = [fp, fp]
            L.orc_sabine_t60.restype = ctypes.c_double
            L.orc_env_pred.argtypes = [dp, ctypes.c_long, dp, ctypes.c_long, ctypes.c_int,
                                       ctypes.c_float, fp, fp, dp, dp]
            L.orc_env_pred.restype = None
            L.orc_philox4x32_10.argtypes = [up, up, up]
            L.orc_philox4x32_10.restype = None
            L.orc_tail_stream.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                          ctypes.c_long, up]
            L.orc_tail_stream.restype = None
            L.orc_tail.argtypes = [dp, dp, dp, ctypes.c_long, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_uint64, ctypes.c_uint64, up, ctypes.c_int, dp,
                                   ctypes.c_long]
            L.orc_tail.restype = None
            L.orc_diffuse_from_uniforms.argtypes = [dp, dp, dp, ctypes.c_long, ctypes.c_int,
                                                    ctypes.c_int, fp, dp]
            L.orc_diffuse_from_uniforms.restype = None
            L.orc_ism_f32.argtypes = [fp, fp, fp, ctypes.c_int, fp, ctypes.c_int, fp, fp,
                                      ctypes.c_int, ctypes.c_int, ip, ctypes.c_float,
                                      ctypes.c_float, ctypes.c_int, fp, ctypes.c_long,
                                      ctypes.c_int]
            L.orc_ism_f32.restype = ctypes.c_longlong
            L.orc_rir_f32.argtypes = [fp, fp, fp, ctypes.c_int, fp, ctypes.c_int, fp, fp,
                                      ctypes.c_int, ctypes.c_int, ip, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64,
                                      ctypes.c_int, fp, ctypes.c_long, ctypes.c_int]
            L.orc_rir_f32.restype = ctypes.c_longlong
            _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def _f32(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape is not None:
        a = a.reshape(shape)
    return a


def n_samples(T, fs):
    """ceil(T*fs) in float32 arithmetic, rounded up to even (src/gpuRIR_cuda.cu:831-835)."""
    return lib().orc_n_samples(float(np.float32(T)), float(np.float32(fs)))


def window_len(fs):
    return lib().orc_window_len(float(np.float32(fs)))


def _geometry_args(room_sz, beta, pos_src, pos_rcv, orV_src, orV_rcv, nb_img):
    room = _f32(room_sz, (3,))
    b = _f32(beta, (6,))
    ps = _f32(pos_src).reshape(-1, 3)
    pr = _f32(pos_rcv).reshape(-1, 3)
    os_ = np.zeros_like(ps) if orV_src is None else _f32(orV_src, ps.shape)
    or_ = np.zeros_like(pr) if orV_rcv is None else _f32(orV_rcv, pr.shape)
    nb = np.ascontiguousarray(np.asarray(nb_img, dtype=np.int32).reshape(3))
    return room, b, ps, pr, os_, or_, nb


def amp_tau(room_sz, beta, pos_src, pos_rcv, nb_img, fs, spkr_pattern="omni",
            mic_pattern="omni", orV_src=None, orV_rcv=None, c=343.0):
    """FP64 image amplitudes and delays: (amp, tau) [M_src, M_rcv, N], tau_dp [M_src, M_rcv]."""
    room, b, ps, pr, os_, or_, nb = _geometry_args(room_sz, beta, pos_src, pos_rcv,
                                                   orV_src, orV_rcv, nb_img)
    ms, mr, N = ps.shape[0], pr.shape[0], int(np.prod(nb))
    amp = np.zeros((ms, mr, N))
    tau = np.zeros((ms, mr, N))
    tdp = np.zeros((ms, mr))
    lib().orc_amp_tau(_p(room, ctypes.c_float), _p(b, ctypes.c_float), _p(ps, ctypes.c_float),
                      ms, _p(pr, ctypes.c_float), mr, _p(os_, ctypes.c_float),
                      _p(or_, ctypes.c_float), PATTERNS[spkr_pattern], PATTERNS[mic_pattern],
                      _p(nb, ctypes.c_int), float(np.float32(c)), float(np.float32(fs)),
                      _p(amp, ctypes.c_double), _p(tau, ctypes.c_double), _p(tdp, ctypes.c_double))
    return amp, tau, tdp


def tau_reference_f32(room_sz, pos_src, pos_rcv, nb_img, fs, spkr_pattern="omni", mic_pattern="omni",
                      c=343.0):
    """Image delays rounded in float32 as the reference build forms them (the
    engine's reference-delay mode): tau [M_src, M_rcv, N], tau_dp [M_src, M_rcv]."""
    room, _, ps, pr, _, _, nb = _geometry_args(room_sz, np.zeros(6), pos_src, pos_rcv, None, None, nb_img)
    ms, mr, N = ps.shape[0], pr.shape[0], int(np.prod(nb))
    tau = np.zeros((ms, mr, N), dtype=np.float32)
    tdp = np.zeros((ms, mr), dtype=np.float32)
    lib().orc_tau_ref_f32(_p(room, ctypes.c_float), _p(ps, ctypes.c_float), ms, _p(pr, ctypes.c_float), mr,
                          PATTERNS[spkr_pattern], PATTERNS[mic_pattern], _p(nb, ctypes.c_int),
                          float(np.float32(c)), float(np.float32(fs)), _p(tau, ctypes.c_float),
                          _p(tdp, ctypes.c_float))
    return tau, tdp


def ism_sum(amp, tau, n_ism, fs, ld=None):
    """FP64 windowed-sinc sum, [M, ld] with columns [0, n_ism) filled."""
    amp = np.ascontiguousarray(amp, dtype=np.float64)
    tau = np.ascontiguousarray(tau, dtype=np.float64)
    N = amp.shape[-1]
    M = amp.size // N
    ld = n_ism if ld is None else ld
    out = np.zeros((M, ld))
    lib().orc_ism_sum(_p(amp, ctypes.c_double), _p(tau, ctypes.c_double), M, N, int(n_ism),
                      float(np.float32(fs)), _p(out, ctypes.c_double), ld)
    return out


def ism_sum_lut(amp, tau, n_ism, fs, ld=None):
    """Early part by gpuRIR's lookup-table semantics (FP64 sums), [M, ld]."""
    amp = np.ascontiguousarray(amp, dtype=np.float64)
    tau = np.ascontiguousarray(tau, dtype=np.float64)
    N = amp.shape[-1]
    M = amp.size // N
    ld = n_ism if ld is None else ld
    out = np.zeros((M, ld))
    lib().orc_ism_sum_lut(_p(amp, ctypes.c_double), _p(tau, ctypes.c_double), M, N, int(n_ism),
                          float(np.float32(fs)), _p(out, ctypes.c_double), ld)
    return out


def lut_table(fs):
    """gpuRIR's Hann x sinc lookup table (float32, 16 Tw + 1 entries)."""
    n = lib().orc_lut_len(float(np.float32(fs)))
    T = np.zeros(n, dtype=np.float32)
    lib().orc_lut_table(float(np.float32(fs)), _p(T, ctypes.c_float))
    return T


def sabine_t60(room_sz, beta):
    room = _f32(room_sz, (3,))
    b = _f32(beta, (6,))
    return lib().orc_sabine_t60(_p(room, ctypes.c_float), _p(b, ctypes.c_float))


def env_pred(rir, tau_dp, n_ism, fs, room_sz, beta):
    rir = np.ascontiguousarray(rir, dtype=np.float64)
    M, ld = rir.shape
    tdp = np.ascontiguousarray(tau_dp, dtype=np.float64).reshape(M)
    room = _f32(room_sz, (3,))
    b = _f32(beta, (6,))
    A = np.zeros(M)
    al = np.zeros(M)
    lib().orc_env_pred(_p(rir, ctypes.c_double), ld, _p(tdp, ctypes.c_double), M, int(n_ism),
                       float(np.float32(fs)), _p(room, ctypes.c_float), _p(b, ctypes.c_float),
                       _p(A, ctypes.c_double), _p(al, ctypes.c_double))
    return A, al


def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(np.asarray(ctr, dtype=np.uint32).reshape(4))
    k = np.ascontiguousarray(np.asarray(key, dtype=np.uint32).reshape(2))
    o = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_p(c, ctypes.c_uint32), _p(k, ctypes.c_uint32), _p(o, ctypes.c_uint32))
    return o


def tail_stream(seed, offset, rir_index, n):
    o = np.zeros(int(n), dtype=np.uint32)
    lib().orc_tail_stream(int(seed), int(offset), int(rir_index), int(n), _p(o, ctypes.c_uint32))
    return o


def diffuse_from_uniforms(A, alpha, tau_dp, n_ism, uniforms):
    """The reference's tail transform applied to given uniforms: [M, nDiff] float64."""
    A = np.ascontiguousarray(A, dtype=np.float64).ravel()
    al = np.ascontiguousarray(alpha, dtype=np.float64).ravel()
    tdp = np.ascontiguousarray(tau_dp, dtype=np.float64).ravel()
    M = A.size
    u = np.ascontiguousarray(uniforms, dtype=np.float32).reshape(M, -1)
    out = np.zeros(u.shape)
    lib().orc_diffuse_from_uniforms(_p(A, ctypes.c_double), _p(al, ctypes.c_double),
                                    _p(tdp, ctypes.c_double), M, int(n_ism), u.shape[1],
                                    _p(u, ctypes.c_float), _p(out, ctypes.c_double))
    return out


NOISE_KINDS = {"logistic": 0, "gaussian": 1}


def simulate_rir(room_sz, beta, pos_src, pos_rcv, nb_img, Tmax, fs, Tdiff=None,
                 spkr_pattern="omni", mic_pattern="omni", orV_src=None, orV_rcv=None, c=343.0,
                 seed=1234, offset=0, noise="logistic", return_parts=False, rir_base=0, rir_index=None):
    """FP64 restatement of cuda_simulateRIR (src/gpuRIR_cuda.cu:766-931).

    Returns float64 [M_src, M_rcv, nSamples]: the early part by the ISM, the rest
    by the envelope-shaped Philox noise of the tail (seed, offset).
    """
    if Tdiff is None:
        Tdiff = Tmax
    amp, tau, tdp = amp_tau(room_sz, beta, pos_src, pos_rcv, nb_img, fs, spkr_pattern,
                            mic_pattern, orV_src, orV_rcv, c)
    ms, mr = tdp.shape
    n_ism = n_samples(Tdiff, fs)
    n_tot = n_samples(Tmax, fs)
    n_diff = n_tot - n_ism
    out = ism_sum(amp.reshape(ms * mr, -1), tau.reshape(ms * mr, -1), n_ism, fs, ld=n_tot)
    A, al = env_pred(out, tdp, n_ism, fs, room_sz, beta)
    if n_diff > 0:
        # Philox stream per RIR: its global index in the call (C order [src][rcv] from rir_base,
        # or given per RIR when the pairs are a subset of a larger call)
        idx = (np.arange(rir_base, rir_base + ms * mr, dtype=np.uint32) if rir_index is None else
               np.ascontiguousarray(np.asarray(rir_index, dtype=np.uint32).reshape(ms * mr)))
        lib().orc_tail(_p(A, ctypes.c_double), _p(al, ctypes.c_double),
                       _p(np.ascontiguousarray(tdp.reshape(-1)), ctypes.c_double), ms * mr,
                       n_ism, n_diff, int(seed), int(offset), _p(idx, ctypes.c_uint32),
                       NOISE_KINDS[noise], _p(out, ctypes.c_double), n_tot)
    out = out.reshape(ms, mr, n_tot)
    if return_parts:
        return out, dict(amp=amp, tau=tau, tau_dp=tdp, A=A.reshape(ms, mr),
                         alpha=al.reshape(ms, mr), n_ism=n_ism, n_samples=n_tot)
    return out


def ism_f32(room_sz, beta, pos_src, pos_rcv, nb_img, Tdiff, fs, spkr_pattern="omni",
            mic_pattern="omni", orV_src=None, orV_rcv=None, c=343.0, n_threads=0, out=None):
    """FP32 threaded CPU port of the early part (the timed CPU baseline).

    Returns (rir float32 [M_src, M_rcv, nISM], windowed updates performed).
    """
    room, b, ps, pr, os_, or_, nb = _geometry_args(room_sz, beta, pos_src, pos_rcv,
                                                   orV_src, orV_rcv, nb_img)
    n_ism = n_samples(Tdiff, fs)
    ms, mr = ps.shape[0], pr.shape[0]
    if out is None:
        out = np.zeros((ms, mr, n_ism), dtype=np.float32)
    upd = lib().orc_ism_f32(_p(room, ctypes.c_float), _p(b, ctypes.c_float),
                            _p(ps, ctypes.c_float), ms, _p(pr, ctypes.c_float), mr,
                            _p(os_, ctypes.c_float), _p(or_, ctypes.c_float),
                            PATTERNS[spkr_pattern], PATTERNS[mic_pattern], _p(nb, ctypes.c_int),
                            float(np.float32(c)), float(np.float32(fs)), n_ism,
                            _p(out, ctypes.c_float), n_ism, int(n_threads))
    return out, int(upd)


def rir_f32(room_sz, beta, pos_src, pos_rcv, nb_img, Tmax, fs, Tdiff=None, spkr_pattern="omni",
            mic_pattern="omni", orV_src=None, orV_rcv=None, c=343.0, seed=1234, offset=0, noise="logistic",
            n_threads=0):
    """FP32 threaded CPU port of the whole per-RIR work of the reference (early part,
    envelope, diffuse tail): the timed CPU baseline.

    Returns (rir float32 [M_src, M_rcv, nSamples], windowed updates performed).
    """
    room, b, ps, pr, os_, or_, nb = _geometry_args(room_sz, beta, pos_src, pos_rcv,
                                                   orV_src, orV_rcv, nb_img)
    Tdiff = Tmax if Tdiff is None else Tdiff
    n_ism, n_tot = n_samples(Tdiff, fs), n_samples(Tmax, fs)
    ms, mr = ps.shape[0], pr.shape[0]
    out = np.zeros((ms, mr, n_tot), dtype=np.float32)
    upd = lib().orc_rir_f32(_p(room, ctypes.c_float), _p(b, ctypes.c_float),
                            _p(ps, ctypes.c_float), ms, _p(pr, ctypes.c_float), mr,
                            _p(os_, ctypes.c_float), _p(or_, ctypes.c_float),
                            PATTERNS[spkr_pattern], PATTERNS[mic_pattern], _p(nb, ctypes.c_int),
                            float(np.float32(c)), float(np.float32(fs)), n_ism, n_tot, int(seed), int(offset),
                            NOISE_KINDS[noise], _p(out, ctypes.c_float), n_tot, int(n_threads))
    return out, int(upd)


def windowed_updates(tau, n_ism, fs):
    """Count of (RIR, image, t) triples with 0 <= t < n_ism and |t - tau| < Tw/2."""
    H = window_len(fs) / 2.0
    tau = np.asarray(tau, dtype=np.float64).ravel()
    lo = np.maximum(np.floor(tau - H) + 1, 0)
    hi = np.minimum(np.ceil(tau + H) - 1, n_ism - 1)
    return int(np.maximum(hi - lo + 1, 0).sum())


def trajectory(source_signal, RIRs, timestamps=None, fs=None):
    """numpy restatement of simulateTrajectory (gpuRIR/__init__.py:177-221):
    segmentation, float64 direct convolution, float64 overlap-add."""
    sig = np.asarray(source_signal)
    n = len(sig)
    P, R, L = RIRs.shape
    if timestamps is None:
        fs = n / P
        timestamps = np.arange(P)
    w_ini = np.append((np.asarray(timestamps) * fs).astype(int), n)
    w_len = np.diff(w_ini)
    out = np.zeros((n + L - 1, R))
    for p in range(P):
        seg = np.asarray(sig[w_ini[p]:w_ini[p + 1]], dtype=np.float32).astype(np.float64)
        for r in range(R):
            y = np.convolve(seg, np.asarray(RIRs[p, r], dtype=np.float64))
            out[w_ini[p]:w_ini[p] + len(y), r] += y
    return out


def trajectory_adjoint(source_signal, RIRs, grad_out, timestamps=None, fs=None):
    """FP64 adjoint of `trajectory` (the engine's gpurir_trajectory_adjoint_device):
    given dL/dout [n + L - 1, R], returns (dL/dsignal [n], dL/dRIRs [P, R, L]) by
    direct correlations: dL/dh_pr[k] = sum_t g[w_ini[p] + t + k, r] x_p[t] and
    dL/dx_p[t] = sum_r sum_k g[w_ini[p] + t + k, r] h_pr[k]."""
    sig = np.asarray(source_signal)
    n = len(sig)
    P, R, L = RIRs.shape
    if timestamps is None:
        fs = n / P
        timestamps = np.arange(P)
    w_ini = np.append((np.asarray(timestamps) * fs).astype(int), n)
    g = np.asarray(grad_out, dtype=np.float64)
    gsig = np.zeros(n)
    grir = np.zeros((P, R, L))
    for p in range(P):
        a, b = w_ini[p], w_ini[p + 1]
        seg = np.asarray(sig[a:b], dtype=np.float32).astype(np.float64)
        win = g[a:b + L - 1]                       # the rows the forward pass wrote for this point
        for r in range(R):
            h = np.asarray(RIRs[p, r], dtype=np.float64)
            grir[p, r] = np.correlate(win[:, r], seg, mode="valid")[:L] if len(seg) else 0.0
            gsig[a:b] += np.correlate(win[:, r], h, mode="valid")
    return gsig, grir
