"""ctypes binding of libgpurir_gb300.so (the C ABI declared in include/gpurir_gb300.h).

The library is built in-tree by gpurir_gb300._build.  There is no CPU
fallback: if the library cannot be loaded, every compute call raises.
"""
import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgpurir_gb300.so")

_lib = None
_lock = threading.Lock()

c_int, c_long, c_float, c_u32, c_u64, c_void_p, c_size_t = (
    ctypes.c_int, ctypes.c_long, ctypes.c_float, ctypes.c_uint32, ctypes.c_uint64,
    ctypes.c_void_p, ctypes.c_size_t)
fptr = ctypes.POINTER(ctypes.c_float)
iptr = ctypes.POINTER(ctypes.c_int)
u64ptr = ctypes.POINTER(ctypes.c_uint64)

# name -> (restype, argtypes); must match include/gpurir_gb300.h
SIGNATURES = {
    "gpurir_version": (ctypes.c_char_p, []),
    "gpurir_last_error": (ctypes.c_char_p, []),
    "gpurir_create": (c_int, [c_int, c_int, c_u64, ctypes.POINTER(c_void_p)]),
    "gpurir_destroy": (c_int, [c_void_p]),
    "gpurir_activate_mixed_precision": (c_int, [c_void_p, c_int, iptr]),
    "gpurir_activate_lut": (c_int, [c_void_p, c_int, iptr]),
    "gpurir_get_modes": (c_int, [c_void_p, iptr, iptr]),
    "gpurir_set_reference_delays": (c_int, [c_void_p, c_int, iptr]),
    "gpurir_get_reference_delays": (c_int, [c_void_p, iptr]),
    "gpurir_set_compensation": (c_int, [c_void_p, c_int]),
    "gpurir_set_noise": (c_int, [c_void_p, c_int]),
    "gpurir_set_seed": (c_int, [c_void_p, c_u64, c_u64]),
    "gpurir_get_seed": (c_int, [c_void_p, u64ptr, u64ptr]),
    "gpurir_n_samples": (c_int, [c_float, c_float]),
    "gpurir_simulate_rir": (c_int, [c_void_p, fptr, fptr, c_void_p, c_int, c_void_p, c_void_p,
                                    c_void_p, c_int, c_int, c_int, iptr, c_float, c_float,
                                    c_float, c_float, c_void_p]),
    "gpurir_simulate_rir_device": (c_int, [c_void_p, fptr, fptr, c_void_p, c_int, c_void_p,
                                           c_void_p, c_void_p, c_int, c_int, c_int, iptr,
                                           c_float, c_float, c_float, c_float, c_void_p,
                                           c_void_p]),
    "gpurir_philox_stream_device": (c_int, [c_u64, c_u64, c_u32, c_long, c_void_p, c_void_p]),
    "gpurir_last_envelope": (c_int, [c_void_p, fptr, c_long]),
    "gpurir_set_profiling": (c_int, [c_void_p, c_int]),
    "gpurir_last_timing": (c_int, [c_void_p, fptr, fptr]),
    "gpurir_last_transfer_bytes": (c_int, [c_void_p, u64ptr, u64ptr]),
    "gpurir_last_output_direct": (c_int, [c_void_p, iptr]),
    "gpurir_last_launch_count": (c_int, [c_void_p, iptr]),
    "gpurir_host_alloc": (c_int, [ctypes.c_size_t, ctypes.POINTER(c_void_p)]),
    "gpurir_host_free": (c_int, [c_void_p]),
    "gpurir_probe_peaks": (c_int, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "gpurir_set_tuning": (c_int, [ctypes.c_char_p, c_int]),
    "gpurir_get_tuning": (c_int, [ctypes.c_char_p, iptr]),
    "gpurir_reset_tuning": (c_int, []),
    "gpurir_device_name": (c_int, [ctypes.c_char_p, c_int]),
}


class Room(ctypes.Structure):
    """gpurir_room of include/gpurir_gb300.h."""
    _fields_ = [("room_sz", ctypes.c_float * 3), ("beta", ctypes.c_float * 6),
                ("nb_img", ctypes.c_int * 3), ("Tdiff", ctypes.c_float), ("Tmax", ctypes.c_float),
                ("n_src", ctypes.c_int), ("n_rcv", ctypes.c_int), ("spkr_pattern", ctypes.c_int),
                ("mic_pattern", ctypes.c_int)]


llptr = ctypes.POINTER(ctypes.c_longlong)
SIGNATURES.update({
    "gpurir_batch_layout": (c_int, [c_int, ctypes.POINTER(Room), c_float, llptr]),
    "gpurir_simulate_batch_device": (c_int, [c_void_p, c_int, ctypes.POINTER(Room), c_float, c_float,
                                             c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                             c_void_p]),
    "gpurir_batch_create": (c_int, [c_void_p, c_int, ctypes.POINTER(Room), c_float, c_float,
                                    c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    ctypes.POINTER(c_void_p)]),
    "gpurir_batch_launch": (c_int, [c_void_p, c_void_p]),
    "gpurir_batch_info": (c_int, [c_void_p, llptr, llptr]),
    "gpurir_batch_destroy": (c_int, [c_void_p]),
    "gpurir_device_status": (c_int, [c_void_p]),
    "gpurir_convolutions": (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p, c_int, c_int, c_void_p]),
    "gpurir_convolutions_device": (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p, c_int, c_int,
                                           c_void_p, c_void_p]),
    "gpurir_trajectory_device": (c_int, [c_void_p, c_void_p, c_int, c_int, iptr, c_void_p, c_int, c_int,
                                         c_void_p, c_void_p]),
    "gpurir_trajectory": (c_int, [c_void_p, c_void_p, c_int, c_int, iptr, c_void_p, c_int, c_int,
                                  c_void_p]),
    "gpurir_trajectory_adjoint_device": (c_int, [c_void_p, c_void_p, c_int, c_int, iptr, c_void_p, c_int,
                                                 c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "gpurir_simulate_ism_noalloc": (c_int, [fptr, fptr, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                            c_int, c_int, c_int, iptr, c_float, c_float, c_float,
                                            c_void_p, c_void_p]),
    "gpurir_ism_backward_batch_device": (c_int, [c_void_p, c_int, ctypes.POINTER(Room), c_float,
                                                 c_float] + [c_void_p] * 11),
    "gpurir_adjoint_create": (c_int, [c_void_p, c_int, ctypes.POINTER(Room), c_float, c_float,
                                      ctypes.POINTER(c_void_p)]),
    "gpurir_adjoint_forward": (c_int, [c_void_p] * 8),
    "gpurir_adjoint_backward": (c_int, [c_void_p] * 13),
    "gpurir_adjoint_status": (c_int, [c_void_p, iptr]),
    "gpurir_adjoint_l2_step": (c_int, [c_void_p] * 7 + [c_float] + [c_void_p] * 8),
    "gpurir_adjoint_destroy": (c_int, [c_void_p]),
    "gpurir_simulate_batch_device_beta": (c_int, [c_void_p, c_int, ctypes.POINTER(Room), c_float, c_float]
                                          + [c_void_p] * 7),
    "gpurir_ism_backward_batch_device_beta": (c_int, [c_void_p, c_int, ctypes.POINTER(Room), c_float,
                                                      c_float] + [c_void_p] * 12),
})


class GpuRirError(RuntimeError):
    """A gpurir_gb300 C-ABI call returned a non-zero status."""


def load(build_if_missing=False):
    """Load the library (once).  Raises ImportError if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if build_if_missing:
                from . import _build
                _build.build()
            else:
                raise ImportError(
                    "libgpurir_gb300.so is not built (run `python -c \"import __graft_entry__ as g;"
                    " g.build()\"` or `python -m gpurir_gb300._build`); there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, what=""):
    if status != 0:
        msg = _lib.gpurir_last_error().decode() if _lib is not None else ""
        raise GpuRirError("%s failed (status %d): %s" % (what, status, msg))
    return status
