"""Batched simulation of many rooms in one persistent launch.

gpuRIR simulates one room per call (src/gpuRIR_cuda.cu:766); a batch of
rooms of uneven size, image counts, lengths and source/receiver counts runs
here as one launch whose work items (RIR segments) are ordered largest first.
Output is one flat float32 device array, packed room after room; room r's RIRs
are ``out[offsets[r]:offsets[r+1]].view(n_src, n_rcv, n_samples)``.

A room is a dict with simulateRIR's argument names: room_sz, beta, pos_src,
pos_rcv, nb_img, Tmax, Tdiff (optional), spkr_pattern, mic_pattern, orV_src,
orV_rcv.  All rooms of a batch share fs and c.
"""
import ctypes

import numpy as np

from . import _lib, polar_patterns, simulator


def _room_struct(rooms):
    arr = (_lib.Room * len(rooms))()
    for i, r in enumerate(rooms):
        ps = np.asarray(r["pos_src"]).reshape(-1, 3)
        pr = np.asarray(r["pos_rcv"]).reshape(-1, 3)
        g = arr[i]
        g.room_sz[:] = [float(x) for x in np.asarray(r["room_sz"], dtype=np.float32).reshape(3)]
        g.beta[:] = [float(x) for x in np.asarray(r["beta"], dtype=np.float32).reshape(6)]
        g.nb_img[:] = [int(x) for x in np.asarray(r["nb_img"]).reshape(3)]
        g.Tmax = float(r["Tmax"])
        g.Tdiff = float(r.get("Tdiff") if r.get("Tdiff") is not None else r["Tmax"])
        g.n_src = ps.shape[0]
        g.n_rcv = pr.shape[0]
        g.spkr_pattern = polar_patterns[r.get("spkr_pattern") or "omni"]
        g.mic_pattern = polar_patterns[r.get("mic_pattern") or "omni"]
    return arr


def _cat(rooms, key, fallback_key):
    out = []
    for r in rooms:
        v = r.get(key)
        n = np.asarray(r[fallback_key]).reshape(-1, 3).shape[0]
        out.append(np.zeros((n, 3), np.float32) if v is None else
                   np.asarray(v, dtype=np.float32).reshape(n, 3))
    return np.ascontiguousarray(np.concatenate(out, axis=0))


def pack(rooms):
    """Host arrays of a batch: (room table, pos_src, pos_rcv, orV_src, orV_rcv)."""
    return (_room_struct(rooms), _cat(rooms, "pos_src", "pos_src"), _cat(rooms, "pos_rcv", "pos_rcv"),
            _cat(rooms, "orV_src", "pos_src"), _cat(rooms, "orV_rcv", "pos_rcv"))


def layout(rooms, fs):
    """Element offsets of each room's RIRs in the packed output (n_rooms + 1 values)."""
    table = _room_struct(rooms)
    off = (ctypes.c_longlong * (len(rooms) + 1))()
    L = _lib.load()
    _lib.check(L.gpurir_batch_layout(len(rooms), table, float(fs), off), "gpurir_batch_layout")
    return np.array(off[:], dtype=np.int64)


def shapes(rooms, fs):
    from .workloads import n_samples
    return [(np.asarray(r["pos_src"]).reshape(-1, 3).shape[0],
             np.asarray(r["pos_rcv"]).reshape(-1, 3).shape[0],
             n_samples(r["Tmax"], fs)) for r in rooms]


def unpack(flat, rooms, fs):
    """Views [n_src, n_rcv, n_samples] of each room in the packed output."""
    off = layout(rooms, fs)
    return [flat[off[i]:off[i + 1]].reshape(sh) for i, sh in enumerate(shapes(rooms, fs))]


def simulate_batch(rooms, fs, c=343.0, sim=None, stream=None):
    """Simulate every room in one launch.  Returns (packed float32 CUDA tensor, offsets)."""
    import torch
    sim = sim or simulator()
    table, ps, pr, os_, or_ = pack(rooms)
    off = layout(rooms, fs)
    dev = torch.device("cuda", torch.cuda.current_device())
    d = [torch.from_numpy(a).to(dev) for a in (ps, pr, os_, or_)]
    out = torch.empty(int(off[-1]), dtype=torch.float32, device=dev)
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    L = _lib.load()
    _lib.check(L.gpurir_simulate_batch_device(sim.handle, len(rooms), table, float(fs), float(c),
                                              d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                                              d[3].data_ptr(), out.data_ptr(), ctypes.c_void_p(st)),
               "gpurir_simulate_batch_device")
    return out, off


class BatchPlan:
    """A batch planned once and captured in a CUDA graph; ``launch()`` replays it.

    The device arrays ``pos_src``, ``pos_rcv``, ``orV_src``, ``orV_rcv`` (torch
    tensors) are read at every replay: update them in place to move sources
    and receivers.  ``out`` is the packed output; ``rirs()`` gives per-room views.
    Each replay draws the next diffuse-tail noise of the simulator's seed.
    """

    def __init__(self, rooms, fs, c=343.0, sim=None):
        import torch
        self.sim = sim or simulator()
        self.rooms, self.fs = rooms, fs
        table, ps, pr, os_, or_ = pack(rooms)
        self.offsets = layout(rooms, fs)
        dev = torch.device("cuda", torch.cuda.current_device())
        self.pos_src, self.pos_rcv, self.orV_src, self.orV_rcv = \
            [torch.from_numpy(a).to(dev) for a in (ps, pr, os_, or_)]
        self.out = torch.zeros(int(self.offsets[-1]), dtype=torch.float32, device=dev)
        self._L = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._L.gpurir_batch_create(
            self.sim.handle, len(rooms), table, float(fs), float(c), self.pos_src.data_ptr(),
            self.pos_rcv.data_ptr(), self.orV_src.data_ptr(), self.orV_rcv.data_ptr(),
            self.out.data_ptr(), ctypes.byref(h)), "gpurir_batch_create")
        self._h = h

    def launch(self, stream=None):
        import torch
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _lib.check(self._L.gpurir_batch_launch(self._h, ctypes.c_void_p(st)), "gpurir_batch_launch")
        return self.out

    def rirs(self):
        return [self.out[self.offsets[i]:self.offsets[i + 1]].view(*sh)
                for i, sh in enumerate(shapes(self.rooms, self.fs))]

    def __del__(self):
        L, h = getattr(self, "_L", None), getattr(self, "_h", None)
        if L is not None and h:
            L.gpurir_batch_destroy(h)
            self._h = None
