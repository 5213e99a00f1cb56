"""Page-locked result buffers for the numpy API.

simulateRIR returns a fresh array on every call.  A fresh pageable array is
the slow case for a GPU result: its pages are first touched by the copy (or,
stored from the kernels, fault one by one from the GPU side).  The arrays
handed out here are page-locked and mapped (gpurir_host_alloc), so the
kernels store the RIRs into them directly and the transfer overlaps the
computation.  When an array and all its views are gone, its block returns to a
bounded free list and the next call of a similar size reuses it: a loop of
simulateRIR calls pays the page-locking once.
"""
import atexit
import ctypes
import threading

import numpy as np

from . import _lib

_SMALL = 64 << 10          # blocks below 1 MiB: powers of two from 64 KiB
_GRAIN = 2 << 20           # larger blocks: multiples of 2 MiB


def _size_class(nbytes):
    if nbytes <= (1 << 20):
        n = _SMALL
        while n < nbytes:
            n <<= 1
        return n
    return (nbytes + _GRAIN - 1) // _GRAIN * _GRAIN


class _Block:
    """Owner of one page-locked block; numpy arrays keep it alive as their base."""

    __slots__ = ("ptr", "nbytes", "pool", "__array_interface__")

    def __init__(self, ptr, nbytes, pool, shape, dtype):
        self.ptr, self.nbytes, self.pool = ptr, nbytes, pool
        self.__array_interface__ = {"version": 3, "shape": tuple(shape), "typestr": np.dtype(dtype).str,
                                    "data": (ptr, False), "strides": None}

    def __del__(self):
        pool = self.pool
        if pool is not None:
            self.pool = None
            pool._release(self.ptr, self.nbytes)


class PinnedPool:
    def __init__(self, max_free_bytes=1 << 30):
        self.max_free_bytes = max_free_bytes
        self._free = []            # (nbytes, ptr)
        self._free_bytes = 0
        self._lock = threading.RLock()
        self._closed = False
        self._disabled = False
        atexit.register(self._close)

    def empty(self, shape, dtype=np.float32):
        """A C-contiguous array in page-locked memory (pageable if that fails)."""
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape, dtype=np.int64)) * dtype.itemsize
        if nbytes == 0 or self._disabled:
            return np.empty(shape, dtype=dtype)
        want = _size_class(nbytes)
        ptr = None
        with self._lock:
            best = -1
            for i, (sz, _) in enumerate(self._free):
                if want <= sz <= 2 * want and (best < 0 or sz < self._free[best][0]):
                    best = i
            if best >= 0:
                sz, ptr = self._free.pop(best)
                self._free_bytes -= sz
                want = sz
        if ptr is None:
            L = _lib.load()
            p = ctypes.c_void_p()
            if L.gpurir_host_alloc(want, ctypes.byref(p)) != 0 or not p.value:
                # page-locked memory exhausted: an ordinary array (the library copies into it)
                return np.empty(shape, dtype=dtype)
            ptr = p.value
        return np.asarray(_Block(ptr, want, self, shape, dtype))

    def _release(self, ptr, nbytes):
        if self._closed:
            return          # process exit: the driver reclaims page-locked memory
        with self._lock:
            if self._free_bytes + nbytes <= self.max_free_bytes:
                self._free.append((nbytes, ptr))
                self._free_bytes += nbytes
                return
        _lib.load().gpurir_host_free(ptr)

    def trim(self):
        """Free every cached block."""
        with self._lock:
            blocks, self._free, self._free_bytes = self._free, [], 0
        L = _lib.load()
        for _, ptr in blocks:
            L.gpurir_host_free(ptr)

    def _close(self):
        self._closed = True


_pool = None
_pool_lock = threading.Lock()


def pool():
    global _pool
    with _pool_lock:
        if _pool is None:
            _pool = PinnedPool()
        return _pool
