"""Device memory, streams and events over the library's own C ABI
(gbvlm_mem_*, gbvlm_stream_*, gbvlm_event_*), so the Python layer needs no
other CUDA binding.

``DeviceArray`` is the Python face of vlm::Memory's device buffers
(vlm/include/vlm_memory.hpp:22-37): a contiguous, C-ordered array of float32,
float64, int32 or int64 in device memory, laid out like the reference's
column-major tensors seen in reverse index order (see backend.py).  It has
the small interface the operators read from their arguments -- ``data_ptr()``,
``shape``, ``dtype``, ``is_cuda`` -- so any object with that interface (a
CUDA tensor of another library, for instance) can be passed instead.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import P, call

LOC_DEVICE, LOC_HOST = 0, 1
_DTYPES = {np.dtype(np.float32), np.dtype(np.float64), np.dtype(np.int32), np.dtype(np.int64)}


def dtype_name(dt):
    """'float32' / 'float64' / ... for a numpy dtype or scalar type, a name, or another library's dtype
    object whose str() ends in the name (e.g. 'torch.float32')."""
    s = str(dt)
    if "." in s and not s.startswith("<"):
        return s.rsplit(".", 1)[-1]
    return np.dtype(dt).name


def stream_handle(stream):
    """The raw stream handle of a Stream, of any object with ``cuda_stream``, of an int, or 0 (default)."""
    if stream is None:
        return None
    h = getattr(stream, "cuda_stream", stream)
    return ctypes.c_void_p(int(h)) if h else None


class Stream:
    """A non-blocking CUDA stream owned by the library (gbvlm_stream_create)."""

    def __init__(self):
        h = ctypes.c_void_p()
        call("gbvlm_stream_create", ctypes.cast(ctypes.pointer(h), P))
        self._h = h

    @property
    def cuda_stream(self):
        return self._h.value or 0

    def synchronize(self):
        call("gbvlm_stream_synchronize", self._h)

    def __del__(self):
        try:
            if self._h:
                _lib.lib().gbvlm_stream_destroy(self._h)
                self._h = None
        except Exception:
            pass


class Event:
    """A CUDA event for timing work on a stream (gbvlm_event_*)."""

    def __init__(self):
        h = ctypes.c_void_p()
        call("gbvlm_event_create", ctypes.cast(ctypes.pointer(h), P))
        self._h = h

    def record(self, stream=None):
        call("gbvlm_event_record", self._h, stream_handle(stream))

    def synchronize(self):
        call("gbvlm_event_synchronize", self._h)

    def elapsed_time(self, end):
        """Milliseconds from this event to ``end`` (both recorded and complete)."""
        ms = ctypes.c_float()
        call("gbvlm_event_elapsed_ms", self._h, end._h, ctypes.cast(ctypes.pointer(ms), P))
        return ms.value

    def __del__(self):
        try:
            if self._h:
                _lib.lib().gbvlm_event_destroy(self._h)
                self._h = None
        except Exception:
            pass


def synchronize():
    call("gbvlm_device_synchronize")


def device_info():
    """(SM count, free bytes, total bytes) of the current device."""
    sm, fr, to = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64()
    call("gbvlm_device_info", *[ctypes.cast(ctypes.pointer(x), P) for x in (sm, fr, to)])
    return sm.value, fr.value, to.value


class DeviceArray:
    """A contiguous array in device memory (gbvlm_mem_alloc)."""

    is_cuda = True

    def __init__(self, shape, dtype=np.float32):
        self.shape = tuple(int(x) for x in (shape if isinstance(shape, (tuple, list)) else (shape,)))
        self.dtype = np.dtype(dtype)
        if self.dtype not in _DTYPES:
            raise TypeError("unsupported dtype %s" % self.dtype)
        self.nbytes = int(np.prod(self.shape, dtype=np.int64)) * self.dtype.itemsize
        p = ctypes.c_void_p()
        call("gbvlm_mem_alloc", LOC_DEVICE, self.nbytes, ctypes.cast(ctypes.pointer(p), P))
        self._p = p

    # -- the interface the operators read ---------------------------------
    def data_ptr(self):
        return self._p.value or 0

    def dim(self):
        return len(self.shape)

    def numel(self):
        return int(np.prod(self.shape, dtype=np.int64))

    def is_contiguous(self):
        return True

    def __len__(self):
        return self.shape[0]

    # -- construction and transfer ------------------------------------------
    @classmethod
    def zeros(cls, shape, dtype=np.float32, stream=None):
        a = cls(shape, dtype)
        a.fill(0, stream)
        return a

    @classmethod
    def from_numpy(cls, x, stream=None):
        x = np.ascontiguousarray(x)
        a = cls(x.shape, x.dtype)
        a.copy_from(x, stream)
        return a

    def copy_from(self, x, stream=None):
        """Host array (synchronous) or another DeviceArray (stream-ordered) into this one."""
        if isinstance(x, DeviceArray):
            if x.nbytes != self.nbytes:
                raise ValueError("size mismatch")
            call("gbvlm_mem_copy", LOC_DEVICE, self._p, 1, LOC_DEVICE, x._p, 1, 1, self.nbytes, stream_handle(stream))
            return self
        x = np.ascontiguousarray(x, dtype=self.dtype)
        if x.nbytes != self.nbytes:
            raise ValueError("size mismatch: %d bytes into %d" % (x.nbytes, self.nbytes))
        call("gbvlm_mem_copy", LOC_DEVICE, self._p, 1, LOC_HOST, ctypes.c_void_p(x.ctypes.data), 1, 1, self.nbytes,
             stream_handle(stream))
        return self

    def numpy(self, stream=None):
        """A host copy (synchronous)."""
        out = np.empty(self.shape, self.dtype)
        call("gbvlm_mem_copy", LOC_HOST, ctypes.c_void_p(out.ctypes.data), 1, LOC_DEVICE, self._p, 1, 1, self.nbytes,
             stream_handle(stream))
        return out

    def fill(self, value, stream=None):
        n = self.numel()
        if self.dtype == np.float32:
            call("gbvlm_mem_fill_f32", LOC_DEVICE, self._p, 1, ctypes.c_float(value), n, stream_handle(stream))
        elif self.dtype == np.float64:
            call("gbvlm_mem_fill_f64", LOC_DEVICE, self._p, 1, ctypes.c_double(value), n, stream_handle(stream))
        else:
            self.copy_from(np.full(self.shape, value, self.dtype), stream)
        return self

    def view(self, *shape):
        """The same memory with another shape of the same size (no copy)."""
        shape = tuple(shape[0]) if len(shape) == 1 and isinstance(shape[0], (tuple, list)) else shape
        if int(np.prod(shape, dtype=np.int64)) != self.numel():
            raise ValueError("view size mismatch")
        v = object.__new__(DeviceArray)
        v.shape, v.dtype, v.nbytes, v._p = tuple(shape), self.dtype, self.nbytes, self._p
        v._base = self
        return v

    def __del__(self):
        try:
            if getattr(self, "_base", None) is None and self._p:
                _lib.lib().gbvlm_mem_free(LOC_DEVICE, self._p)
                self._p = None
        except Exception:
            pass

    def __repr__(self):
        return "DeviceArray(shape=%s, dtype=%s)" % (self.shape, self.dtype)


class PinnedArray(np.ndarray):
    """A numpy array in pinned host memory (gbvlm_mem_alloc on the host), for
    asynchronous copies."""

    def __new__(cls, shape, dtype=np.float32):
        dt = np.dtype(dtype)
        n = int(np.prod(shape, dtype=np.int64)) * dt.itemsize
        p = ctypes.c_void_p()
        call("gbvlm_mem_alloc", LOC_HOST, max(n, 1), ctypes.cast(ctypes.pointer(p), P))
        buf = (ctypes.c_char * max(n, 1)).from_address(p.value)
        obj = np.ndarray.__new__(cls, shape, dt, buffer=buf)
        obj._pinned = _PinnedOwner(p)
        return obj

    def __array_finalize__(self, obj):
        if obj is not None:
            self._pinned = getattr(obj, "_pinned", None)


class _PinnedOwner:
    def __init__(self, p):
        self.p = p

    def __del__(self):
        try:
            if self.p:
                _lib.lib().gbvlm_mem_free(LOC_HOST, self.p)
                self.p = None
        except Exception:
            pass
