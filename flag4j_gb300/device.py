"""Device context and buffers over the C ABI, with Flag4j's exception mapping.

Status codes map to the exception types Flag4j throws for the same condition
(src/main/java/org/flag4j/util/ValidateParameters.java:62-67 for shapes,
src/main/java/org/flag4j/arrays/sparse/SparseValidation.java for CSR/COO):
shape errors -> LinearAlgebraException, bad arguments / invalid sparse
structure -> IllegalArgumentException, device failures -> Flag4jDeviceException.
"""
import ctypes
import os
import threading
import weakref

import numpy as np

from . import _lib
from ._lib import Flag4jDeviceException


class LinearAlgebraException(RuntimeError):
    """Mirror of org.flag4j.util.exceptions.LinearAlgebraException."""


class IllegalArgumentException(ValueError):
    """Mirror of java.lang.IllegalArgumentException."""


def check(rc):
    if rc == _lib.F4J_OK:
        return
    msg = _lib.last_error()
    if rc == _lib.F4J_ERR_SHAPE:
        raise LinearAlgebraException(msg)
    if rc in (_lib.F4J_ERR_ARG, _lib.F4J_ERR_CSR):
        raise IllegalArgumentException(msg)
    raise Flag4jDeviceException("status %d: %s" % (rc, msg))


class DeviceBuffer:
    """An f4j_buf: device memory owned by a Context, or (wrap) memory the
    device can address in place, such as pinned host memory."""

    def __init__(self, ctx, nbytes, wrap_ptr=None):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        h = ctypes.c_void_p()
        if wrap_ptr is None:
            check(ctx.lib.f4j_buf_alloc(ctx.handle, self.nbytes, ctypes.byref(h)))
        else:
            check(ctx.lib.f4j_buf_wrap(ctx.handle, ctypes.c_void_p(wrap_ptr), self.nbytes, ctypes.byref(h)))
        self.handle = h

    def upload(self, arr, offset=0, sync=True):
        arr = np.ascontiguousarray(arr)
        f = self.ctx.lib.f4j_buf_upload if sync else self.ctx.lib.f4j_buf_upload_async
        check(f(self.ctx.handle, self.handle, arr.ctypes.data, arr.nbytes, offset))
        return self

    def download(self, out, offset=0, sync=True):
        assert out.flags["C_CONTIGUOUS"]
        f = self.ctx.lib.f4j_buf_download if sync else self.ctx.lib.f4j_buf_download_async
        check(f(self.ctx.handle, self.handle, out.ctypes.data, out.nbytes, offset))
        return out

    def to_numpy(self, dtype, count):
        out = np.empty(count, dtype)
        return self.download(out)

    def zero(self):
        check(self.ctx.lib.f4j_buf_zero(self.ctx.handle, self.handle))

    def free(self):
        if self.handle is not None and self.ctx.handle is not None:
            self.ctx.lib.f4j_buf_free(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """One f4j_ctx: a device and the CUDA stream its work runs on."""

    def __init__(self, device=0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        check(self.lib.f4j_create(int(device), ctypes.byref(h)))
        self.handle = h
        self.device = device

    def alloc(self, nbytes):
        return DeviceBuffer(self, nbytes)

    def wrap(self, arr):
        """Buffer over a C-contiguous numpy array's memory (no copy): kernels
        read and write it in place across the host link.  The array must stay
        alive (and, unless the device walks host page tables, be registered
        with f4j_host_register) while the buffer is in use."""
        assert arr.flags["C_CONTIGUOUS"]
        return DeviceBuffer(self, arr.nbytes, wrap_ptr=arr.ctypes.data)

    def from_numpy(self, arr):
        arr = np.ascontiguousarray(arr)
        return DeviceBuffer(self, max(arr.nbytes, 8)).upload(arr)

    def sync(self):
        check(self.lib.f4j_sync(self.handle))

    def launches(self):
        return int(self.lib.f4j_launch_count(self.handle))

    def timer_record(self, slot):
        check(self.lib.f4j_timer_record(self.handle, slot))

    def timer_elapsed(self, a, b):
        ms = ctypes.c_float()
        check(self.lib.f4j_timer_elapsed(self.handle, a, b, ctypes.byref(ms)))
        return ms.value

    def close(self):
        if self.handle is not None:
            self.lib.f4j_destroy(self.handle)
            self.handle = None


def pinned_empty(shape, dtype=np.float64):
    """An uninitialised numpy array in page-locked host memory (f4j_host_alloc),
    for the host-buffer entry points and async copies: on GB300 its copies run
    at the host link's full rate.  The memory is freed (f4j_host_free) once the
    array and every view of it are gone."""
    lib = _lib.load()
    dtype = np.dtype(dtype)
    count = int(np.prod(shape, dtype=np.int64))
    nbytes = max(count * dtype.itemsize, 1)
    ptr = ctypes.c_void_p()
    check(lib.f4j_host_alloc(nbytes, ctypes.byref(ptr)))
    block = (ctypes.c_char * nbytes).from_address(ptr.value)
    weakref.finalize(block, lib.f4j_host_free, ptr.value)
    return np.frombuffer(block, dtype=dtype, count=count).reshape(shape)


_default = None
_dlock = threading.Lock()


def default_context():
    """Process-wide context on device F4J_DEVICE (default 0)."""
    global _default
    with _dlock:
        if _default is None:
            _default = Context(int(os.environ.get("F4J_DEVICE", "0")))
    return _default


_mode = os.environ.get("F4J_GEMM_MODE", "auto").lower()


def set_gemm_mode(mode):
    """Select the dense product path: 'auto' (split, DMMA for NaN/Inf),
    'split', 'plain' (FP64 DMMA) or 'exact' (Flag4j's order, bit-identical)."""
    global _mode
    if mode not in _lib.MODES:
        raise IllegalArgumentException("unknown GEMM mode %r" % (mode,))
    _mode = mode


def gemm_mode():
    return _lib.MODES[_mode]
