"""Minimal device buffers over the C ABI (nbg_dev_alloc / nbg_h2d / nbg_d2h),
so the check harness can call device-pointer entry points without torch."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class DeviceArray:
    def __init__(self, host: np.ndarray = None, *, shape=None, dtype=None):
        if host is not None:
            host = np.ascontiguousarray(host)
            shape, dtype = host.shape, host.dtype
        self.shape, self.dtype = tuple(shape), np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        p = C.c_void_p()
        L.check(L.lib().nbg_dev_alloc(C.byref(p), max(1, self.nbytes)), "dev_alloc")
        self.ptr = p.value
        if host is not None:
            self.upload(host)

    def upload(self, host):
        host = np.ascontiguousarray(host, self.dtype)
        assert host.nbytes == self.nbytes
        L.check(L.lib().nbg_h2d(self.ptr, host.ctypes.data, self.nbytes, None), "h2d")
        L.check(L.lib().nbg_stream_sync(None), "sync")

    def numpy(self):
        out = np.empty(self.shape, self.dtype)
        L.check(L.lib().nbg_d2h(out.ctypes.data, self.ptr, self.nbytes, None), "d2h")
        L.check(L.lib().nbg_stream_sync(None), "sync")
        return out

    def free(self):
        if self.ptr:
            L.lib().nbg_dev_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
