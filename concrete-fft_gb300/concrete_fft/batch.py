"""Mixed-size transforms in one persistent launch (cfft_batch_* of include/cfft.h)."""
import ctypes

import numpy as np

from . import _buffers as B
from ._lib import check, load
from .ordered import FftAlgo

ORDERED, UNORDERED = 0, 1
FWD, INV, FWD_THEN_INV = 1, 2, 3

ITEM_DTYPE = np.dtype([("offset", np.uint64), ("log2n", np.uint32), ("kind", np.uint32),
                       ("direction", np.uint32), ("reserved", np.uint32)])


class Batch:
    """items: structured array of ITEM_DTYPE (or a list of (offset, log2n, kind, direction))."""

    def __init__(self, items, tune_seconds=0.0):
        lib = load()
        if not isinstance(items, np.ndarray):
            items = np.array([tuple(list(it) + [0]) for it in items], dtype=ITEM_DTYPE)
        self.items = np.ascontiguousarray(items, dtype=ITEM_DTYPE)
        h = ctypes.c_void_p()
        check(lib.cfft_batch_create(ctypes.c_void_p(self.items.ctypes.data), len(self.items), float(tune_seconds),
                                    ctypes.byref(h)))
        self._h = h
        self._lib = lib

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.cfft_batch_destroy(self._h)
            self._h = None

    def units(self):
        return self._lib.cfft_batch_units(self._h)

    def schedule(self, kind, log2n, direction):
        a, b, t = ctypes.c_int(), ctypes.c_size_t(), ctypes.c_uint32()
        check(self._lib.cfft_batch_schedule(self._h, kind, log2n, direction, ctypes.byref(a), ctypes.byref(b),
                                            ctypes.byref(t)))
        return FftAlgo(a.value), b.value, t.value

    def run(self, data, stream=None):
        """One persistent launch over every item, in place on the device buffer `data`."""
        if not B.is_device(data):
            raise TypeError("batch data must be a CUDA tensor")
        s = B.stream_of(data) if stream is None else ctypes.c_void_p(stream)
        check(self._lib.cfft_batch_run(self._h, B.ptr(data), s))
        return data

    def run_host(self, host, dev, stream=None):
        """The batch from host memory and back through the device buffer `dev` (same
        layout), copies and transforms pipelined over chunks of items.  `host` is a
        C-contiguous complex128/float64 array or CPU tensor, best pinned; it is
        updated in place (only the items' point ranges)."""
        if not B.is_device(dev):
            raise TypeError("dev must be a CUDA tensor")
        if B.is_device(host):
            raise TypeError("host must be host memory")
        if B.points(host, 16) != B.points(dev, 16):
            raise ValueError("host and device buffers differ in size")
        s = B.stream_of(dev) if stream is None else ctypes.c_void_p(stream)
        check(self._lib.cfft_batch_run_host(self._h, B.ptr(host), B.ptr(dev), s))
        return host
