"""ordered::Plan on the GPU (mirror of src/ordered.rs).

    plan = Plan(1024, Method.Measure(0.01))          # or Method.UserProvided(FftAlgo.Dif16)
    plan.fwd(buf); plan.inv(buf)                      # in place, unnormalised, batched over
                                                      # leading dimensions
"""
import ctypes
import enum

from . import _buffers as B
from ._lib import check, load


class FftAlgo(enum.IntEnum):
    """src/ordered.rs:28-45 (same discriminant order)."""
    Dif2 = 0
    Dit2 = 1
    Dif4 = 2
    Dit4 = 3
    Dif8 = 4
    Dit8 = 5
    Dif16 = 6
    Dit16 = 7


class Method:
    """src/ordered.rs:50-59."""

    class UserProvided:
        def __init__(self, algo):
            self.algo = FftAlgo(algo)

    class Measure:
        def __init__(self, seconds):
            self.seconds = float(seconds)


class Plan:
    """Ordered FFT plan; n a power of two, n <= 1024 (src/ordered.rs:242-278)."""

    def __init__(self, n, method):
        lib = load()
        h = ctypes.c_void_p()
        if isinstance(method, Method.UserProvided):
            check(lib.cfft_ordered_plan_create(n, int(method.algo), ctypes.byref(h)))
        elif isinstance(method, Method.Measure):
            check(lib.cfft_ordered_plan_create_measure(n, method.seconds, ctypes.byref(h)))
        else:
            raise TypeError("method must be Method.UserProvided or Method.Measure")
        self._h = h
        self._lib = lib

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.cfft_ordered_plan_destroy(self._h)
            self._h = None

    def fft_size(self):
        return self._lib.cfft_ordered_fft_size(self._h)

    def algo(self):
        return FftAlgo(self._lib.cfft_ordered_algo(self._h))

    def set_int_adds(self, eighths):
        """Share (in eighths) of butterfly additions issued on the integer pipe; results are unchanged."""
        check(self._lib.cfft_ordered_set_int_adds(self._h, int(eighths)))

    def set_cluster_size(self, ctas):
        """CTAs per transform: 0 automatic, 1 one CTA, 2/4/8 a thread-block cluster; results unchanged."""
        check(self._lib.cfft_ordered_set_cluster_size(self._h, int(ctas)))

    def int_adds(self):
        return self._lib.cfft_ordered_int_adds(self._h)

    def fft_scratch(self):
        """Bytes of caller scratch per call (0: the GPU path needs none)."""
        return self._lib.cfft_ordered_scratch_bytes(self._h)

    def _run(self, buf, fwd):
        B.check_dtype(buf, B.C64_DTYPES)
        batch = B.batch_of(buf, self.fft_size(), 16)
        if B.is_device(buf):
            fn = self._lib.cfft_ordered_fwd if fwd else self._lib.cfft_ordered_inv
            check(fn(self._h, B.ptr(buf), batch, B.stream_of(buf)))
        else:
            fn = self._lib.cfft_ordered_fwd_host if fwd else self._lib.cfft_ordered_inv_host
            check(fn(self._h, B.ptr(buf), batch))
        return buf

    def fwd(self, buf):
        """Forward transform in place (src/ordered.rs:342-347)."""
        return self._run(buf, True)

    def inv(self, buf):
        """Inverse transform in place, unnormalised (src/ordered.rs:368-373)."""
        return self._run(buf, False)

    def __repr__(self):
        return "Plan { algo: %s, fft_size: %d }" % (self.algo().name, self.fft_size())
