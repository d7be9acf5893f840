"""fft128::Plan on the GPU (mirror of src/fft128/mod.rs:1832-1960): split
double-double buffers re0, re1, im0, im1 of n f64 each (batched)."""
import ctypes

from . import _buffers as B
from ._lib import check, load


class Plan:
    def __init__(self, n):
        lib = load()
        h = ctypes.c_void_p()
        check(lib.cfft_f128_plan_create(n, ctypes.byref(h)))
        self._h = h
        self._lib = lib

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.cfft_f128_plan_destroy(self._h)
            self._h = None

    def fft_size(self):
        return self._lib.cfft_f128_fft_size(self._h)

    def _run(self, re0, re1, im0, im1, fwd):
        bufs = (re0, re1, im0, im1)
        for b in bufs:
            B.check_dtype(b, ("float64",))
        batch = B.batch_of(re0, self.fft_size(), 8)
        if any(B.batch_of(b, self.fft_size(), 8) != batch for b in bufs):
            from ._lib import CfftError
            raise CfftError(-3, "re0/re1/im0/im1 lengths differ")
        if B.is_device(re0):
            fn = self._lib.cfft_f128_fwd if fwd else self._lib.cfft_f128_inv
            check(fn(self._h, *[B.ptr(b) for b in bufs], batch, B.stream_of(re0)))
        else:
            fn = self._lib.cfft_f128_fwd_host if fwd else self._lib.cfft_f128_inv_host
            check(fn(self._h, *[B.ptr(b) for b in bufs], batch))

    def fwd(self, re0, re1, im0, im1):
        """Forward negacyclic FFT, bit-reversed output (src/fft128/mod.rs:1905-1927)."""
        self._run(re0, re1, im0, im1, True)

    def inv(self, re0, re1, im0, im1):
        """Inverse negacyclic FFT, unnormalised (src/fft128/mod.rs:1938-1960)."""
        self._run(re0, re1, im0, im1, False)
