"""unordered::Plan on the GPU (mirror of src/unordered.rs)."""
import ctypes

from . import _buffers as B
from ._lib import check, load
from .ordered import FftAlgo


class Method:
    """src/unordered.rs:526-537."""

    class UserProvided:
        def __init__(self, base_algo, base_n):
            self.base_algo = FftAlgo(base_algo)
            self.base_n = int(base_n)

    class Measure:
        def __init__(self, seconds):
            self.seconds = float(seconds)


class Plan:
    """Unordered FFT plan: forward output and inverse input in the plan's
    permuted order, which depends only on (n, base_n)."""

    def __init__(self, n, method):
        lib = load()
        h = ctypes.c_void_p()
        if isinstance(method, Method.UserProvided):
            check(lib.cfft_unordered_plan_create(n, int(method.base_algo), method.base_n, ctypes.byref(h)))
        elif isinstance(method, Method.Measure):
            check(lib.cfft_unordered_plan_create_measure(n, method.seconds, ctypes.byref(h)))
        else:
            raise TypeError("method must be Method.UserProvided or Method.Measure")
        self._h = h
        self._lib = lib

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.cfft_unordered_plan_destroy(self._h)
            self._h = None

    def fft_size(self):
        return self._lib.cfft_unordered_fft_size(self._h)

    def algo(self):
        a, b = ctypes.c_int(), ctypes.c_size_t()
        self._lib.cfft_unordered_algo(self._h, ctypes.byref(a), ctypes.byref(b))
        return FftAlgo(a.value), b.value

    def set_int_adds(self, eighths):
        """Share (in eighths) of butterfly additions issued on the integer pipe; results are unchanged."""
        check(self._lib.cfft_unordered_set_int_adds(self._h, int(eighths)))

    def set_cluster_size(self, ctas):
        """CTAs per transform: 0 automatic, 1 one CTA, 2/4/8 a thread-block cluster; results unchanged."""
        check(self._lib.cfft_unordered_set_cluster_size(self._h, int(ctas)))

    def set_block_points(self, points):
        """Sub-transform size one CTA holds in shared memory: 0 automatic, else one of the
        plan's level sizes of at most 4096 points; results unchanged."""
        check(self._lib.cfft_unordered_set_block_points(self._h, int(points)))

    def block_points(self):
        return self._lib.cfft_unordered_block_points(self._h)

    def int_adds(self):
        return self._lib.cfft_unordered_int_adds(self._h)

    def fft_scratch(self):
        return self._lib.cfft_unordered_scratch_bytes(self._h)

    def _run(self, buf, fwd):
        B.check_dtype(buf, B.C64_DTYPES)
        batch = B.batch_of(buf, self.fft_size(), 16)
        if B.is_device(buf):
            fn = self._lib.cfft_unordered_fwd if fwd else self._lib.cfft_unordered_inv
            check(fn(self._h, B.ptr(buf), batch, B.stream_of(buf)))
        else:
            fn = self._lib.cfft_unordered_fwd_host if fwd else self._lib.cfft_unordered_inv_host
            check(fn(self._h, B.ptr(buf), batch))
        return buf

    def fwd(self, buf):
        """src/unordered.rs:826-839"""
        return self._run(buf, True)

    def inv(self, buf):
        """src/unordered.rs:927-940"""
        return self._run(buf, False)

    def fwd_monomial(self, degree, buf):
        """FFT of X^degree into buf, permuted order (src/unordered.rs:844-900)."""
        B.check_dtype(buf, B.C64_DTYPES)
        if B.batch_of(buf, self.fft_size(), 16) != 1:
            raise ValueError("fwd_monomial takes one buffer of fft_size points")
        if B.is_device(buf):
            check(self._lib.cfft_unordered_fwd_monomial(self._h, degree, B.ptr(buf), B.stream_of(buf)))
        else:
            check(self._lib.cfft_unordered_fwd_monomial_host(self._h, degree, B.ptr(buf)))
        return buf

    def to_standard(self, permuted, standard):
        """Element order of serialize_fourier_buffer (src/unordered.rs:951-970)."""
        return self._perm(permuted, standard, True)

    def from_standard(self, standard, permuted):
        """Element order of deserialize_fourier_buffer (src/unordered.rs:981-1036)."""
        return self._perm(standard, permuted, False)

    def _perm(self, src, dst, to_std):
        batch = B.batch_of(src, self.fft_size(), 16)
        if B.batch_of(dst, self.fft_size(), 16) != batch:
            raise ValueError("source and destination sizes differ")
        sd, dd = B.is_device(src), B.is_device(dst)
        if sd and dd:
            fn = self._lib.cfft_unordered_to_standard if to_std else self._lib.cfft_unordered_from_standard
            check(fn(self._h, B.ptr(src), B.ptr(dst), batch, B.stream_of(src)))
        elif not sd and not dd:
            fn = self._lib.cfft_unordered_to_standard_host if to_std else self._lib.cfft_unordered_from_standard_host
            check(fn(self._h, B.ptr(src), B.ptr(dst), batch))
        elif not to_std and dd:  # serialized host data straight into a device Fourier buffer
            check(self._lib.cfft_unordered_from_standard_h2d(self._h, B.ptr(src), B.ptr(dst), batch, B.stream_of(dst)))
        elif to_std and sd:  # a device Fourier buffer straight into serialized host data
            check(self._lib.cfft_unordered_to_standard_d2h(self._h, B.ptr(src), B.ptr(dst), batch, B.stream_of(src)))
        else:
            raise ValueError("permuted data must be on the device when the standard-order side is on the host")
        return dst

    def serialize_fourier_buffer(self, buf):
        """Standard-order copy of a permuted Fourier buffer (the serde wire order)."""
        import numpy as np
        out = np.empty_like(buf) if not B.is_device(buf) else buf.clone()
        return self.to_standard(buf, out)

    def deserialize_fourier_buffer(self, standard, buf):
        """Fill buf (permuted order) from a standard-order sequence; the length
        must equal fft_size (src/unordered.rs:1027-1031)."""
        if B.points(standard, 16) != B.points(buf, 16):
            from ._lib import CfftError
            raise CfftError(-3, "invalid length %d, expected a sequence of %d 64-bit complex numbers"
                            % (B.points(standard, 16), B.points(buf, 16)))
        return self.from_standard(standard, buf)

    def __repr__(self):
        a, b = self.algo()
        return "Plan { base_algo: %s, base_size: %d, fft_size: %d }" % (a.name, b, self.fft_size())
