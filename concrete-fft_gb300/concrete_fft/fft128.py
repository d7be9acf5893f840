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

    def set_block_points(self, points):
        """Points per shared-memory block: 0 automatic, else a power of two in [256, 4096];
        results unchanged."""
        check(self._lib.cfft_f128_set_block_points(self._h, int(points)))

    def block_points(self):
        return self._lib.cfft_f128_block_points(self._h)

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


def init_negacyclic_twiddles(twid_re0, twid_re1, twid_im0, twid_im1):
    """src/fft128/mod.rs:1805-1828: fills positions 1..n-1 of four host float64 arrays of
    n = len(twid_re0) (position 0 is left as it is)."""
    arrs = (twid_re0, twid_re1, twid_im0, twid_im1)
    n = len(twid_re0)
    for a in arrs:
        B.check_dtype(a, ("float64",))
        if B.is_device(a) or len(a) != n:
            raise ValueError("twiddles: four host arrays of equal length")
    check(load().cfft_f128_init_negacyclic_twiddles(n, *[B.ptr(a) for a in arrs]))


def _raw(data, twid, fwd):
    on_device = [B.is_device(a) for a in (*data, *twid)]
    if any(on_device) and not all(on_device):
        raise TypeError("negacyclic_fwd_fft/inv_fft: all eight arrays on the device, or all in host memory")
    for a in (*data, *twid):
        B.check_dtype(a, ("float64",))
    n = B.points(twid[0], 8)
    batch = B.batch_of(data[0], n, 8)
    if any(B.batch_of(d, n, 8) != batch for d in data) or any(B.points(t, 8) != n for t in twid):
        raise ValueError("data arrays must hold the same whole number of transforms of the twiddles' length")
    lib = load()
    if all(on_device):
        fn = lib.cfft_f128_negacyclic_fwd if fwd else lib.cfft_f128_negacyclic_inv
        check(fn(n, batch, *[B.ptr(d) for d in data], *[B.ptr(t) for t in twid], B.stream_of(data[0])))
    else:  # the reference's slice form: host arrays, transformed in place
        fn = lib.cfft_f128_negacyclic_fwd_host if fwd else lib.cfft_f128_negacyclic_inv_host
        check(fn(n, batch, *[B.ptr(d) for d in data], *[B.ptr(t) for t in twid]))


def negacyclic_fwd_fft(data_re0, data_re1, data_im0, data_im1, twid_re0, twid_re1, twid_im0, twid_im1):
    """src/fft128/mod.rs:1041-1071, batched over whole multiples of n: device tensors (on their
    stream) or host arrays (the reference's slices; returns when done)."""
    _raw((data_re0, data_re1, data_im0, data_im1), (twid_re0, twid_re1, twid_im0, twid_im1), True)


def negacyclic_inv_fft(data_re0, data_re1, data_im0, data_im1, twid_re0, twid_re1, twid_im0, twid_im1):
    """src/fft128/mod.rs:1073-1104 (unnormalised), device tensors or host arrays."""
    _raw((data_re0, data_re1, data_im0, data_im1), (twid_re0, twid_re1, twid_im0, twid_im1), False)


def sincospi(x_hi, x_lo=0.0):
    """f128::sincospi (src/fft128/f128_ops.rs:534-575) on the host: ((sin_hi, sin_lo),
    (cos_hi, cos_lo)) of pi * (x_hi + x_lo), for inputs in [-1, 1]."""
    s = (ctypes.c_double * 2)()
    c = (ctypes.c_double * 2)()
    check(load().cfft_f128_sincospi(float(x_hi), float(x_lo), s, c))
    return (s[0], s[1]), (c[0], c[1])
