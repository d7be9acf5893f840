"""Fused negacyclic polynomial products (the caller-side pipeline that TFHE-rs
builds on unordered::Plan and fft128::Plan), on device tensors."""
import ctypes

from . import _buffers as B
from ._lib import check, load
from .ordered import FftAlgo


class U64ProductPlan:
    """out = a * B mod (X^N + 1) with u64 coefficients (torus Z/2^64)."""

    def __init__(self, N, base_algo=FftAlgo.Dif16, base_n=None, measure_seconds=None):
        lib = load()
        h = ctypes.c_void_p()
        if measure_seconds is not None:
            check(lib.cfft_u64_product_plan_create_measure(N, float(measure_seconds), ctypes.byref(h)))
        else:
            base_n = N // 2 if base_n is None else base_n
            check(lib.cfft_u64_product_plan_create(N, int(base_algo), base_n, ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self.N = N

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.cfft_u64_product_plan_destroy(self._h)
            self._h = None

    def set_int_adds(self, eighths):
        """Share (in eighths) of butterfly additions issued on the integer pipe; results are unchanged."""
        check(self._lib.cfft_u64_product_set_int_adds(self._h, int(eighths)))

    def int_adds(self):
        return self._lib.cfft_u64_product_int_adds(self._h)

    def algo(self):
        a, b = ctypes.c_int(), ctypes.c_size_t()
        self._lib.cfft_u64_product_algo(self._h, ctypes.byref(a), ctypes.byref(b))
        return FftAlgo(a.value), b.value

    def prepare_operand(self, b, bhat):
        """b: int64 device tensor (count, N) -> bhat: float64 device tensor (count, N/2, 2)."""
        count = B.batch_of(b, self.N, 8)
        check(self._lib.cfft_u64_prepare_operand(self._h, B.ptr(b), B.ptr(bhat), count, B.stream_of(b)))
        return bhat

    def product(self, a, bhat, out, shared_operand=False):
        """a, out: uint64/int64 tensors (count, N); device or host (bhat always on device)."""
        count = B.batch_of(a, self.N, 8)
        stride = 0 if shared_operand else self.N // 2
        if B.is_device(a):
            check(self._lib.cfft_u64_product(self._h, B.ptr(a), B.ptr(bhat), stride, B.ptr(out), count,
                                             B.stream_of(a)))
        else:
            check(self._lib.cfft_u64_product_host(self._h, B.ptr(a), B.ptr(bhat), stride, B.ptr(out), count))
        return out


    def set_cluster_size(self, ctas):
        """CTAs per product: 0 automatic, 1 one CTA, 2/4/8 a thread-block cluster; results unchanged."""
        check(self._lib.cfft_u64_product_set_cluster_size(self._h, int(ctas)))

    def product_unfused(self, a, bhat, out, z):
        """The same product as five separate launches (fold+twist, the N/2-point unordered
        forward transform, pointwise product, inverse transform, untwist+round): the plain
        Plan path.  a, out: (count, N) device; z: (count, N/2) complex128 device scratch.
        Bit-identical to product()."""
        count = B.batch_of(a, self.N, 8)
        s = B.stream_of(a)
        fft = self._lib.cfft_u64_product_fft(self._h)
        check(self._lib.cfft_u64_fold_twist(self._h, B.ptr(a), B.ptr(z), count, s))
        check(self._lib.cfft_unordered_fwd(fft, B.ptr(z), count, s))
        check(self._lib.cfft_c64_pointwise(B.ptr(bhat), self.N // 2, B.ptr(z), self.N // 2, count, s))
        check(self._lib.cfft_unordered_inv(fft, B.ptr(z), count, s))
        check(self._lib.cfft_u64_untwist_round(self._h, B.ptr(z), B.ptr(out), count, s))
        return out

    def fourier_mul_monomial(self, degree, z):
        """z: (count, N/2) complex128 device tensor in the plan's Fourier layout (a prepared
        operand, or a folded, twisted and forward-transformed polynomial); multiplied in place
        by the Fourier form of X^degree mod (X^N + 1), degree taken mod 2N."""
        count = B.batch_of(z, self.N // 2, 16)
        check(self._lib.cfft_u64_fourier_mul_monomial(self._h, int(degree) % (2 * self.N), B.ptr(z), count,
                                                      B.stream_of(z)))
        return z

    def product_sum(self, a, bhat, out):
        """a: (count, terms, N) device int64/uint64; bhat: (count, terms, N/2) complex128;
        out: (count, N).  out[g] = sum_t a[g, t] * B[g, t], accumulated in the Fourier domain."""
        count, terms = a.shape[0], a.shape[1]
        check(self._lib.cfft_u64_product_sum(self._h, B.ptr(a), B.ptr(bhat), terms, B.ptr(out), count,
                                             B.stream_of(a)))
        return out


class U128ProductPlan:
    """out = a * B mod (X^N + 1) with u128 coefficients as (lo, hi) u64 pairs."""

    def __init__(self, N):
        lib = load()
        h = ctypes.c_void_p()
        check(lib.cfft_u128_product_plan_create(N, ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self.N = N

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.cfft_u128_product_plan_destroy(self._h)
            self._h = None

    def prepare_operand(self, b, bhat4):
        count = B.batch_of(b, self.N, 8)
        check(self._lib.cfft_u128_prepare_operand(self._h, B.ptr(b), B.ptr(bhat4), count, B.stream_of(b)))
        return bhat4

    def product(self, a, bhat4, out, shared_operand=False):
        """a, out: (count, N, 2) u64 (lo, hi) words, device or host (bhat4 always on device)."""
        count = B.batch_of(a, 2 * self.N, 8)
        stride = 0 if shared_operand else 2 * self.N
        if B.is_device(a):
            check(self._lib.cfft_u128_product(self._h, B.ptr(a), B.ptr(bhat4), stride, B.ptr(out), count,
                                              B.stream_of(a)))
        else:
            check(self._lib.cfft_u128_product_host(self._h, B.ptr(a), B.ptr(bhat4), stride, B.ptr(out), count))
        return out
