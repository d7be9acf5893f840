"""The integer-pipe double addition used inside the FFT kernels must equal the
native FP64 add bit for bit (it is the same IEEE operation on another pipe)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_dadd_int_equals_native_add(cuda, cfft_lib):
    import concrete_fft as cf
    bad = ctypes.c_uint64()
    pair = (ctypes.c_uint64 * 2)()
    for seed in (1, 2, 3):
        cf.check(cfft_lib.cfft_diag_dadd_check(1 << 28, seed, ctypes.byref(bad), pair))
        assert bad.value == 0, "first mismatch x=%016x y=%016x" % (pair[0], pair[1])


def test_dadd_int_rate_is_reported(cuda, cfft_lib):
    import concrete_fft as cf
    r = ctypes.c_double()
    cf.check(cfft_lib.cfft_diag_dadd_int_rate(ctypes.byref(r)))
    assert r.value > 1e10


def test_fp64_rates(cfft_lib):
    """The FP64 roof microbenchmarks: four positive rates, the peak is their best."""
    import concrete_fft as cf
    r = (ctypes.c_double * 4)()
    cf.check(cfft_lib.cfft_diag_fp64_rates(r))
    rates = list(r)
    assert all(x > 1e10 for x in rates), rates
    p = ctypes.c_double()
    cf.check(cfft_lib.cfft_diag_fp64_peak(ctypes.byref(p)))
    assert p.value > 0.9 * max(rates)
