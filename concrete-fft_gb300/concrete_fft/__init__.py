"""GB300 (sm_103a) implementation of concrete-fft's FFT hot path.

Modules mirror the reference crate: `ordered`, `unordered`, `fft128`, plus the
fused negacyclic products in `product`.  Everything runs through the C ABI of
libcfft_gb300.so (include/cfft.h); there is no CPU fallback.
"""
from ._lib import CfftError, EXPORTED, LIB_PATH, check, load
from .ordered import FftAlgo
from . import ordered, unordered, fft128, product, batch, serving

__all__ = ["CfftError", "EXPORTED", "LIB_PATH", "FftAlgo", "check", "load", "ordered", "unordered", "fft128",
           "product", "batch", "serving"]
