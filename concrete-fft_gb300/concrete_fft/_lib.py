"""ctypes binding of libcfft_gb300.so (the C ABI declared in include/cfft.h).

There is no fallback: importing this module without the built library, or
calling it without an sm_103 device, raises.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "lib", "libcfft_gb300.so")

c_size = ctypes.c_size_t
c_int = ctypes.c_int
c_dbl = ctypes.c_double
vp = ctypes.c_void_p
pp = ctypes.POINTER(ctypes.c_void_p)


class CfftError(RuntimeError):
    """A cfft_status other than CFFT_OK; `status` holds the code."""

    def __init__(self, status, message):
        super().__init__("cfft status %d: %s" % (status, message))
        self.status = status


STATUS = {
    0: "CFFT_OK", -1: "CFFT_ERR_INVALID_SIZE", -2: "CFFT_ERR_INVALID_ARGUMENT",
    -3: "CFFT_ERR_LENGTH_MISMATCH", -4: "CFFT_ERR_CUDA", -5: "CFFT_ERR_OUT_OF_MEMORY",
    -6: "CFFT_ERR_NO_DEVICE", -7: "CFFT_ERR_TIMEOUT",
}

# (name, restype, argtypes) for every entry point of include/cfft.h
_SIGS = [
    ("cfft_last_error", ctypes.c_char_p, []),
    ("cfft_version", ctypes.c_char_p, []),
    ("cfft_device_check", c_int, []),
    ("cfft_diag_fp64_peak", c_int, [ctypes.POINTER(c_dbl)]),
    ("cfft_diag_fp64_rates", c_int, [ctypes.POINTER(c_dbl)]),
    ("cfft_tune_save", c_int, [ctypes.c_char_p]),
    ("cfft_tune_load", c_int, [ctypes.c_char_p]),
    ("cfft_tune_clear", None, []),
    ("cfft_tune_entries", c_size, []),
    ("cfft_diag_dadd_check", c_int, [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64),
                                     ctypes.POINTER(ctypes.c_uint64)]),
    ("cfft_diag_dadd_int_rate", c_int, [ctypes.POINTER(c_dbl)]),
    ("cfft_diag_host_mapping", c_int, [vp, c_size, vp]),
    ("cfft_diag_set_cluster_policy", c_int, [c_int]),
    ("cfft_diag_set_spread", c_int, [c_int]),
    ("cfft_diag_set_host_chunks", c_int, [c_int, c_int, c_int, c_int]),
    ("cfft_ordered_plan_create", c_int, [c_size, c_int, pp]),
    ("cfft_ordered_plan_create_measure", c_int, [c_size, c_dbl, pp]),
    ("cfft_ordered_plan_destroy", None, [vp]),
    ("cfft_ordered_fft_size", c_size, [vp]),
    ("cfft_ordered_algo", c_int, [vp]),
    ("cfft_ordered_scratch_bytes", c_size, [vp]),
    ("cfft_ordered_fwd", c_int, [vp, vp, c_size, vp]),
    ("cfft_ordered_inv", c_int, [vp, vp, c_size, vp]),
    ("cfft_ordered_fwd_host", c_int, [vp, vp, c_size]),
    ("cfft_ordered_inv_host", c_int, [vp, vp, c_size]),
    ("cfft_ordered_set_int_adds", c_int, [vp, c_int]),
    ("cfft_ordered_set_cluster_size", c_int, [vp, c_int]),
    ("cfft_unordered_set_cluster_size", c_int, [vp, c_int]),
    ("cfft_unordered_set_block_points", c_int, [vp, c_size]),
    ("cfft_unordered_block_points", c_size, [vp]),
    ("cfft_ordered_int_adds", c_int, [vp]),
    ("cfft_unordered_set_int_adds", c_int, [vp, c_int]),
    ("cfft_unordered_int_adds", c_int, [vp]),
    ("cfft_unordered_plan_create", c_int, [c_size, c_int, c_size, pp]),
    ("cfft_unordered_plan_create_measure", c_int, [c_size, c_dbl, pp]),
    ("cfft_unordered_plan_destroy", None, [vp]),
    ("cfft_unordered_fft_size", c_size, [vp]),
    ("cfft_unordered_algo", None, [vp, ctypes.POINTER(c_int), ctypes.POINTER(c_size)]),
    ("cfft_unordered_scratch_bytes", c_size, [vp]),
    ("cfft_unordered_fwd", c_int, [vp, vp, c_size, vp]),
    ("cfft_unordered_inv", c_int, [vp, vp, c_size, vp]),
    ("cfft_unordered_fwd_host", c_int, [vp, vp, c_size]),
    ("cfft_unordered_inv_host", c_int, [vp, vp, c_size]),
    ("cfft_unordered_fwd_monomial", c_int, [vp, c_size, vp, vp]),
    ("cfft_unordered_fwd_monomial_host", c_int, [vp, c_size, vp]),
    ("cfft_unordered_to_standard", c_int, [vp, vp, vp, c_size, vp]),
    ("cfft_unordered_from_standard", c_int, [vp, vp, vp, c_size, vp]),
    ("cfft_unordered_to_standard_host", c_int, [vp, vp, vp, c_size]),
    ("cfft_unordered_from_standard_host", c_int, [vp, vp, vp, c_size]),
    ("cfft_unordered_from_standard_h2d", c_int, [vp, vp, vp, c_size, vp]),
    ("cfft_unordered_to_standard_d2h", c_int, [vp, vp, vp, c_size, vp]),
    ("cfft_f128_plan_create", c_int, [c_size, pp]),
    ("cfft_f128_plan_destroy", None, [vp]),
    ("cfft_f128_fft_size", c_size, [vp]),
    ("cfft_f128_set_block_points", c_int, [vp, c_size]),
    ("cfft_f128_block_points", c_size, [vp]),
    ("cfft_u128_product_fft", vp, [vp]),
    ("cfft_f128_fwd", c_int, [vp, vp, vp, vp, vp, c_size, vp]),
    ("cfft_f128_inv", c_int, [vp, vp, vp, vp, vp, c_size, vp]),
    ("cfft_f128_fwd_host", c_int, [vp, vp, vp, vp, vp, c_size]),
    ("cfft_f128_inv_host", c_int, [vp, vp, vp, vp, vp, c_size]),
    ("cfft_f128_init_negacyclic_twiddles", c_int, [c_size, vp, vp, vp, vp]),
    ("cfft_f128_negacyclic_fwd", c_int, [c_size, c_size, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    ("cfft_f128_negacyclic_inv", c_int, [c_size, c_size, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    ("cfft_f128_negacyclic_fwd_host", c_int, [c_size, c_size, vp, vp, vp, vp, vp, vp, vp, vp]),
    ("cfft_f128_negacyclic_inv_host", c_int, [c_size, c_size, vp, vp, vp, vp, vp, vp, vp, vp]),
    ("cfft_f128_sincospi", c_int, [c_dbl, c_dbl, vp, vp]),
    ("cfft_u64_product_plan_create", c_int, [c_size, c_int, c_size, pp]),
    ("cfft_u64_product_plan_create_measure", c_int, [c_size, c_dbl, pp]),
    ("cfft_u64_product_plan_destroy", None, [vp]),
    ("cfft_u64_product_poly_size", c_size, [vp]),
    ("cfft_u64_product_algo", None, [vp, ctypes.POINTER(c_int), ctypes.POINTER(c_size)]),
    ("cfft_u64_product_sum", c_int, [vp, vp, vp, c_size, vp, c_size, vp]),
    ("cfft_u64_fold_twist", c_int, [vp, vp, vp, c_size, vp]),
    ("cfft_c64_pointwise", c_int, [vp, c_size, vp, c_size, c_size, vp]),
    ("cfft_u64_untwist_round", c_int, [vp, vp, vp, c_size, vp]),
    ("cfft_u64_product_fft", vp, [vp]),
    ("cfft_u64_fourier_mul_monomial", c_int, [vp, ctypes.c_ulonglong, vp, c_size, vp]),
    ("cfft_u64_product_set_int_adds", c_int, [vp, c_int]),
    ("cfft_u64_product_set_cluster_size", c_int, [vp, c_int]),
    ("cfft_u64_product_int_adds", c_int, [vp]),
    ("cfft_u64_prepare_operand", c_int, [vp, vp, vp, c_size, vp]),
    ("cfft_u64_product", c_int, [vp, vp, vp, c_size, vp, c_size, vp]),
    ("cfft_u64_product_host", c_int, [vp, vp, vp, c_size, vp, c_size]),
    ("cfft_batch_create", c_int, [vp, c_size, c_dbl, pp]),
    ("cfft_batch_destroy", None, [vp]),
    ("cfft_batch_units", c_size, [vp]),
    ("cfft_batch_schedule", c_int, [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(c_int),
                                    ctypes.POINTER(c_size), ctypes.POINTER(ctypes.c_uint32)]),
    ("cfft_batch_run", c_int, [vp, vp, vp]),
    ("cfft_batch_run_host", c_int, [vp, vp, vp, vp]),
    ("cfft_product_engine_create", c_int, [vp, c_size, pp]),
    ("cfft_product_engine_destroy", None, [vp]),
    ("cfft_product_engine_workspace_bytes", c_size, [vp]),
    ("cfft_product_engine_plan", vp, [vp, ctypes.c_uint32]),
    ("cfft_product_engine_run", c_int, [vp, vp, c_size, vp, vp, vp]),
    ("cfft_product_queue_create", c_int, [vp, vp, vp]),
    ("cfft_product_queue_destroy", None, [vp]),
    ("cfft_product_queue_submit", c_int, [vp, vp, c_size, vp]),
    ("cfft_product_queue_poll", c_int, [vp, ctypes.c_uint64]),
    ("cfft_product_queue_wait", c_int, [vp, ctypes.c_uint64]),
    ("cfft_product_engine_run_static", c_int, [vp, vp, c_size, vp]),
    ("cfft_server_create", c_int, [vp, vp, c_size, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, pp]),
    ("cfft_server_destroy", None, [vp]),
    ("cfft_server_run", c_int, [vp, vp, vp]),
    ("cfft_server_recorded", c_size, [vp]),
    ("cfft_server_recorded_ids", c_int, [vp, vp, c_size]),
    ("cfft_server_recorded_output", c_int, [vp, ctypes.c_uint64, vp, c_size]),
    ("cfft_server_request_shape", c_int, [vp, vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint32),
                                          ctypes.POINTER(ctypes.c_uint32)]),
    ("cfft_server_request_inputs", c_int, [vp, vp, ctypes.c_uint64, vp, vp]),
    ("cfft_server_run_alone", c_int, [vp, vp, ctypes.c_uint64, vp, c_size]),
    ("cfft_u128_product_plan_create", c_int, [c_size, pp]),
    ("cfft_u128_product_plan_destroy", None, [vp]),
    ("cfft_u128_product_poly_size", c_size, [vp]),
    ("cfft_u128_prepare_operand", c_int, [vp, vp, vp, c_size, vp]),
    ("cfft_u128_product", c_int, [vp, vp, vp, c_size, vp, c_size, vp]),
    ("cfft_u128_product_host", c_int, [vp, vp, vp, c_size, vp, c_size]),
]

EXPORTED = [s[0] for s in _SIGS]

_lib = None


def load(path=LIB_PATH):
    """Load the shared library once and attach the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libcfft_gb300.so not built (%s): run `python concrete-fft_gb300/build.py`" % path)
    lib = ctypes.CDLL(path)
    for name, res, args in _SIGS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != 0:
        msg = load().cfft_last_error().decode(errors="replace")
        raise CfftError(status, "%s: %s" % (STATUS.get(status, "?"), msg))
    return status
