"""The C ABI library without a GPU: it loads, exports every declared symbol,
and rejects invalid arguments before touching the device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = "".join(open(os.path.join(ROOT, "include", h)).read() for h in sorted(os.listdir(os.path.join(ROOT, "include")))
                  if h.endswith(".h"))
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cfft_\w+)\s*\(", txt)))


def test_every_declared_symbol_is_exported(cfft_lib):
    names = declared_functions()
    assert len(names) >= 40
    for name in names:
        assert hasattr(cfft_lib, name), name


def rust_ffi_functions():
    """The `extern "C"` functions the Rust drop-in crate declares (concrete-fft_gb300/rust)."""
    txt = open(os.path.join(ROOT, "concrete-fft_gb300", "rust", "src", "ffi.rs")).read()
    block = txt[txt.index('extern "C" {'):]
    block = block[:block.index("\n}\n")]
    return sorted(set(re.findall(r"pub fn (cfft_\w+)\s*\(", block)))


def test_rust_crate_binds_only_declared_exported_symbols(cfft_lib):
    """Every function of the Rust crate's FFI module is declared in include/*.h and
    exported by the library; the crate wraps every entry point of the reference's API."""
    names = rust_ffi_functions()
    declared = set(declared_functions())
    assert len(names) >= 50
    for name in names:
        assert name in declared, name
        assert hasattr(cfft_lib, name), name
    for needed in ("cfft_ordered_plan_create_measure", "cfft_unordered_fwd_monomial_host",
                   "cfft_unordered_to_standard_host", "cfft_unordered_from_standard_host", "cfft_f128_fwd_host",
                   "cfft_f128_init_negacyclic_twiddles", "cfft_f128_negacyclic_fwd_host",
                   "cfft_f128_negacyclic_inv_host", "cfft_f128_sincospi"):
        assert needed in names, needed


def test_python_signatures_cover_the_header(cfft_lib):
    import concrete_fft
    assert sorted(concrete_fft.EXPORTED) == declared_functions()


def test_argument_errors_without_device(cfft_lib):
    h = ctypes.c_void_p()
    L = cfft_lib
    assert L.cfft_ordered_plan_create(3, 0, ctypes.byref(h)) == -1           # not a power of two
    assert L.cfft_ordered_plan_create(2048, 0, ctypes.byref(h)) == -1        # n > 1024 (ordered.rs:244)
    assert L.cfft_ordered_plan_create(1024, 9, ctypes.byref(h)) == -2        # unknown FftAlgo
    assert L.cfft_ordered_plan_create(1024, 0, None) == -2
    assert L.cfft_unordered_plan_create(1024, 2, 16, ctypes.byref(h)) == -2  # base < 32 and != n
    assert L.cfft_unordered_plan_create(1024, 2, 2048, ctypes.byref(h)) == -2
    assert L.cfft_unordered_plan_create(1000, 2, 32, ctypes.byref(h)) == -1
    assert L.cfft_f128_plan_create(16, ctypes.byref(h)) == -1                # n < 32 (fft128/mod.rs:1866)
    assert L.cfft_u64_product_plan_create(2048, 6, 4096, ctypes.byref(h)) == -2
    assert L.cfft_u64_product_plan_create(100, 6, 32, ctypes.byref(h)) == -1
    assert L.cfft_u128_product_plan_create(1 << 26, ctypes.byref(h)) == -1     # N > 2^25
    assert L.cfft_unordered_plan_create(1 << 29, 2, 1024, ctypes.byref(h)) == -1  # n > 2^28
    assert L.cfft_f128_plan_create(1 << 25, ctypes.byref(h)) == -1            # n > 2^24
    assert L.cfft_u64_product_plan_create(1 << 30, 2, 1024, ctypes.byref(h)) == -1  # N > 2^29
    assert b"power of two" in L.cfft_last_error()
    buf = (ctypes.c_double * 8)()
    assert L.cfft_batch_run_host(None, buf, buf, None) == -2                 # null batch
    assert L.cfft_u128_product_host(None, buf, buf, 0, buf, 1) == -2         # null plan
    assert L.cfft_u64_product_host(None, buf, buf, 0, buf, 1) == -2
    assert L.cfft_f128_negacyclic_fwd(24, 1, *[buf] * 8, None) == -1         # not a power of two
    assert L.cfft_f128_negacyclic_inv(2048, 1, *[buf] * 4, None, buf, buf, buf, None) == -2  # null twiddles
    assert L.cfft_ordered_set_cluster_size(None, 4) == -2
    assert L.cfft_unordered_set_cluster_size(None, 3) == -2
    assert L.cfft_unordered_set_block_points(None, 1024) == -2
    assert L.cfft_f128_set_block_points(None, 1024) == -2
    assert L.cfft_unordered_block_points(None) == 0 and L.cfft_f128_block_points(None) == 0
    assert L.cfft_unordered_from_standard_h2d(None, buf, buf, 1, None) == -2
    assert L.cfft_unordered_to_standard_d2h(None, buf, buf, 1, None) == -2
    assert L.cfft_u64_fourier_mul_monomial(None, 3, buf, 1, None) == -2
    assert L.cfft_u128_product_fft(None) is None
    q = ctypes.c_void_p()
    assert L.cfft_product_queue_create(None, None, ctypes.byref(q)) == -2    # null engine
    assert L.cfft_product_queue_submit(None, None, 0, ctypes.byref(q)) == -2
    assert L.cfft_product_queue_poll(None, 1) == -2
    assert L.cfft_product_queue_wait(None, 1) == -2
    L.cfft_product_queue_destroy(None)  # no-op
    mapped = ctypes.c_void_p(1)
    assert L.cfft_diag_host_mapping(None, 8, ctypes.byref(mapped)) == 0 and mapped.value is None


def test_no_device_is_reported(cfft_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    assert cfft_lib.cfft_device_check() == -6


def test_library_has_no_oracle_dependency():
    """The product library must not link or load the oracle."""
    import subprocess
    import concrete_fft
    out = subprocess.run(["ldd", concrete_fft.LIB_PATH], capture_output=True, text=True).stdout
    assert "oracle" not in out
    strings = open(concrete_fft.LIB_PATH, "rb").read()
    assert b"liboracle" not in strings


def test_tune_cache_file_round_trip(cfft_lib, tmp_path):
    """Persisted Measure results: load, count, save, reload; malformed lines are rejected."""
    L = cfft_lib
    L.cfft_tune_clear()
    src = tmp_path / "tune.txt"
    src.write_text("NVIDIA GB300\t2\t2048\t2\t1024\t128\t1\t0\nNVIDIA GB300\t0\t1024\t3\t1024\t256\t1\t0\n")
    assert L.cfft_tune_load(str(src).encode()) == 0
    assert L.cfft_tune_entries() == 2
    out = tmp_path / "saved.txt"
    assert L.cfft_tune_save(str(out).encode()) == 0
    assert sorted(out.read_text().splitlines()) == sorted(src.read_text().splitlines())
    bad = tmp_path / "bad.txt"
    bad.write_text("NVIDIA GB300\t2\t2048\t9\t1024\t128\t1\t0\n")  # algo 9 does not exist
    assert L.cfft_tune_load(str(bad).encode()) == -2
    assert b"out of range" in L.cfft_last_error()
    L.cfft_tune_clear()
    assert L.cfft_tune_entries() == 0


def test_f128_init_negacyclic_twiddles_matches_oracle(cfft_lib, oracle):
    """init_negacyclic_twiddles is host code: positions 1..n-1 equal the oracle's table
    bit for bit, position 0 is left untouched (src/fft128/mod.rs:1805-1828)."""
    import numpy as np
    import concrete_fft as cf
    for n in (2, 16, 512, 4096):
        t = [np.full(n, 7.0) for _ in range(4)]
        cf.fft128.init_negacyclic_twiddles(*t)
        want = oracle.f128_twiddles(n)
        for k in range(4):
            assert t[k][0] == 7.0
            assert np.array_equal(t[k][1:].view(np.uint64), want[k][1:].view(np.uint64)), (n, k)
    assert cfft_lib.cfft_f128_init_negacyclic_twiddles(24, *[ctypes.c_void_p(t[0].ctypes.data)] * 4) == -1


def test_f128_sincospi_entry_point_matches_oracle(cfft_lib, oracle):
    """f128::sincospi through the C ABI is host code: bit-identical to the oracle's restatement
    of src/fft128/f128_ops.rs:534-575, and inputs outside [-1, 1] are refused (the crate
    panics there)."""
    import numpy as np
    import concrete_fft as cf
    rng = np.random.default_rng(21)
    xs = list(rng.uniform(-1, 1, 200)) + [0.0, 0.5, -0.5, 1.0, -1.0, 0.25, 1 / 16, -3 / 16]
    for x in xs:
        lo = -x * rng.uniform(0, 1) * 2.0 ** -54
        got = cf.fft128.sincospi(x, lo)
        want = oracle.f128_sincospi((x, lo))
        assert np.array_equal(np.array(got).view(np.uint64), np.array(want).view(np.uint64)), (x, lo)
    s = (ctypes.c_double * 2)()
    c = (ctypes.c_double * 2)()
    assert cfft_lib.cfft_f128_sincospi(1.0, 1e-30, s, c) == -2
    assert cfft_lib.cfft_f128_sincospi(-1.5, 0.0, s, c) == -2
    assert cfft_lib.cfft_f128_sincospi(1.0, 0.0, s, c) == 0


def test_missing_library_fails_loudly(tmp_path):
    """No silent fallback: without the built library the package refuses to load."""
    import concrete_fft._lib as L
    saved = L._lib
    L._lib = None
    try:
        with pytest.raises(ImportError, match="not built"):
            L.load(str(tmp_path / "libcfft_gb300.so"))
    finally:
        L._lib = saved
