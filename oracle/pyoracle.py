"""numpy front end of the CPU oracle (liboracle.so).  TEST INFRASTRUCTURE ONLY:
imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
S = ctypes.c_size_t

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.run(["make", "-s", "-C", HERE], check=True)
        L = ctypes.CDLL(LIB)
        L.oracle_bit_rev_twice.restype = S
        L.oracle_bit_rev_twice_inv.restype = S
        L.oracle_round_mod64.restype = ctypes.c_uint64
        L.oracle_round_mod64.argtypes = [ctypes.c_double]
        L.oracle_sincospi64.argtypes = [ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_f128_binop.argtypes = [ctypes.c_int] + [ctypes.c_double] * 4 + [ctypes.c_void_p]
        L.oracle_f128_sincospi.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_stdrng_uniform01.argtypes = [ctypes.c_uint64, S, ctypes.c_void_p]
        _lib = L
    return _lib


def P(a):
    return ctypes.c_void_p(a.ctypes.data)


def _ok(rc):
    if rc != 0:
        raise ValueError("oracle rejected the arguments (rc=%d)" % rc)


def as_c64(x):
    """complex128 view of a (..., n) complex array or (..., n, 2) float64 array."""
    x = np.ascontiguousarray(x)
    if x.dtype == np.complex128:
        return x
    return x.view(np.complex128)[..., 0]


def sincospi64(a):
    s, c = np.zeros(1), np.zeros(1)
    lib().oracle_sincospi64(a, P(s), P(c))
    return s[0], c[0]


def ordered_twiddles(r, n):
    w, wi = np.zeros(2 * n, np.complex128), np.zeros(2 * n, np.complex128)
    _ok(lib().oracle_init_wt(r, S(n), P(w), P(wi)))
    return w, wi


def radix(algo):
    return 2 << (int(algo) // 2)


def ordered_fwd(algo, x):
    x = np.array(as_c64(x), dtype=np.complex128, copy=True)
    n = x.shape[-1]
    w, _ = ordered_twiddles(radix(algo), n)
    flat = x.reshape(-1, n)
    _ok(lib().oracle_ordered_batch(1, int(algo), S(n), S(flat.shape[0]), P(flat), P(w), 1))
    return x


def ordered_inv(algo, x):
    x = np.array(as_c64(x), dtype=np.complex128, copy=True)
    n = x.shape[-1]
    _, wi = ordered_twiddles(radix(algo), n)
    flat = x.reshape(-1, n)
    _ok(lib().oracle_ordered_batch(0, int(algo), S(n), S(flat.shape[0]), P(flat), P(wi), 1))
    return x


def unordered_twiddles(n, base_n, base_algo):
    w = np.zeros(n + base_n, np.complex128)
    wi = np.zeros(n + base_n, np.complex128)
    _ok(lib().oracle_unordered_twiddles(S(n), S(base_n), int(base_algo), P(w), P(wi)))
    return w, wi


def unordered_fwd(base_algo, base_n, x, nthreads=1):
    x = np.array(as_c64(x), dtype=np.complex128, copy=True)
    n = x.shape[-1]
    w, _ = unordered_twiddles(n, base_n, base_algo)
    flat = x.reshape(-1, n)
    _ok(lib().oracle_unordered_batch(1, int(base_algo), S(n), S(base_n), S(flat.shape[0]), P(flat), P(w), nthreads))
    return x


def unordered_inv(base_algo, base_n, x, nthreads=1):
    x = np.array(as_c64(x), dtype=np.complex128, copy=True)
    n = x.shape[-1]
    _, wi = unordered_twiddles(n, base_n, base_algo)
    flat = x.reshape(-1, n)
    _ok(lib().oracle_unordered_batch(0, int(base_algo), S(n), S(base_n), S(flat.shape[0]), P(flat), P(wi), nthreads))
    return x


def bit_rev_twice(nbits, base_nbits, i):
    return lib().oracle_bit_rev_twice(nbits, base_nbits, S(i))


def to_standard(n, base_n, permuted):
    permuted = np.ascontiguousarray(as_c64(permuted))
    out = np.zeros_like(permuted)
    for p, o in zip(permuted.reshape(-1, n), out.reshape(-1, n)):
        _ok(lib().oracle_unordered_to_standard(S(n), S(base_n), P(p), P(o)))
    return out


def from_standard(n, base_n, standard):
    standard = np.ascontiguousarray(as_c64(standard))
    out = np.zeros_like(standard)
    for s, o in zip(standard.reshape(-1, n), out.reshape(-1, n)):
        _ok(lib().oracle_unordered_from_standard(S(n), S(base_n), P(s), P(o)))
    return out


def fwd_monomial(n, base_n, degree):
    out = np.zeros(n, np.complex128)
    _ok(lib().oracle_unordered_fwd_monomial(S(n), S(base_n), S(degree), P(out)))
    return out


def f128_twiddles(n):
    t = np.zeros((4, n))
    _ok(lib().oracle_f128_twiddles(S(n), P(t[0]), P(t[1]), P(t[2]), P(t[3])))
    return t


def f128_fwd(re0, re1, im0, im1):
    a = [np.array(v, dtype=np.float64, copy=True) for v in (re0, re1, im0, im1)]
    n = a[0].shape[-1]
    t = f128_twiddles(n)
    for row in range(a[0].reshape(-1, n).shape[0]):
        v = [x.reshape(-1, n)[row] for x in a]
        _ok(lib().oracle_f128_fwd(S(n), *[P(x) for x in v], *[P(x) for x in t]))
    return a


def f128_inv(re0, re1, im0, im1):
    a = [np.array(v, dtype=np.float64, copy=True) for v in (re0, re1, im0, im1)]
    n = a[0].shape[-1]
    t = f128_twiddles(n)
    for row in range(a[0].reshape(-1, n).shape[0]):
        v = [x.reshape(-1, n)[row] for x in a]
        _ok(lib().oracle_f128_inv(S(n), *[P(x) for x in v], *[P(x) for x in t]))
    return a


def f128_binop(op, a, b):
    out = np.zeros(2)
    _ok(lib().oracle_f128_binop(op, a[0], a[1], b[0], b[1], P(out)))
    return out[0], out[1]


def f128_sincospi(x):
    s, c = np.zeros(2), np.zeros(2)
    _ok(lib().oracle_f128_sincospi(x[0], x[1], P(s), P(c)))
    return (s[0], s[1]), (c[0], c[1])


def u64_schoolbook(a, b):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.int64)
    N = a.shape[-1]
    out = np.zeros_like(a)
    for ar, br, orow in zip(a.reshape(-1, N), np.broadcast_to(b, a.shape).reshape(-1, N), out.reshape(-1, N)):
        br = np.ascontiguousarray(br)
        _ok(lib().oracle_negacyclic_u64_schoolbook(S(N), P(ar), P(br), P(orow)))
    return out


def u64_prepare(N, base_algo, base_n, b):
    b = np.ascontiguousarray(b, dtype=np.int64)
    out = np.zeros(b.shape[:-1] + (N // 2,), np.complex128)
    for br, orow in zip(b.reshape(-1, N), out.reshape(-1, N // 2)):
        _ok(lib().oracle_u64_prepare_b(S(N), int(base_algo), S(base_n), P(br), P(orow)))
    return out


def c64_pointwise(bhat, z):
    """bhat: (n,) complex128; z: (count, n) complex128 -> bhat * z per row (the reference's
    FMA complex product)."""
    b = np.ascontiguousarray(bhat, dtype=np.complex128)
    out = np.array(z, dtype=np.complex128, copy=True, order="C")
    n = b.shape[-1]
    lib().oracle_c64_pointwise(S(n), S(out.size // n), P(b), P(out))
    return out


def u64_product(N, base_algo, base_n, a, bhat, nthreads=1):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    bhat = np.ascontiguousarray(bhat, dtype=np.complex128)
    count = a.size // N
    if bhat.size // (N // 2) != count:
        bhat = np.ascontiguousarray(np.broadcast_to(bhat.reshape(-1, N // 2)[0], (count, N // 2)))
    out = np.zeros_like(a)
    _ok(lib().oracle_u64_product_batch(S(N), int(base_algo), S(base_n), S(count), P(a), P(bhat), P(out), nthreads))
    return out


def u64_product_sum(N, base_algo, base_n, a, bhat, nthreads=1):
    """a: (count, terms, N) uint64; bhat: (count, terms, N/2) complex128 -> (count, N) uint64."""
    a = np.ascontiguousarray(a, dtype=np.uint64)
    bhat = np.ascontiguousarray(bhat, dtype=np.complex128)
    count, terms = a.shape[0], a.shape[1]
    out = np.zeros((count, N), np.uint64)
    _ok(lib().oracle_u64_product_sum(S(N), int(base_algo), S(base_n), S(terms), S(count), P(a), P(bhat), P(out),
                                     nthreads))
    return out


def u128_schoolbook(a, b):
    """a: (..., N, 2) uint64 (lo, hi); b: (..., N) int64."""
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.int64)
    N = b.shape[-1]
    out = np.zeros_like(a)
    for ar, br, orow in zip(a.reshape(-1, 2 * N), b.reshape(-1, N), out.reshape(-1, 2 * N)):
        _ok(lib().oracle_negacyclic_u128_schoolbook(S(N), P(ar), P(np.ascontiguousarray(br)), P(orow)))
    return out


def u128_prepare(N, b):
    b = np.ascontiguousarray(b, dtype=np.int64)
    out = np.zeros(b.shape[:-1] + (4, N // 2))
    for br, orow in zip(b.reshape(-1, N), out.reshape(-1, 2 * N)):
        _ok(lib().oracle_u128_prepare_b(S(N), P(br), P(orow)))
    return out


def u128_product(N, a, bhat4, nthreads=1):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    bhat4 = np.ascontiguousarray(bhat4, dtype=np.float64)
    count = a.size // (2 * N)
    out = np.zeros_like(a)
    _ok(lib().oracle_u128_product_batch(S(N), S(count), P(a), P(bhat4), P(out), nthreads))
    return out


def stdrng_uniform01(seed, count):
    out = np.zeros(count)
    _ok(lib().oracle_stdrng_uniform01(seed, S(count), P(out)))
    return out


def round_mod64(x):
    return lib().oracle_round_mod64(float(x))


# ---- in-place batch calls for the timed CPU baseline (no copies around the call) ----
def ordered_batch_inplace(fwd, algo, flat, tw, nthreads=1):
    """flat: (count, n) complex128, C-contiguous, transformed in place; tw: the init_wt table
    of the direction (ordered_twiddles)."""
    n = flat.shape[-1]
    _ok(lib().oracle_ordered_batch(int(bool(fwd)), int(algo), S(n), S(flat.size // n), P(flat), P(tw), nthreads))


def unordered_batch_inplace(fwd, base_algo, base_n, flat, tw, nthreads=1):
    n = flat.shape[-1]
    _ok(lib().oracle_unordered_batch(int(bool(fwd)), int(base_algo), S(n), S(base_n), S(flat.size // n), P(flat),
                                     P(tw), nthreads))


def f128_batch_inplace(fwd, bufs, t, nthreads=1):
    """bufs: four (count, n) float64 arrays (re0, re1, im0, im1), transformed in place;
    t: f128_twiddles(n)."""
    n = bufs[0].shape[-1]
    _ok(lib().oracle_f128_batch(int(bool(fwd)), S(n), S(bufs[0].size // n), *[P(x) for x in bufs],
                                *[P(np.ascontiguousarray(x)) for x in t], nthreads))


def schoolbook_batch(a, b, nthreads=0):
    """Exact negacyclic products of a batch, threaded: a (count, N) uint64 (u64) or
    (count, N, 2) uint64 (u128 as lo, hi); b (count, N) int64."""
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.int64)
    N = b.shape[-1]
    words = 2 if a.ndim == 3 else 1
    out = np.zeros_like(a)
    _ok(lib().oracle_schoolbook_batch(words, S(N), S(b.size // N), P(a), P(b), P(out), nthreads))
    return out


def bench_call(kind, n, algo=0, base_n=0, seconds=0.05):
    """Single-threaded per-call CPU time (seconds) of the restated reference; see
    oracle_bench_call in cfft_oracle.h for `kind`.  The repetition count grows until the
    loop runs at least `seconds`."""
    ns = ctypes.c_double()
    reps = 1
    while True:
        _ok(lib().oracle_bench_call(int(kind), int(algo), S(n), S(base_n or n), S(reps), ctypes.byref(ns)))
        if ns.value * reps * 1e-9 >= seconds or reps >= 1 << 24:
            return ns.value * 1e-9
        reps *= 4
