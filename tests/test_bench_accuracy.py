"""The bench's accuracy arithmetic, checked on the CPU: the exact u64 products it
computes with wrapping numpy arithmetic equal the oracle's schoolbook, and its torus
error in bits (signed 64- and 128-bit differences) equals a Python big-integer
computation."""
import importlib.util
import math
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("cfft_bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_exact_u64_products_equal_the_schoolbook(oracle):
    b = _bench()
    rng = np.random.default_rng(1)
    N = 64
    a = rng.integers(0, 2 ** 64, (5, N), dtype=np.uint64)
    d = rng.integers(-2 ** 7, 2 ** 7, (5, N))
    got = b.exact_u64_products(np, a, d, [0, 2, 4])
    want = oracle.schoolbook_batch(a[[0, 2, 4]], d[[0, 2, 4]], 2)
    assert np.array_equal(got, want)


def _bits(diffs):
    worst = max(abs(x) for x in diffs)
    return math.log2(worst) if worst else 0.0


def test_torus_bits_u64_matches_big_integers():
    b = _bench()
    rng = np.random.default_rng(2)
    exact = rng.integers(0, 2 ** 64, 200, dtype=np.uint64)
    delta = rng.integers(-2 ** 40, 2 ** 40, 200).astype(np.int64)
    delta[:20] = 0
    got = (exact + delta.view(np.uint64))
    bits, frac = b.torus_bits_u64(got, exact)
    assert abs(bits - _bits([int(x) for x in delta])) < 1e-9
    assert frac == (delta == 0).mean()


def test_torus_bits_u128_matches_big_integers():
    b = _bench()
    rng = np.random.default_rng(3)
    M = 1 << 128
    ex = [int(x) for x in rng.integers(0, 2 ** 63, 300)]
    ex = [(x << 65) ^ int(y) for x, y in zip(ex, rng.integers(0, 2 ** 63, 300))]
    deltas = [int(v) for v in rng.integers(-2 ** 62, 2 ** 62, 300)]
    deltas[:10] = [0] * 10
    deltas[10:20] = [(-1) ** i * (1 << (70 + i)) + i for i in range(10)]  # beyond 64 bits, both signs
    deltas[20:25] = [-1, 1, -(1 << 64), (1 << 64) - 1, -((1 << 64) - 1)]
    got = [(e + d) % M for e, d in zip(ex, deltas)]

    def pairs(vals):
        return np.array([[v & (2 ** 64 - 1), v >> 64] for v in vals], dtype=np.uint64)

    bits, frac = b.torus_bits_u128(pairs(got), pairs(ex))
    assert abs(bits - _bits(deltas)) < 1e-6
    assert frac == sum(d == 0 for d in deltas) / len(deltas)
