"""The host double-double type of the C++ API (concrete-fft_gb300/cpp/f128.hpp,
the counterpart of src/fft128/f128_ops.rs): bit-identical to the oracle's
restatement for the f128 x f128 operations and sincospi, and within the
double-double error bound of an mpmath evaluation for the mixed f64 forms."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "concrete-fft_gb300")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("f128") / "f128_host_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-o", exe,
                        os.path.join(PKG, "cpp", "f128_host_check.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run(exe, rows):
    txt = "\n".join("%d %016x %016x %016x %016x" % tuple([op] + [int(v) for v in np.array(vals).view(np.uint64)])
                    for op, vals in rows)
    out = subprocess.run([exe], input=txt + "\n", capture_output=True, text=True, check=True).stdout.split("\n")
    res = []
    for line in out:
        if line.strip():
            res.append(np.array([int(w, 16) for w in line.split()], dtype=np.uint64).view(np.float64))
    return res


def operands(rng, k):
    e = rng.integers(-40, 40, k).astype(np.float64)
    hi = rng.uniform(-1, 1, k) * 2.0 ** e
    lo = hi * rng.uniform(-1, 1, k) * 2.0 ** -53
    return hi, lo


def test_f128_ops_bit_exact_against_oracle(checker, oracle):
    rng = np.random.default_rng(11)
    ah, al = operands(rng, 400)
    bh, bl = operands(rng, 400)
    rows, want = [], []
    for op in range(7):
        for i in range(400):
            a, b = (ah[i], al[i]), (bh[i], bl[i])
            if op == 5 and b[0] == 0.0:
                continue
            rows.append((op, [a[0], a[1], b[0], b[1]]))
            want.append(oracle.f128_binop(op, a, b))
    got = run(checker, rows)
    for (op, vals), g, w in zip(rows, got, want):
        assert np.array_equal(np.array(g[:2]).view(np.uint64), np.array(w).view(np.uint64)), (op, vals)


def test_f128_sincospi_bit_exact_against_oracle(checker, oracle):
    rng = np.random.default_rng(12)
    xs = list(rng.uniform(-1, 1, 300)) + [0.0, 0.5, -0.5, 1.0, -1.0, 0.25, 1 / 16, -3 / 16]
    # low parts point toward zero, so that |hi + lo| stays within [-1, 1]
    rows = [(7, [x, -x * rng.uniform(0, 1) * 2.0 ** -54, 0.0, 0.0]) for x in xs]
    got = run(checker, rows)
    for (op, vals), g in zip(rows, got):
        s, c = oracle.f128_sincospi((vals[0], vals[1]))
        assert np.array_equal(np.array(g).view(np.uint64), np.array([s[0], s[1], c[0], c[1]]).view(np.uint64)), vals


def test_f128_mixed_forms_within_double_double_bound(checker):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 300
    rng = np.random.default_rng(13)
    ah, al = operands(rng, 200)
    bh, bl = operands(rng, 200)
    rows = []
    for op in (8, 9, 10, 11, 12, 13):
        for i in range(200):
            rows.append((op, [ah[i], al[i], bh[i], bl[i]]))
    got = run(checker, rows)
    for (op, (a0, a1, b0, b1)), g in zip(rows, got):
        A = mpmath.mpf(a0) + mpmath.mpf(a1)
        B = mpmath.mpf(b0) + (mpmath.mpf(b1) if op == 13 else 0)
        if op == 12:
            A = mpmath.mpf(a0)
        exact = {8: A + B, 9: A - B, 10: A * B, 11: A / B, 12: A / B, 13: A / B}[op]
        r = mpmath.mpf(g[0]) + mpmath.mpf(g[1])
        assert abs(r - exact) <= abs(exact) * mpmath.mpf(2) ** -100, (op, a0, b0)
