"""The oracle against the reference's own known-answer data (CPU only)."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_stdrng_restatement_matches_fixture(oracle):
    """rand 0.8 StdRng::seed_from_u64(0) + gen_range(0.0..1.0), C restatement vs the
    pure-Python one that produced the committed input fixture."""
    inp = np.load(os.path.join(GOLDEN, "unordered_fwd_n2048_dif4_base32_input.npy"))
    c = oracle.stdrng_uniform01(0, 4096).reshape(2048, 2)
    assert np.array_equal(c.view(np.uint64), inp.view(np.uint64))


def test_unordered_golden_vector_bit_exact(oracle):
    """src/unordered.rs:1176-9395 (test_equivalency): n = 2048, Dif4, base 32, assert_eq!."""
    inp = np.load(os.path.join(GOLDEN, "unordered_fwd_n2048_dif4_base32_input.npy"))
    exp = np.load(os.path.join(GOLDEN, "unordered_fwd_n2048_dif4_base32_expected.npy"))
    out = oracle.unordered_fwd(2, 32, inp)
    assert np.array_equal(out.view(np.float64).reshape(2048, 2).view(np.uint64), exp.view(np.uint64))


def _parse_inc(path):
    import re
    txt = open(path).read()
    out = {}
    for name, body in re.findall(r"const f128 (\w+)(?:\[\d+\])? = (.*?);\n", txt):
        vals = re.findall(r"\{([-0-9.e+]+), ([-0-9.e+]+)\}", body)
        out[name] = [[float(a), float(b)] for a, b in vals]
    return out


@pytest.mark.parametrize("inc", ["oracle/f128_constants.inc", "concrete-fft_gb300/csrc/f128_constants.inc"])
def test_f128_constants_match_reference_literals(inc):
    ref = json.load(open(os.path.join(GOLDEN, "f128_constants_reference.json")))
    got = _parse_inc(os.path.join(ROOT, inc))
    names = {"pi": "kF128Pi", "sinpi_taylor": "kSinPiTaylor", "cospi_taylor": "kCosPiTaylor",
             "sin_k_pi_over_16": "kSinKPiOver16", "cos_k_pi_over_16": "kCosKPiOver16"}
    for k, cname in names.items():
        want = [[float(a), float(b)] for a, b in ref[k]]
        assert got[cname] == want, k


def test_sincospi64_accuracy(oracle):
    """fft_simd.rs sincospi64: within 1 ulp of sin/cos(pi x) on the twiddle grid."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    for n in (8, 64, 1024, 65536):
        for k in range(0, 2 * n, max(1, n // 64)):
            x = -2.0 * k / n
            s, c = oracle.sincospi64(x)
            assert abs(s - mpmath.sinpi(x)) <= 1.2e-16 and abs(c - mpmath.cospi(x)) <= 1.2e-16


def test_f128_ops_vs_mpmath(oracle):
    """Error bounds of src/fft128/f128_ops.rs:1044-1215 (rug at 1024 bits there, mpmath here)."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 300
    rng = np.random.default_rng(0)

    def dd(x):
        hi = float(x)
        return hi, float(x - hi)

    def val(p):
        return mpmath.mpf(p[0]) + mpmath.mpf(p[1])

    for _ in range(200):
        a = dd(mpmath.mpf(rng.standard_normal()) * (1 + mpmath.mpf(rng.standard_normal()) * 2 ** -60))
        b = dd(mpmath.mpf(rng.standard_normal()) * (1 + mpmath.mpf(rng.standard_normal()) * 2 ** -60))
        A, Bv = val(a), val(b)
        for op, exact, bound in ((0, A + Bv, 2 ** -104), (1, A - Bv, 2 ** -104), (2, A * Bv, 2 ** -104),
                                 (3, A + Bv, 2 ** -101), (4, A - Bv, 2 ** -101), (5, A / Bv, 2 ** -104)):
            r = val(oracle.f128_binop(op, a, b))
            if exact != 0:
                assert abs((r - exact) / exact) <= bound * 4, (op, a, b)
    for _ in range(200):
        x = dd(mpmath.mpf(rng.uniform(-1, 1)))
        s, c = oracle.f128_sincospi(x)
        X = val(x)
        assert abs(val(s) - mpmath.sinpi(X)) <= 2 ** -103 * 4
        assert abs(val(c) - mpmath.cospi(X)) <= 2 ** -103 * 4
