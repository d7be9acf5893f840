"""Build the golden fixtures in tests/golden/ from the reference crate's own tests.

Run it where the reference crate's sources are checked out, giving their root
directory as the argument or in CFFT_REFERENCE_ROOT:

    python tests/golden/extract_reference_golden.py <path to concrete-fft v0.5.1>

It reads the reference's Rust test sources as text (nothing is compiled or run)
and writes:

* unordered_fwd_n2048_dif4_base32_expected.npy -- the 2048 complex outputs that
  src/unordered.rs:1176-9395 (test_equivalency) compares with assert_eq!, in the
  plan's permuted order, as a (2048, 2) float64 array;
* unordered_fwd_n2048_dif4_base32_input.npy -- that test's input: StdRng
  seed_from_u64(0), re then im per element from gen_range(0.0..1.0), produced by
  the pure-Python rand 0.8 restatement below (ChaCha12 + PCG32 seed expansion);
* f128_constants_reference.json -- the double-double literals of
  src/fft128/f128_ops.rs:579-620.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
M32 = 0xFFFFFFFF
M64 = 0xFFFFFFFFFFFFFFFF


def _rotl(v, c):
    return ((v << c) | (v >> (32 - c))) & M32


def chacha12_block(key, counter):
    st = [0x61707865, 0x3320646E, 0x79622D32, 0x6B206574] + list(key) + [
        counter & M32, (counter >> 32) & M32, 0, 0]
    x = list(st)

    def qr(a, b, c, d):
        x[a] = (x[a] + x[b]) & M32; x[d] = _rotl(x[d] ^ x[a], 16)
        x[c] = (x[c] + x[d]) & M32; x[b] = _rotl(x[b] ^ x[c], 12)
        x[a] = (x[a] + x[b]) & M32; x[d] = _rotl(x[d] ^ x[a], 8)
        x[c] = (x[c] + x[d]) & M32; x[b] = _rotl(x[b] ^ x[c], 7)

    for _ in range(6):
        qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15)
        qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14)
    return [(x[i] + st[i]) & M32 for i in range(16)]


def stdrng_uniform01(seed, count):
    """rand 0.8: StdRng::seed_from_u64(seed) then `count` gen_range(0.0..1.0) draws."""
    state = seed & M64
    key = []
    for _ in range(8):
        state = (state * 6364136223846793005 + 11634580027462260723) & M64
        xorshifted = (((state >> 18) ^ state) >> 27) & M32
        rot = state >> 59
        key.append(((xorshifted >> rot) | (xorshifted << ((32 - rot) & 31))) & M32)
    out, words, counter = [], [], 0
    while len(out) < count:
        if not words:
            words = chacha12_block(key, counter)
            counter += 1
        lo, hi = words[0], words[1]
        words = words[2:]
        v = (hi << 32) | lo
        bits = (v >> 12) | 0x3FF0000000000000
        f = np.frombuffer(np.uint64(bits).tobytes(), dtype=np.float64)[0]
        out.append(float(f) - 1.0)
    return np.array(out, dtype=np.float64)


def extract_equivalency_target(src):
    start = src.index("fn test_equivalency")
    body = src[start:]
    body = body[body.index("let target"):body.index("assert_eq!(target")]
    pairs = re.findall(r"re:\s*([-0-9.eE+]+),\s*im:\s*([-0-9.eE+]+),", body)
    return np.array([[float(a), float(b)] for a, b in pairs], dtype=np.float64)


def extract_f128_constants(src):
    def grab(name):
        i = src.index(name)
        i = src.index("=", i)
        j = src.index(";\n", i)
        vals = re.findall(r"f128\(\s*([-0-9.eE+]+),\s*([-0-9.eE+]+)\s*\)", src[i:j])
        return [[float(a), float(b)] for a, b in vals]
    return {
        "pi": grab("pub const PI: Self")[0],
        "sinpi_taylor": grab("const SINPI_TAYLOR"),
        "cospi_taylor": grab("const COSPI_TAYLOR"),
        "sin_k_pi_over_16": grab("const SIN_K_PI_OVER_16_TABLE"),
        "cos_k_pi_over_16": grab("const COS_K_PI_OVER_16_TABLE"),
    }


def main(ref_root):
    with open(os.path.join(ref_root, "src", "unordered.rs")) as f:
        target = extract_equivalency_target(f.read())
    assert target.shape == (2048, 2), target.shape
    np.save(os.path.join(HERE, "unordered_fwd_n2048_dif4_base32_expected.npy"), target)
    draws = stdrng_uniform01(0, 2 * 2048).reshape(2048, 2)  # re then im per element
    np.save(os.path.join(HERE, "unordered_fwd_n2048_dif4_base32_input.npy"), draws)
    with open(os.path.join(ref_root, "src", "fft128", "f128_ops.rs")) as f:
        consts = extract_f128_constants(f.read())
    with open(os.path.join(HERE, "f128_constants_reference.json"), "w") as f:
        json.dump({k: [[repr(a), repr(b)] for a, b in (v if k != "pi" else [v])] for k, v in consts.items()},
                  f, indent=1)
    print("wrote fixtures:", target.shape, draws.shape, {k: len(v) for k, v in consts.items()})


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CFFT_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: extract_reference_golden.py <reference crate root> (or set CFFT_REFERENCE_ROOT)")
    main(root)
