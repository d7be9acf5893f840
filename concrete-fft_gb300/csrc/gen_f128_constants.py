"""Generate f128_constants.inc: the double-double constants of fft128 twiddle generation.

Definitions (src/fft128/f128_ops.rs:1219-1272 of concrete-fft): pi,
(-1)^i pi^(2i+1)/(2i+1)! and (-1)^i pi^(2i)/(2i)! for i = 1..9, sin(k pi/16)
and cos(k pi/16) for k = 1..4, evaluated at 1024 bits and split into
hi = nearest double, lo = nearest double to (x - hi).  Needs mpmath; the
generated file is committed, so builds do not.
"""
import os

import mpmath


def _nearest_double(x):
    with mpmath.workprec(53):
        return float(+x)


def _split(x):
    hi = _nearest_double(x)
    lo = _nearest_double(x - mpmath.mpf(hi))
    return hi, lo


def main():
    mpmath.mp.prec = 1024
    pi = +mpmath.pi
    rows = [("kF128Pi", [_split(pi)], False)]
    for name, odd in (("kSinPiTaylor", True), ("kCosPiTaylor", False)):
        vals = []
        for i in range(1, 10):
            k = 2 * i + 1 if odd else 2 * i
            x = pi ** k / mpmath.mpf(int(mpmath.factorial(k)))
            hi, lo = _split(x)
            sgn = -1.0 if i % 2 else 1.0
            vals.append((sgn * hi, sgn * lo))
        rows.append((name, vals, True))
    rows.append(("kSinKPiOver16", [_split(mpmath.sinpi(mpmath.mpf(k) / 16)) for k in range(1, 5)], True))
    rows.append(("kCosKPiOver16", [_split(mpmath.cospi(mpmath.mpf(k) / 16)) for k in range(1, 5)], True))
    out = ["// Generated by gen_f128_constants.py; do not edit."]
    for name, vals, is_array in rows:
        lits = ", ".join("{%r, %r}" % v for v in vals)
        if is_array:
            out.append("const f128 %s[%d] = {%s};" % (name, len(vals), lits))
        else:
            out.append("const f128 %s = %s;" % (name, lits))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "f128_constants.inc")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
