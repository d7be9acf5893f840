"""Regenerate the double-double constants used by the oracle's fft128 restatement.

The reference (src/fft128/f128_ops.rs:1219-1272, ``generate_constants``) defines
them as pi, (-1)^i pi^(2i+1)/(2i+1)!, (-1)^i pi^(2i)/(2i)! for i = 1..9 and
sin/cos(k pi/16) for k = 1..4, each evaluated at 1024 bits and split as
hi = round_to_nearest_f64(x), lo = round_to_nearest_f64(x - hi).  This script
evaluates the same definitions with mpmath and writes oracle/f128_constants.inc.
tests/test_oracle_golden.py checks the result against the reference's literals.

Usage: python oracle/gen_f128_constants.py
"""
import os
import mpmath


def split(x):
    with mpmath.workprec(53):
        hi = +x  # round to nearest at 53 bits
    hi = float(hi)
    with mpmath.workprec(53):
        lo = +(x - hi)
    return hi, float(lo)


def constants():
    mpmath.mp.prec = 1024
    pi = mpmath.pi
    out = {"pi": split(+pi)}
    sin_t, cos_t = [], []
    fact = 1
    for i in range(1, 10):
        k = 2 * i + 1
        fact *= (k - 1) * k
        hi, lo = split(pi ** k / fact)
        s = -1.0 if i % 2 else 1.0
        sin_t.append((s * hi, s * lo))
    fact = 1
    for i in range(1, 10):
        k = 2 * i
        fact *= (k - 1) * k
        hi, lo = split(pi ** k / fact)
        s = -1.0 if i % 2 else 1.0
        cos_t.append((s * hi, s * lo))
    out["sinpi_taylor"] = sin_t
    out["cospi_taylor"] = cos_t
    out["sin_k_pi_over_16"] = [split(mpmath.sinpi(mpmath.mpf(k) / 16)) for k in range(1, 5)]
    out["cos_k_pi_over_16"] = [split(mpmath.cospi(mpmath.mpf(k) / 16)) for k in range(1, 5)]
    return out


def emit(path, type_name="f128", prefix="k"):
    c = constants()

    def lit(v):
        return "{%r, %r}" % (v[0], v[1])

    lines = ["// Generated by gen_f128_constants.py; do not edit."]
    lines.append("const %s %sF128Pi = %s;" % (type_name, prefix, lit(c["pi"])))
    for name, key in (("SinPiTaylor", "sinpi_taylor"), ("CosPiTaylor", "cospi_taylor"),
                      ("SinKPiOver16", "sin_k_pi_over_16"), ("CosKPiOver16", "cos_k_pi_over_16")):
        vals = ", ".join(lit(v) for v in c[key])
        lines.append("const %s %s%s[%d] = {%s};" % (type_name, prefix, name, len(c[key]), vals))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    emit(os.path.join(os.path.dirname(os.path.abspath(__file__)), "f128_constants.inc"))
