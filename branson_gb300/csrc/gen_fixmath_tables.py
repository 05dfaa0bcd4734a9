"""Generate bgs_fixmath_tables.h: fixed-point tables for the integer log/exp.

Values are computed with Python's decimal module at 80 significant digits
and rounded to nearest:
  LOG_INVF[j] = 2^64 / F_j            F_j = 1 + j/1024, j = 1..1023 (j = 0 unused)
  LOG_LNF[j]  = ln(F_j) * 2^120       as (hi, lo) 64-bit words
  EXP2_NEG[j] = 2^(63 - j/1024)       j = 0..1023
  LN2_120     = ln 2 * 2^120          (hi, lo)
  LN2_1024_96 = ln 2 / 1024 * 2^96    (hi, lo)
  K_1024_LN2  = 1024/ln 2 * 2^32      (estimate multiplier for the exp reduction)
  2/pi * 2^128, pi/2 * 2^62, and in Q64 the magnitudes of the coefficients
  of the sin/cos polynomials (below)

The sin/cos polynomials are minimax approximations (Remez exchange, run with
mpmath at 60 digits, weight y): with t in [0, pi/4] and y = t^2,
  sin t = t (1 - y B(y)),  B of degree 6,  max |y (B - (1 - sin t / t)/y)| ~ 2^-68
  cos t = 1 - y C(y),      C of degree 7,  max |y (C - (1 - cos t)/y)|     ~ 2^-75
(the Taylor forms need degrees 8 and 8 for the same accuracy).  Their
coefficients alternate in sign, and the tables hold the magnitudes.

    python branson_gb300/csrc/gen_fixmath_tables.py > branson_gb300/csrc/bgs_fixmath_tables.h
"""
from decimal import Decimal, getcontext

import mpmath as mp

getcontext().prec = 80
N = 1024
LN2 = Decimal(2).ln()


def rnd(x: Decimal) -> int:
    return int(x.to_integral_value(rounding="ROUND_HALF_EVEN"))


def hi_lo(v: int):
    return v >> 64, v & ((1 << 64) - 1)


def remez(f, n, lo, hi, iters=25, grid=2000):
    """Coefficients c_0..c_n of the polynomial minimising max |y (f(y) - p(y))|
    on [lo, hi] (Remez exchange on a grid)."""
    w = lambda y: y
    pts = [lo + (hi - lo) * (1 - mp.cos(mp.pi * i / (n + 1))) / 2 for i in range(n + 2)]
    c = None
    for _ in range(iters):
        A = mp.matrix(n + 2, n + 2)
        b = mp.matrix(n + 2, 1)
        for i, x in enumerate(pts):
            for k in range(n + 1):
                A[i, k] = x ** k
            A[i, n + 1] = (-1) ** i / w(x) if x != 0 else 0
            b[i] = f(x)
        sol = mp.lu_solve(A, b)
        c = [sol[k] for k in range(n + 1)]
        xs = [lo + (hi - lo) * i / grid for i in range(grid + 1)]
        es = [w(x) * (f(x) - sum(c[k] * x ** k for k in range(n + 1))) for x in xs]
        ext = [(xs[i], es[i]) for i in range(grid + 1)
               if i in (0, grid) or (abs(es[i]) >= abs(es[i - 1]) and abs(es[i]) >= abs(es[i + 1]))]
        alt = []
        for x, e in ext:
            if alt and mp.sign(e) == mp.sign(alt[-1][1]):
                if abs(e) > abs(alt[-1][1]):
                    alt[-1] = (x, e)
            else:
                alt.append((x, e))
        while len(alt) > n + 2:
            alt.pop(0 if abs(alt[0][1]) < abs(alt[-1][1]) else -1)
        if len(alt) < n + 2:
            break
        pts = [x for x, _ in alt]
    return c


def sincos_coefficients():
    mp.mp.dps = 60
    Y = (mp.pi / 4) ** 2
    B = lambda y: mp.mpf(1) / 6 if y == 0 else (1 - mp.sin(mp.sqrt(y)) / mp.sqrt(y)) / y
    C = lambda y: mp.mpf(1) / 2 if y == 0 else (1 - mp.cos(mp.sqrt(y))) / y
    out = []
    for f, n in ((B, 6), (C, 7)):
        c = remez(f, n, mp.mpf(0), Y)
        assert all(mp.sign(c[k]) == (-1) ** k for k in range(n + 1)), "coefficients must alternate"
        out.append([int(mp.nint(abs(ck) * mp.mpf(2) ** 64)) for ck in c])
    return out


def main():
    invf = [0] + [rnd(Decimal(2) ** 64 / (1 + Decimal(j) / N)) for j in range(1, N)]
    lnf = [rnd((1 + Decimal(j) / N).ln() * Decimal(2) ** 120) for j in range(N)]
    exp2 = [rnd(Decimal(2) ** (Decimal(63) - Decimal(j) / N)) for j in range(N)]
    ln2_120 = rnd(LN2 * Decimal(2) ** 120)
    ln2_1024_96 = rnd(LN2 / N * Decimal(2) ** 96)
    k = rnd(Decimal(N) / LN2 * Decimal(2) ** 32)
    assert all(0 < v < 2 ** 64 for v in invf[1:]) and all(0 < v <= 2 ** 63 for v in exp2)
    out = ["// Generated by gen_fixmath_tables.py (decimal, 80 digits); do not edit.",
           "#pragma once", "#include <cstdint>", "", "namespace bgs {", "namespace fixtab {",
           f"constexpr int kBins = {N};",
           "constexpr uint64_t kLn2_120_hi = 0x%016xULL, kLn2_120_lo = 0x%016xULL;" % hi_lo(ln2_120),
           "constexpr uint64_t kLn2_1024_96_hi = 0x%016xULL, kLn2_1024_96_lo = 0x%016xULL;" % hi_lo(ln2_1024_96),
           "constexpr uint64_t kInvLn2_1024_q32 = 0x%016xULL;" % k, ""]

    def table(name, vals, per=4):
        lines = [f"#define BGS_{name}_INIT \\"]
        for i in range(0, len(vals), per):
            chunk = ", ".join("0x%016xULL" % v for v in vals[i:i + per])
            lines.append(f"  {chunk}, \\")
        lines.append("")
        return lines

    out += table("LOG_INVF", invf)
    lnf_words = []
    for v in lnf:
        h, l = hi_lo(v)
        lnf_words += [h, l]
    out += table("LOG_LNF", lnf_words)
    out += table("EXP2_NEG", exp2)
    # sin/cos: 2/pi * 2^128, pi/2 * 2^62, minimax coefficient magnitudes in Q64
    pi = Decimal("3.14159265358979323846264338327950288419716939937510582097494459230781640628620899862803482534211706798214808651")
    two_pi = rnd(2 / pi * Decimal(2) ** 128)
    out += ["constexpr uint64_t kTwoOverPi_128_hi = 0x%016xULL, kTwoOverPi_128_lo = 0x%016xULL;" % hi_lo(two_pi),
            "constexpr uint64_t kPiOver2_q62 = 0x%016xULL;" % rnd(pi / 2 * Decimal(2) ** 62), ""]
    sin_c, cos_c = sincos_coefficients()
    out += ["constexpr int kSinTerms = %d, kCosTerms = %d;" % (len(sin_c), len(cos_c)), ""]
    out += table("SIN_COEF", sin_c, per=2)
    out += table("COS_COEF", cos_c, per=2)
    out += ["}  // namespace fixtab", "}  // namespace bgs", ""]
    print("\n".join(out))


if __name__ == "__main__":
    main()
