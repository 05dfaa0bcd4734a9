"""Generate bgs_fixmath_tables.h: fixed-point tables for the integer log/exp.

Values are computed with Python's decimal module at 80 significant digits
and rounded to nearest:
  LOG_INVF[j] = 2^64 / F_j            F_j = 1 + j/1024, j = 1..1023 (j = 0 unused)
  LOG_LNF[j]  = ln(F_j) * 2^120       as (hi, lo) 64-bit words
  EXP2_NEG[j] = 2^(63 - j/1024)       j = 0..1023
  LN2_120     = ln 2 * 2^120          (hi, lo)
  LN2_1024_96 = ln 2 / 1024 * 2^96    (hi, lo)
  K_1024_LN2  = 1024/ln 2 * 2^12      (estimate multiplier for the exp reduction)
  2/pi * 2^128, pi/2 * 2^62, and 1/(2k+1)!, 1/(2k)! (k = 1..10) in Q64 for sin/cos

    python branson_gb300/csrc/gen_fixmath_tables.py > branson_gb300/csrc/bgs_fixmath_tables.h
"""
from decimal import Decimal, getcontext

getcontext().prec = 80
N = 1024
LN2 = Decimal(2).ln()


def rnd(x: Decimal) -> int:
    return int(x.to_integral_value(rounding="ROUND_HALF_EVEN"))


def hi_lo(v: int):
    return v >> 64, v & ((1 << 64) - 1)


def main():
    invf = [0] + [rnd(Decimal(2) ** 64 / (1 + Decimal(j) / N)) for j in range(1, N)]
    lnf = [rnd((1 + Decimal(j) / N).ln() * Decimal(2) ** 120) for j in range(N)]
    exp2 = [rnd(Decimal(2) ** (Decimal(63) - Decimal(j) / N)) for j in range(N)]
    ln2_120 = rnd(LN2 * Decimal(2) ** 120)
    ln2_1024_96 = rnd(LN2 / N * Decimal(2) ** 96)
    k = rnd(Decimal(N) / LN2 * Decimal(2) ** 12)
    assert all(0 < v < 2 ** 64 for v in invf[1:]) and all(0 < v <= 2 ** 63 for v in exp2)
    out = ["// Generated by gen_fixmath_tables.py (decimal, 80 digits); do not edit.",
           "#pragma once", "#include <cstdint>", "", "namespace bgs {", "namespace fixtab {",
           f"constexpr int kBins = {N};",
           "constexpr uint64_t kLn2_120_hi = 0x%016xULL, kLn2_120_lo = 0x%016xULL;" % hi_lo(ln2_120),
           "constexpr uint64_t kLn2_1024_96_hi = 0x%016xULL, kLn2_1024_96_lo = 0x%016xULL;" % hi_lo(ln2_1024_96),
           "constexpr uint64_t kInvLn2_1024_q12 = 0x%016xULL;" % k, ""]

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
    # sin/cos: 2/pi * 2^128, pi/2 * 2^62, Taylor coefficients 1/(2k+1)! and 1/(2k)! in Q64
    import math
    pi = Decimal("3.14159265358979323846264338327950288419716939937510582097494459230781640628620899862803482534211706798214808651")
    two_pi = rnd(2 / pi * Decimal(2) ** 128)
    out += ["constexpr uint64_t kTwoOverPi_128_hi = 0x%016xULL, kTwoOverPi_128_lo = 0x%016xULL;" % hi_lo(two_pi),
            "constexpr uint64_t kPiOver2_q62 = 0x%016xULL;" % rnd(pi / 2 * Decimal(2) ** 62), ""]
    out += table("SIN_COEF", [rnd(Decimal(2) ** 64 / math.factorial(2 * k + 1)) for k in range(1, 11)], per=2)
    out += table("COS_COEF", [rnd(Decimal(2) ** 64 / math.factorial(2 * k)) for k in range(1, 11)], per=2)
    out += ["}  // namespace fixtab", "}  // namespace bgs", ""]
    print("\n".join(out))


if __name__ == "__main__":
    main()
