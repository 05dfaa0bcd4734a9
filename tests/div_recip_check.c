/* Division by a stored reciprocal, as the transport kernels do it
 * (div_recip in branson_gb300/csrc/bgs_physics.cuh): y = RN(1/b), q0 =
 * RN(a*y), r = fma(-q0, b, a), q = fma(r, y, q0).  Checks q == a/b bit for
 * bit on n random operand pairs of the kernels' kinds (face gap over a
 * direction cosine, -log(u) over an opacity) plus divisors with long runs of
 * ones or zeros in the mantissa.  Exit status 1 on any mismatch. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t st[2] = {0x9E3779B97F4A7C15ULL, 0xD1B54A32D192ED03ULL};
static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t next(void) {
  uint64_t s0 = st[0], s1 = st[1], r = s0 + s1;
  s1 ^= s0;
  st[0] = rotl(s0, 24) ^ s1 ^ (s1 << 16);
  st[1] = rotl(s1, 37);
  return r;
}
static double u01(void) { return (double)((next() >> 11) | 1) * 0x1p-53; }

int main(int argc, char **argv) {
  const long n = argc > 1 ? atol(argv[1]) : 10000000L;
  long bad = 0;
  for (long i = 0; i < n; ++i) {
    double a, b;
    switch (i % 3) {
      case 0: a = (u01() - 0.5) * 2.0; b = (u01() - 0.5) * 2.0; break;
      case 1: a = -log(u01()); b = exp((u01() - 0.5) * 20.0); break;
      default: {
        uint64_t mb = 0x3FF0000000000000ULL | (next() & 0x000FFFFFFFFFFFFFULL);
        const int k = (int)(next() % 52);
        if (next() & 1) mb |= (1ULL << k) - 1; else mb &= ~((1ULL << k) - 1);
        memcpy(&b, &mb, sizeof b);
        b = ldexp(b, (int)(next() % 40) - 20);
        if (next() & 1) b = -b;
        a = ldexp(u01() + 1.0, (int)(next() % 40) - 20);
      }
    }
    const double y = 1.0 / b;
    const double q0 = a * y;
    const double r = fma(-q0, b, a);
    const double q = fma(r, y, q0);
    const double t = a / b;
    if (memcmp(&q, &t, sizeof q) != 0) {
      if (bad < 5) printf("mismatch: %a / %a = %a, got %a\n", a, b, t, q);
      ++bad;
    }
  }
  printf("%ld pairs, %ld mismatches\n", n, bad);
  return bad != 0;
}
