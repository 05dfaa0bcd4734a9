// Integer fixed-point evaluation of the transcendental functions on the
// transport hot path, rounded once to IEEE double.
//
// GB300 executes FP64 at 2 lanes/clock/SM, while 32-bit integer arithmetic
// issues at up to 64 lanes/clock/SM.  These functions evaluate log and exp
// with ~62-63 significant bits using only 64/128-bit integer arithmetic and
// round the result to nearest, so they take the integer pipes instead of
// the FP64 pipe, and their results are the correctly rounded doubles except
// when the exact value lies within about 2^-9 ulp of a rounding midpoint.
//
// Methods (published, restated here in fixed point):
//   log: P. T. P. Tang, "Table-driven implementation of the logarithm
//        function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990:
//        x = F_j (1 + r) with F_j = 1 + j/1024, ln(1+r) by its Taylor series;
//        near u = 1 the series of -ln(1 - v) in the exact v = 1 - u.
//   exp: P. T. P. Tang, "Table-driven implementation of the exponential
//        function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989:
//        tau = (32*q + j) ln2/1024 + s, exp(-tau) = 2^-q 2^(-j/1024) e^(-s),
//        e^(-s) by its Taylor series.
//   sin/cos: Cody-Waite style reduction by pi/2 with a 128-bit 2/pi, octant
//        symmetry, minimax polynomials on [0, pi/4] (Remez exchange, in
//        gen_fixmath_tables.py).
// Tables (bgs_fixmath_tables.h) are generated from Python's decimal module.
// The same source compiles for the host (tests compare it against quad
// precision and glibc) and for the device.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "bgs_fixmath_tables.h"

#if defined(__CUDACC__)
// every routine inlined into its caller: calls (argument moves, saved
// registers, the return) measured slower than the larger loop body
#define BGS_HD __host__ __device__ __forceinline__
#else
#define BGS_HD inline
#endif

namespace bgs {
namespace fix {

typedef unsigned __int128 u128;

#if defined(__CUDACC__)
__device__ const uint64_t d_log_invf[fixtab::kBins] = {BGS_LOG_INVF_INIT};
__device__ const uint64_t d_log_lnf[2 * fixtab::kBins] = {BGS_LOG_LNF_INIT};
__device__ const uint64_t d_exp2_neg[fixtab::kBins] = {BGS_EXP2_NEG_INIT};
#endif
static const uint64_t h_log_invf[fixtab::kBins] = {BGS_LOG_INVF_INIT};
static const uint64_t h_log_lnf[2 * fixtab::kBins] = {BGS_LOG_LNF_INIT};
static const uint64_t h_exp2_neg[fixtab::kBins] = {BGS_EXP2_NEG_INIT};

BGS_HD uint64_t log_invf(uint32_t j) {
#if defined(__CUDA_ARCH__)
  return __ldg(&d_log_invf[j]);
#else
  return h_log_invf[j];
#endif
}
BGS_HD u128 log_lnf(uint32_t j) {
#if defined(__CUDA_ARCH__)
  const uint64_t hi = __ldg(&d_log_lnf[2 * j]), lo = __ldg(&d_log_lnf[2 * j + 1]);
#else
  const uint64_t hi = h_log_lnf[2 * j], lo = h_log_lnf[2 * j + 1];
#endif
  return ((u128)hi << 64) | lo;
}
BGS_HD uint64_t exp2_neg(uint32_t j) {
#if defined(__CUDA_ARCH__)
  return __ldg(&d_exp2_neg[j]);
#else
  return h_exp2_neg[j];
#endif
}

BGS_HD uint64_t mulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((u128)a * b) >> 64);
#endif
}

// mulhi(y, b) for b < 2^32 from the high word of y alone: floor(y_hi b / 2^32)
// is mulhi(y, b) or one below it (one 32 x 32 -> 64-bit product)
BGS_HD uint64_t mulhi_b32(uint64_t y, uint64_t b) {
  return ((y >> 32) * (uint64_t)(uint32_t)b) >> 32;
}

// the high 64 bits of a * b from the high words alone: below mulhi(a, b) by
// less than 2^33, for the innermost series terms, whose error is scaled down
// by the higher powers of the small argument
BGS_HD uint64_t mulhi_hh(uint64_t a, uint64_t b) { return (a >> 32) * (b >> 32); }

BGS_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

BGS_HD double bits_to_double(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
#endif
}

BGS_HD uint64_t double_to_bits(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t b;
  std::memcpy(&b, &d, sizeof b);
  return b;
#endif
}

// The positive value W * 2^-scale rounded to the nearest double, for a W
// whose top set bit is at 117 or above, so the mantissa and the rounding
// position both lie in the high word (the sine and exp results): one 64-bit
// shift and compare.  Values below the normal range flush to zero (callers
// never produce them on the paths that use this).
BGS_HD double round_u128_high(u128 W, int scale) {
  const uint64_t hi = (uint64_t)(W >> 64), lo = (uint64_t)W;
  const int ph = 63 - clz64(hi);  // top set bit of W is ph + 64
  const int sh = ph - 52;         // bits of hi below the mantissa, >= 1
  uint64_t mant = hi >> sh;
  const uint64_t rem = hi & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
  const bool up = rem > half || (rem == half && (lo != 0 || (mant & 1)));
  int e2 = ph + 64 - scale;  // value = mant * 2^(e2 - 52)
  mant += up ? 1ULL : 0ULL;  // data-dependent: no branch, so no split warp
  const int carry = (int)(mant >> 53);
  mant >>= carry;
  e2 += carry;
  const int be = e2 + 1023;
  if (be <= 0) return 0.0;
  return bits_to_double(((uint64_t)be << 52) | (mant & 0x000FFFFFFFFFFFFFULL));
}

// The same for any W with a nonzero high word (the log results): W is first
// normalised so its top bit is bit 127 (a funnel shift by clz, branch-free),
// then the mantissa and rounding bit sit at fixed positions of the high
// word, as in round_u128_high.  The log's results span both sides of the
// word boundary of the generic shift, which made lanes of a warp diverge.
BGS_HD double round_u128_norm(u128 W, int scale) {
  const uint64_t hi = (uint64_t)(W >> 64), lo = (uint64_t)W;
  const int lz = clz64(hi);                                   // < 64: hi != 0
  const uint64_t nh = (hi << lz) | (lz ? lo >> (64 - lz) : 0ULL);
  const uint64_t nl = lo << lz;
  uint64_t mant = nh >> 11;
  const uint64_t rem = nh & 0x7FFULL;
  const bool up = rem > 0x400ULL || (rem == 0x400ULL && (nl != 0 || (mant & 1)));
  int e2 = 127 - lz - scale;  // value = mant * 2^(e2 - 52)
  mant += up ? 1ULL : 0ULL;  // data-dependent: no branch, so no split warp
  const int carry = (int)(mant >> 53);
  mant >>= carry;
  e2 += carry;
  const int be = e2 + 1023;
  if (be <= 0) return 0.0;
  return bits_to_double(((uint64_t)be << 52) | (mant & 0x000FFFFFFFFFFFFFULL));
}

// v * 2^-64 for v in [2^63, 2^64) rounded to the nearest double (the cosine
// on [0, pi/4], as 1 - cb)
BGS_HD double round_unit_q64(uint64_t v) {
  uint64_t mant = v >> 11;
  const uint64_t rem = v & 0x7FFULL;
  mant += (rem > 0x400ULL || (rem == 0x400ULL && (mant & 1))) ? 1ULL : 0ULL;
  if (mant >> 53) return 1.0;  // rounded up to the value 1
  return bits_to_double((1022ULL << 52) | (mant & 0x000FFFFFFFFFFFFFULL));
}

// -ln(u) for the RNG draw u = m * 2^-53 (u01fixedpt: m odd, 1 <= m < 2^53).
// The result is the value -log(u) rounds to (the upstream distance to
// collision numerator, history_based_transport.h:62-63).
BGS_HD double neg_log_u53(uint64_t m) {
  const uint64_t n = (1ULL << 53) - m;  // v = 1 - u = n * 2^-53, exact
  if (n < (1ULL << 42)) {
    // v < 2^-11: -ln(1-v) = v (1 + v/2 + v^2/3 + v^3/4 + v^4/5 + v^5/6), V = v*2^64
    const uint64_t V = n << 11;
    uint64_t t = 0x2AAAAAAAAAAAAAABULL;           // 1/6
    t = 0x3333333333333333ULL + mulhi(V, t);       // 1/5
    t = 0x4000000000000000ULL + mulhi(V, t);       // 1/4
    t = 0x5555555555555555ULL + mulhi(V, t);       // 1/3
    t = 0x8000000000000000ULL + mulhi(V, t);       // 1/2
    const uint64_t T = mulhi(V, t);                // (S - 1) * 2^64
    const u128 L = ((u128)V << 64) + (u128)V * T;  // L * 2^128
    return round_u128_norm(L, 128);
  }
  const int e = 63 - clz64(m);                     // m in [2^e, 2^(e+1))
  const uint64_t k = 53 - e;                       // u = x 2^-k, x in [1, 2)
  const uint64_t X = m << (63 - e);                // x * 2^63
  const uint32_t j = (uint32_t)(X >> 53) & 1023u;  // F_j = 1 + j/1024
  const uint64_t f = X & ((1ULL << 53) - 1);       // (x - F_j) * 2^63
  // R = r * 2^74 with r = (x - F_j)/F_j < 2^-10
  const uint64_t R = j ? mulhi(f << 11, log_invf(j)) : (f << 11);
  // ln(1+r) = r - r^2 (1/2 - r(1/3 - r(1/4 - r(1/5 - r(1/6 - r/7)))))
  uint64_t b = 0x2AAAAAAAAAAAAAABULL - (mulhi_hh(R, 0x2492492492492492ULL) >> 10);  // 1/6 - r/7
  b = 0x3333333333333333ULL - (mulhi_hh(R, b) >> 10);                                // 1/5 - ...
  b = 0x4000000000000000ULL - (mulhi(R, b) >> 10);                                // 1/4 - ...
  b = 0x5555555555555555ULL - (mulhi(R, b) >> 10);                                // 1/3 - ...
  b = 0x8000000000000000ULL - (mulhi(R, b) >> 10);                                // 1/2 - ...
  const uint64_t R2 = (uint64_t)(((u128)R * R) >> 64);                           // r^2 * 2^84
  const uint64_t Q = mulhi(R2, b);                                                // r^2 b * 2^84
  // L = k ln2 - ln F_j - r + r^2 b, scaled by 2^120
  const u128 ln2 = ((u128)fixtab::kLn2_120_hi << 64) | fixtab::kLn2_120_lo;
  u128 W = ln2 * k;
  W -= log_lnf(j);
  W -= (u128)R << 46;
  W += (u128)Q << 36;
  return round_u128_norm(W, 120);  // W >= 2^108: the result is above 2^-12
}

// exp(-tau) for tau >= 0: the factor exp(-sigma_a*f*d) of the implicit-capture
// weight decay (history_based_transport.h:74).  tau above 700 (result below
// 1e-304) returns the CUDA/libm value instead of the fixed-point path.
BGS_HD double exp_neg(double tau) {
  const uint64_t tb = double_to_bits(tau);
  const int te = (int)((tb >> 52) & 0x7FF);
  if (te == 0) return 1.0;  // tau = 0 (or subnormal: exp rounds to 1)
  // tau > 700 (or a NaN) by the bit pattern: 700.0 is 0x4085E00000000000
  if (tb > 0x4085E00000000000ULL) return tau == tau ? exp(-tau) : tau;
  // T = tau * 2^96 as a 128-bit integer (truncating below 2^-96)
  const uint64_t tm = (tb & 0x000FFFFFFFFFFFFFULL) | 0x0010000000000000ULL;
  const int sh = te - 1075 + 96;  // tau = tm * 2^(te-1075)
  u128 T;
  if (sh >= 0) T = (u128)tm << sh;
  else T = sh > -64 ? (u128)(tm >> (-sh)) : (u128)0;
  // N ~ floor(tau * 1024/ln2) from the top bits, then corrected exactly.
  // The estimate (tau to 2^-32, a 43-bit multiplier) is off by less than
  // 4e-7 before the floor, so the corrections almost never run (a warp's
  // lanes seldom diverge there)
  const uint64_t A = (uint64_t)(T >> 64);  // tau * 2^32
  uint64_t N = mulhi(A, fixtab::kInvLn2_1024_q32);
  const u128 L = ((u128)fixtab::kLn2_1024_96_hi << 64) | fixtab::kLn2_1024_96_lo;
  u128 NL = L * N;
  // N is then the floor or one off it either way: one predicated step each
  // way (no loop; the upward one runs for about a tenth of the arguments)
  if (NL > T) { --N; NL -= L; }
  u128 S = T - NL;
  if (S >= L) { ++N; S -= L; }
  // s * 2^73 (s < ln2/1024 < 2^-10.5)
  const uint64_t s73 = (uint64_t)(S >> 23);
  // e^-s = 1 - s (1 - s (1/2 - s (1/6 - s (1/24 - s/120))))
  uint64_t b = 0x0AAAAAAAAAAAAAABULL - (mulhi_hh(s73, 0x0222222222222222ULL) >> 9);  // 1/24 - s/120
  b = 0x2AAAAAAAAAAAAAABULL - (mulhi(s73, b) >> 9);                                // 1/6 - ...
  b = 0x8000000000000000ULL - (mulhi(s73, b) >> 9);                                // 1/2 - ...
  b = (uint64_t)0 - (mulhi(s73, b) >> 9);                                          // 1 - s(...) (mod 2^64)
  // P = 1 - s*b: b represents 1 - small (b == 0 means exactly 1)
  const uint64_t sb = b ? (mulhi(s73, b) >> 9) : (s73 >> 9);
  const uint32_t j = (uint32_t)(N & 1023u);
  const uint64_t q = N >> 10;
  const uint64_t E = exp2_neg(j);  // 2^(63 - j/1024)
  u128 W;
  if (sb == 0) {
    W = (u128)E << 64;
  } else {
    const uint64_t P = (uint64_t)0 - sb;  // (1 - s b) * 2^64
    W = (u128)E * P;
  }
  return round_u128_high(W, 127 + (int)q);  // W in (2^125, 2^127]
}


// sin and cos of 0 < phi < 8, the scattering azimuth phi = 2 pi u
// (get_uniform_angle, sampling_functions.h:63-67).  phi * 2/pi is formed
// exactly enough in Q124 (128-bit constant), the quadrant and octant are
// taken off by symmetry, and sin/cos of the remaining angle in [0, pi/4] are
// polynomials in fixed point; the small one of the pair is always a
// sine computed relative to its argument, so tiny results keep full
// precision.  Results are rounded to nearest.
struct SinCos {
  double s, c;
};

BGS_HD SinCos sincos_phi_v(double phi) {
  constexpr uint64_t kS[fixtab::kSinTerms] = {BGS_SIN_COEF_INIT};
  constexpr uint64_t kCo[fixtab::kCosTerms] = {BGS_COS_COEF_INIT};
  const uint64_t pb = double_to_bits(phi);
  const int be = (int)((pb >> 52) & 0x7FF);
  // 0 < phi < 8 by the bit pattern (8.0 is 0x4020000000000000; a set sign
  // bit, a NaN or a zero/subnormal exponent all fall outside)
  if (be == 0 || pb >= 0x4020000000000000ULL) {
    SinCos r;
#if defined(__CUDA_ARCH__)
    sincos(phi, &r.s, &r.c);
#else
    r.s = std::sin(phi);
    r.c = std::cos(phi);
#endif
    return r;
  }
  const int e = be - 1023;  // phi = M * 2^(e - 52), e <= 2
  const uint64_t M = (pb & 0x000FFFFFFFFFFFFFULL) | 0x0010000000000000ULL;
  // M * (2/pi * 2^128) as three words w2:w1:w0
  const u128 plo = (u128)M * fixtab::kTwoOverPi_128_lo;
  const u128 phi_ = (u128)M * fixtab::kTwoOverPi_128_hi;
  const uint64_t w0 = (uint64_t)plo;
  const u128 mid = (plo >> 64) + (uint64_t)phi_;
  const uint64_t w1 = (uint64_t)mid;
  const uint64_t w2 = (uint64_t)(phi_ >> 64) + (uint64_t)(mid >> 64);
  // Y = phi * 2/pi * 2^124 = (w2:w1:w0) >> (56 - e)
  const int sh = 56 - e;  // 54 .. 107 for the phi this is called with
  u128 Y;
  if (sh < 64) {
    Y = ((u128)w2 << (128 - sh)) | ((((u128)w1 << 64) | w0) >> sh);
  } else if (sh < 128) {
    Y = (((u128)w2 << 64) | w1) >> (sh - 64);
  } else {
    Y = (u128)(w2 >> (sh - 128));
  }
  (void)w0;
  const unsigned quad = (unsigned)(Y >> 124) & 3u;
  const u128 mask = (((u128)1) << 124) - 1;
  u128 t = Y & mask;
  const u128 half = ((u128)1) << 123;
  const bool swap = t > half;
  const u128 x = swap ? ((((u128)1) << 124) - t) : t;  // x in (0, 1/2], Q124
  double sv, cv;  // sin and cos of x*pi/2
  if (x == 0) {
    sv = 0.0;
    cv = 1.0;
  } else {
    const uint64_t xh = (uint64_t)(x >> 64), xl = (uint64_t)x;
    const int lz = xh ? clz64(xh) : 64 + clz64(xl);
    const u128 xn = x << lz;
    const uint64_t Xn = (uint64_t)(xn >> 64);               // x = Xn * 2^(-60-lz)
    const uint64_t Tm = mulhi(Xn, fixtab::kPiOver2_q62);     // theta = Tm * 2^(-58-lz)
    const uint64_t th64 = lz >= 6 ? (lz - 6 >= 64 ? 0 : Tm >> (lz - 6)) : Tm << (6 - lz);  // theta * 2^64
    const uint64_t y = mulhi(th64, th64);                    // theta^2 * 2^64
    // the running term never exceeds the coefficient it started from, so
    // where that coefficient is below 2^32 one 32 x 32-bit product serves
    // (the two innermost steps of each series)
    uint64_t b = kS[fixtab::kSinTerms - 1];
#pragma unroll
    for (int k = fixtab::kSinTerms - 2; k >= 0; --k)  // ~1/3! - y(1/5! - ...)
      b = kS[k] - (kS[k + 1] < (1ULL << 32) ? mulhi_b32(y, b) : mulhi(y, b));
    const uint64_t sb = mulhi(y, b);                          // y * b
    const u128 Ws = sb ? (u128)Tm * ((uint64_t)0 - sb) : ((u128)Tm << 64);
    sv = round_u128_high(Ws, 122 + lz);  // Ws in [2^124, 2^127)
    uint64_t c = kCo[fixtab::kCosTerms - 1];
#pragma unroll
    for (int k = fixtab::kCosTerms - 2; k >= 0; --k)  // ~1/2! - y(1/4! - ...)
      c = kCo[k] - (kCo[k + 1] < (1ULL << 32) ? mulhi_b32(y, c) : mulhi(y, c));
    const uint64_t cb = mulhi(y, c);
    cv = cb ? round_unit_q64((uint64_t)0 - cb) : 1.0;  // cos >= cos(pi/4): 2^64 - cb >= 2^63
  }
  const double so = swap ? cv : sv;  // sin, cos of (t*pi/2)
  const double co = swap ? sv : cv;
  // quadrant q: sin = (so, co, -so, -co)[q], cos = (co, -so, -co, so)[q], by
  // selects and sign-bit flips (lanes of a warp hold different quadrants)
  const uint64_t sgn = 0x8000000000000000ULL;
  const uint64_t sb = double_to_bits((quad & 1u) ? co : so) ^ ((quad & 2u) ? sgn : 0ULL);
  const uint64_t cb = double_to_bits((quad & 1u) ? so : co) ^ (((quad + 1u) & 2u) ? sgn : 0ULL);
  return {bits_to_double(sb), bits_to_double(cb)};
}

BGS_HD void sincos_phi(double phi, double *s_out, double *c_out) {
  const SinCos r = sincos_phi_v(phi);
  *s_out = r.s;
  *c_out = r.c;
}


// ------------------------------------------------------------------------
// Correctly rounded square root in integer arithmetic.  It reproduces the
// IEEE-754 round-to-nearest-even result exactly (checked bit for bit against
// the hardware FP64 square root) for positive normal operands; anything else
// goes to the FP64 operation.

// floor(f * 2^shift) for a positive normal float, from its bits, saturating
// at 2^64 - 1 (no floating-point conversion instruction needed)
BGS_HD uint64_t float_to_fixed(float f, int shift) {
  uint32_t b;
#if defined(__CUDA_ARCH__)
  b = __float_as_uint(f);
#else
  std::memcpy(&b, &f, sizeof b);
#endif
  const int e = (int)((b >> 23) & 0xFF) - 150 + shift;  // f = m * 2^(exp-150)
  const uint64_t m = (b & 0x7FFFFFu) | 0x800000u;
  if (e > 40) return ~0ULL;
  if (e >= 0) return m << e;
  return e > -64 ? m >> (-e) : 0ULL;
}

BGS_HD float u64_to_float_approx(uint64_t x) {  // x < 2^24, exact
#if defined(__CUDA_ARCH__)
  return __uint2float_rn((unsigned)x);
#else
  return (float)x;
#endif
}

// sqrt(x) rounded to nearest for normal x > 0: 1/sqrt by Newton in fixed
// point from a float seed, the root w*r, then the exact floor and rounding
// checked with 128-bit integer squares.
BGS_HD double sqrt_rn(double x) {
  const uint64_t xb = double_to_bits(x);
  const int ex = (int)((xb >> 52) & 0x7FF);
  if (ex == 0 || ex == 0x7FF || (xb >> 63)) {
#if defined(__CUDA_ARCH__)
    return __dsqrt_rn(x);
#else
    return std::sqrt(x);
#endif
  }
  uint64_t M = (xb & 0x000FFFFFFFFFFFFFULL) | 0x0010000000000000ULL;
  int e = ex - 1075;  // x = M * 2^e
  const int odd = e & 1;  // e even, 2^52 <= M < 2^54 (a shift, not a branch)
  M <<= odd;
  e -= odd;
  const u128 N = (u128)M << 52;  // sqrt(x) = sqrt(N) * 2^((e-52)/2), sqrt(N) in [2^52, 2^53)
  const uint64_t W = M << 10;    // w = M/2^54 in [1/4, 1), Q64
  const float wf = u64_to_float_approx(M >> 30) * (1.0f / 16777216.0f);
#if defined(__CUDA_ARCH__)
  const float rsf = rsqrtf(wf);
#else
  const float rsf = 1.0f / std::sqrt(wf);
#endif
  uint64_t R = float_to_fixed(rsf, 62);  // r = 1/sqrt(w) in (1, 2], Q62
  // two Newton steps r <- r (3 - w r^2)/2: 23 -> ~46 -> ~62 bits
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const uint64_t R2 = (uint64_t)(((u128)R * R) >> 64);   // r^2, Q60
    const uint64_t wr2 = mulhi(W, R2);                       // w r^2, Q60 (~2^60)
    const uint64_t t = 3ULL * (1ULL << 60) - wr2;           // (3 - w r^2), Q60
    R = (uint64_t)(((u128)R * t) >> 61);                     // r (3 - w r^2)/2, Q62
  }
  uint64_t y = mulhi(W, R) >> 9;  // sqrt(w) * 2^53 ~ floor(sqrt(N))
  // exact floor(sqrt(N)) from one square: (y -+ 1)^2 = y^2 -+ (2y -+ 1)
  u128 sq = (u128)y * y;
#pragma unroll 1
  for (int it = 0; it < 8 && sq > N; ++it) {
    sq -= (u128)(2 * y - 1);
    --y;
  }
#pragma unroll 1
  for (int it = 0; it < 8 && sq + (u128)(2 * y + 1) <= N; ++it) {
    sq += (u128)(2 * y + 1);
    ++y;
  }
  // nearest: N - y^2 > y  <=>  sqrt(N) > y + 1/2 (no exact ties)
  y += (N - sq > (u128)y) ? 1ULL : 0ULL;
  int eo = (e - 52) / 2 + 52;  // value = y * 2^(eo - 52)
  if (y >> 53) { y >>= 1; ++eo; }
  return bits_to_double(((uint64_t)(eo + 1023) << 52) | (y & 0x000FFFFFFFFFFFFFULL));
}

}  // namespace fix
}  // namespace bgs
