// Test shim: exposes the integer log/exp of branson_gb300/csrc/bgs_fixmath.cuh
// compiled for the host, next to quad-precision and libm references.
#include <cmath>
#include <cstdint>
#include <quadmath.h>

#include "bgs_fixmath.cuh"

extern "C" {
double fix_neg_log_u53(uint64_t m) { return bgs::fix::neg_log_u53(m); }
double fix_exp_neg(double t) { return bgs::fix::exp_neg(t); }
double quad_neg_log_u53(uint64_t m) {
  __float128 u = (__float128)m / (__float128)9007199254740992.0;
  return (double)(-logq(u));
}
double quad_exp_neg(double t) { return (double)expq(-(__float128)t); }
double libm_neg_log_u53(uint64_t m) { return -std::log((double)m * (1.0 / 9007199254740992.0)); }
double libm_exp_neg(double t) { return std::exp(-t); }
}
extern "C" {
void fix_sincos(double phi, double *s, double *c) { bgs::fix::sincos_phi(phi, s, c); }
void quad_sincos(double phi, double *s, double *c) {
  *s = (double)sinq((__float128)phi);
  *c = (double)cosq((__float128)phi);
}
void libm_sincos(double phi, double *s, double *c) {
  *s = std::sin(phi);
  *c = std::cos(phi);
}
}
extern "C" {
double fix_sqrt(double x) { return bgs::fix::sqrt_rn(x); }
}
