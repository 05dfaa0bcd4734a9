// TEST INFRASTRUCTURE ONLY.  The GPU path's integer fixed-point -log(u),
// exp(-t) and sin/cos of the azimuth (branson_gb300/csrc/bgs_fixmath.cuh),
// compiled for the host and linked into the oracle's BO_GPU_MATH build (the
// diagnostic twin described in branson_oracle.c).  The default oracle build
// does not use this file: it calls the host libm, as the upstream code does.
#include <cstdint>

#include "bgs_fixmath.cuh"

extern "C" {
double bo_gm_neg_log_u53(uint64_t m) { return bgs::fix::neg_log_u53(m); }
double bo_gm_exp_neg(double t) { return bgs::fix::exp_neg(t); }
void bo_gm_sincos_phi(double phi, double *s, double *c) { bgs::fix::sincos_phi(phi, s, c); }
}
