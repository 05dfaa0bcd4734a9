// Internal device data model and helpers of the GB300 replicated IMC step.
//
// Layout in HBM (one context):
//   mesh     : plane arrays x[ngx+1], y[ngy+1], z[ngz+1]; cell_region[n];
//              region table (n_regions x 8 doubles)
//   cells    : structure of arrays of doubles, one entry per cell
//              (T_e, T_r initial, T_s, op_a, op_s, f, emission/census/source E,
//              T_r diagnostic) plus the transport table XS[n] (32 B per cell)
//   tallies  : TallyCell[n] = 128-bit fixed-point absorbed energy and its
//              cutoff-kill part (32 B per cell), order-independent integer
//              sums; the track tally is formed from them per cell
//   photons  : two banks, each a structure of arrays sized to the capacity
//   counts   : per-cell photon counts and their exclusive prefix sums
//   diag     : one DeviceDiag (step scalars, flags)
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bgs {

// Constants namespace (constants.h:16-24)
constexpr double kPi = 3.1415926535897932384626433832795;
constexpr double kC = 299.792458;
constexpr double kA = 0.01372;
constexpr double kCutoff = 0.01;

enum : int { REFLECT = 0, VACUUM = 1, ELEMENT = 2, SOURCE = 3, PROCESSOR = 4 };
enum : uint8_t { EXIT = 0, PASS = 1, CENSUS = 2, SCATTER = 3, KILLED = 4, BOUND = 5 };

// device-side check bits (DeviceDiag::flags)
enum : uint32_t {
  FLAG_CAPACITY = 1u << 0,      // bank would overflow: no photons made
  FLAG_TALLY_RANGE = 1u << 1,   // a tally contribution outside the fixed-point range
  FLAG_SEGMENT_LIMIT = 1u << 2, // a history exceeded the segment limit and was killed
  FLAG_BAD_CELL = 1u << 3,      // a photon referenced a cell outside the mesh
  FLAG_NAN = 1u << 4,           // a non-finite tally contribution was dropped
  FLAG_BAD_COUNTS = 1u << 5,    // caller-supplied photon counts disagree with the cell energies
};

// Upper bound on loop trips of one history inside one step; a history that
// reaches it is ended as KILLED and FLAG_SEGMENT_LIMIT is raised.
constexpr uint32_t kMaxSegmentsPerHistory = 100000000u;

// Per-cell transport coefficients, derived each step from op_a, op_s, f.
// Each is formed with the exact expression transport_photon evaluates
// (history_based_transport.h:56-59, :74, :77, :97), so results are bitwise
// those of the upstream loop:
//   sig_eff  = (1 - f)*sigma_a + sigma_s   (effective scattering opacity)
//   neg_saf  = -sigma_a * f                (exponent rate, negated)
//   p_scat   = sigma_s / sig_eff           (physical-scatter probability)
//   inv_se   = RN(1/sig_eff) for the correctly rounded division
//              -log(u)/sig_eff by one multiply and two fma (div_recip in
//              bgs_physics.cuh); 0 if sig_eff is 0 or out of that range
// One entry is one 32-byte sector: a segment's table read is one sector.
// The track-length factor RN(1/(sigma_a f)), read once per cell per step
// when the tallies are converted, is in its own array (CellsDev::inv_saf).
struct __align__(32) CellXS {
  double sig_eff, neg_saf, p_scat, inv_se;
};

// 128-bit fixed-point tally cell: value = (hi*2^64 + lo) * 2^-scale_abs.
// abs is the absorbed energy (Cell_Tally::abs_E); dep is the part of it
// deposited by cutoff kills.  The track-length tally is formed per cell
// from the two: track_E = (abs - dep) / (sigma_a f), since sigma_a f is
// constant in a cell over a step and a kill deposit adds to abs_E only
// (history_based_transport.h:74-82); so a visit flushes one tally, and a
// kill a second one.
struct __align__(32) TallyCell {
  unsigned long long abs_lo, abs_hi, dep_lo, dep_hi;
};

// Photon bank: structure of arrays (photon.h:172-181 fields).
struct Bank {
  double *px, *py, *pz, *dx, *dy, *dz, *E, *E0, *life;
  uint32_t *cell, *group;
  uint8_t *desc, *stype;
  unsigned long long *stream, *ctr;
};

struct MeshDev {
  uint32_t ngx, ngy, ngz, n_groups;
  uint32_t n_cells, n_regions;
  // floor(2^64 / d) + 1 for d = ngx and ngx*ngy (0 for d = 1): a cell's
  // coordinates by multiplies instead of divisions (cell_coords)
  unsigned long long inv_ngx, inv_ngxy;
  const double *x, *y, *z;
  const uint32_t *region;
  const double *regions;  // n_regions x 8
  int bc[6];
  double T_source;
  // 1: one group and no physical scattering in any cell (every op_s zero),
  // so a scatter's effective-scatter test and group resample only advance
  // the RNG counter; the history kernel then runs a build without them
  uint32_t gray;
};

// the multiplier of MeshDev::inv_ngx / inv_ngxy for divisor d >= 1
inline unsigned long long div_multiplier(uint64_t d) {
  return d <= 1 ? 0ULL : (unsigned long long)(((unsigned __int128)1 << 64) / d) + 1ULL;
}

// n / d for n, d < 2^32 from M = floor(2^64/d) + 1: n M / 2^64 exceeds n/d
// by less than n / 2^64 < 2^-32 <= 1/d, which never carries past the next
// integer (the fraction of n/d is at most 1 - 1/d)
__device__ __forceinline__ uint32_t div_by_multiplier(uint32_t n, uint32_t d, unsigned long long M) {
  return d <= 1 ? n : (uint32_t)__umul64hi((unsigned long long)n, M);
}

// (i, j, k) of cell g = i + ngx (j + ngy k)
__device__ __forceinline__ void cell_coords(const MeshDev &m, uint32_t g, uint32_t &i, uint32_t &j, uint32_t &k) {
  const uint32_t q = div_by_multiplier(g, m.ngx, m.inv_ngx);  // j + ngy k
  k = div_by_multiplier(g, m.ngx * m.ngy, m.inv_ngxy);
  i = g - q * m.ngx;
  j = q - k * m.ngy;
}

struct CellsDev {
  double *T_e, *T_r, *T_s, *op_a, *op_s, *f, *em_E, *ce_E, *so_E, *T_r_diag;
  double *group_v;        // op_a * (1/(op_a*N)): one CDF step of sample_emission_group
  CellXS *xs;
  double *inv_saf;        // RN(1/(op_a f)): the track-length factor (the tally contribution
                          // absorbed/(sigma_a f) is formed as a product, within 1 ulp)
  TallyCell *tally;
  int8_t *source_face;    // Cell::get_source_face (cell.h:69-76), -1 if none
  uint32_t *n_em, *n_so, *n_ce;          // photons per cell
  unsigned long long *off_new, *off_ce;  // exclusive prefix sums (n+1 entries)
};

// Event-mode state: per-photon carried tallies and surface, the active list
// and the per-event queues (indices into the bank), with device counters.
struct EventState {
  double *thr_abs;             // per-cell-visit absorbed energy carried between stages
  uint8_t *surface;            // face crossed by a boundary event
  uint32_t *active, *next, *q_scatter, *q_boundary;
  unsigned int *n_active, *n_next, *n_scatter, *n_boundary;  // device counters
};

// Adjoint replay (bgs_adjoint.cu).  Per cell: w = dL/dE_abs of the cell,
// f2 = f^2 = d(sigma_a f)/d sigma_a, g2 = 1 - f^2 = d sigma_eff/d sigma_a, and
// inv_se = 1/sigma_eff (0 when sigma_eff is 0).
struct __align__(32) AdjCell {
  double w, f2, g2, inv_se;
};

// One problem of an adjoint replay launch (bgs_adjoint.cu): its mesh, the
// saved step (start states, transport table, adjoint coefficients), its
// gradient sums and their fixed-point range.
struct AdjProblem {
  MeshDev m;
  const CellXS *xs;
  const double *group_v;
  Bank t;                         // start states saved by the forward
  const AdjCell *cell;
  const double *src;              // f/sigma_a: d ln(emission weight)/d sigma_a per cell
  unsigned long long *grad;       // per cell (lo, hi): 128-bit two's-complement fixed point
  unsigned long long seed_hi;
  double visit_bound;             // |contribution of one visit| above this is a range error
  int scale;                      // fixed-point exponent of the gradient sums
};

// Scratch shared by all problems of a replay launch.
struct AdjShared {
  double *log_a, *log_b;          // per-thread visit logs, log_len entries each
  uint32_t *log_cell;
  uint32_t log_len;
  unsigned long long *long_list;  // work items (over all problems) with more visits than a log holds
  double *long_G;                 // their totals (second replay)
  unsigned int *n_long;
  unsigned long long *work;       // work-queue head
  uint32_t *flags;
};

// Scalars of one step kept on the device (so a step never waits for the host).
struct DeviceDiag {
  double total_photon_E, emission_E, census_cell_E, source_E, pre_mat_E;
  double census_E_in;                 // energy of the census carried into the step
  unsigned long long n_new, n_init_census, n_census_in, n_bank;
  unsigned long long n_census_out, n_segments;
  unsigned long long work_counter;    // transport work queue head
  unsigned long long census_counter;  // (unused by the scan path)
  unsigned long long sum_census[2], sum_exit[2], sum_abs[2];  // 128-bit fixed point
  double census_E, exit_E, absorbed_E, post_mat_E;
  int scale_abs;                      // fixed-point exponent of this step's energy sums
  uint32_t flags;
  uint32_t serial_needed;             // a photon count needed the serial energy sum
  uint32_t bad_counts_cell;           // 1 + a cell whose supplied photon counts disagreed (0: none)
};

// ------------------------------------------------------------------ RNG
// Threefry2x64-20 (Salmon et al., SC'11), key (stream, 0), counter
// (ctr, seed << 32): the generator RNG::generate_random_number draws from
// (RNG.h:262-285, threefry.h:190-293).
__device__ __forceinline__ unsigned long long rotl64(unsigned long long x, int r) {
  return (x << r) | (x >> (64 - r));
}

__device__ __forceinline__ unsigned long long threefry2x64_20_w0(unsigned long long c0,
                                                                 unsigned long long c1,
                                                                 unsigned long long k0) {
  const unsigned long long k2 = 0x1BD11BDAA9FC1A22ULL ^ k0;  // k1 = 0
  unsigned long long x0 = c0 + k0, x1 = c1;
#define BGS_MIX(R) { x0 += x1; x1 = rotl64(x1, R); x1 ^= x0; }
  BGS_MIX(16) BGS_MIX(42) BGS_MIX(12) BGS_MIX(31)
  x0 += 0;  x1 += k2 + 1ULL;   // injection 1: ks[1], ks[2] + 1
  BGS_MIX(16) BGS_MIX(32) BGS_MIX(24) BGS_MIX(21)
  x0 += k2; x1 += k0 + 2ULL;   // injection 2: ks[2], ks[0] + 2
  BGS_MIX(16) BGS_MIX(42) BGS_MIX(12) BGS_MIX(31)
  x0 += k0; x1 += 3ULL;        // injection 3: ks[0], ks[1] + 3
  BGS_MIX(16) BGS_MIX(32) BGS_MIX(24) BGS_MIX(21)
  x0 += 0;  x1 += k2 + 4ULL;   // injection 4: ks[1], ks[2] + 4
  BGS_MIX(16) BGS_MIX(42) BGS_MIX(12) BGS_MIX(31)
  x0 += k2;                    // injection 5: ks[2] (x1 is not needed)
#undef BGS_MIX
  return x0;
}

// u01fixedpt<double, uint64_t> (RNG.h:202-238): ((w >> 11) | 1) * 2^-53,
// assembled from integer bits (exact; no floating-point conversion needed).
// u * 2^scale (scale 0 or 1: exact) for the draw u = m * 2^-53
__device__ __forceinline__ double u01_from_bits(unsigned long long w, int scale = 0) {
  const unsigned long long m = (w >> 11) | 1ULL;     // 1 <= m < 2^53, odd
  const int s = __clzll(m) - 11;                     // shift to put the top bit at 52
  const unsigned long long mant = (m << s) & 0x000FFFFFFFFFFFFFULL;
  const unsigned long long expo = (unsigned long long)(1023 - 1 - s + scale);  // u in [2^-1-s, 2^-s)
  return __longlong_as_double((long long)((expo << 52) | mant));
}

// mu = u*2 - 1 for u = m * 2^-53 (sampling_functions.h:63): exactly
// (m - 2^52) * 2^-52, assembled from integer bits (m odd, so never zero)
__device__ __forceinline__ double mu_from_m53(unsigned long long m) {
  const long long k = (long long)m - (1LL << 52);
  const unsigned long long a = (unsigned long long)(k < 0 ? -k : k);  // 1 <= a < 2^52
  const int s = __clzll((long long)a) - 11;
  const unsigned long long mant = (a << s) & 0x000FFFFFFFFFFFFFULL;
  const unsigned long long expo = (unsigned long long)(1023 - s);  // a*2^-52 in [2^-s, 2^(1-s))
  return __longlong_as_double((long long)(((k < 0 ? 1ULL : 0ULL) << 63) | (expo << 52) | mant));
}

struct Rng {
  unsigned long long stream, ctr, hi;  // hi = seed << 32
  __device__ __forceinline__ double next() {
    const double u = u01_from_bits(threefry2x64_20_w0(ctr, hi, stream));
    ++ctr;
    return u;
  }
  // 2u for the next draw u, exactly (the azimuth's u * 2.0)
  __device__ __forceinline__ double next_twice() {
    const double u2 = u01_from_bits(threefry2x64_20_w0(ctr, hi, stream), 1);
    ++ctr;
    return u2;
  }
  // advance past a draw whose value cannot change the result
  __device__ __forceinline__ void skip() { ++ctr; }
  // the integer m of the next draw u = m * 2^-53 (u01fixedpt, RNG.h:202-238)
  __device__ __forceinline__ unsigned long long next_m53() {
    const unsigned long long w = threefry2x64_20_w0(ctr, hi, stream);
    ++ctr;
    return (w >> 11) | 1ULL;
  }
};

// ------------------------------------------------------ fixed point
// x >= 0 to a 128-bit integer floor(x * 2^scale); contributions far below
// the tally's resolution truncate.  Returns false if out of range.
__device__ __forceinline__ bool to_fixed128(double x, int scale, unsigned long long &lo,
                                            unsigned long long &hi) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7FF);
  lo = 0;
  hi = 0;
  if (bits >> 63) return x == 0.0;   // negative (or -0.0)
  if (e == 0x7FF) return false;      // inf / nan
  if (e == 0) return true;           // zero or subnormal: below resolution
  const unsigned long long m = (bits & 0x000FFFFFFFFFFFFFULL) | 0x0010000000000000ULL;
  const int sh = e - 1075 + scale;   // x = m * 2^(e-1075)
  if (sh >= 0) {
    if (sh > 74) return false;       // would not fit in 128 bits
    if (sh == 0) { lo = m; }
    else if (sh < 64) { lo = m << sh; hi = m >> (64 - sh); }
    else { hi = m << (sh - 64); }
  } else {
    if (sh > -64) lo = m >> (-sh);
  }
  return true;
}

__device__ __forceinline__ void atomic_add128(unsigned long long *lo_p, unsigned long long *hi_p,
                                              unsigned long long lo, unsigned long long hi) {
  if (lo) {
    const unsigned long long old = atomicAdd(lo_p, lo);
    if (old + lo < old) hi += 1ULL;  // carry out of the low word
  }
  if (hi) atomicAdd(hi_p, hi);
}

// signed values in two's complement: |x| as above, negated if x < 0
__device__ __forceinline__ bool to_fixed128_signed(double x, int scale, unsigned long long &lo,
                                                   unsigned long long &hi) {
  const bool ok = to_fixed128(fabs(x), scale, lo, hi);
  if (x < 0.0) {
    lo = ~lo + 1ULL;
    hi = ~hi + (lo == 0ULL ? 1ULL : 0ULL);
  }
  return ok;
}

__host__ __device__ __forceinline__ double from_fixed128(unsigned long long lo, unsigned long long hi,
                                                         int scale) {
  const double v = (double)hi * 18446744073709551616.0 + (double)lo;
#ifdef __CUDA_ARCH__
  return scalbn(v, -scale);
#else
  return __builtin_scalbn(v, -scale);
#endif
}

__host__ __device__ __forceinline__ double from_fixed128_signed(unsigned long long lo, unsigned long long hi,
                                                                int scale) {
  if (!(hi >> 63)) return from_fixed128(lo, hi, scale);
  const unsigned long long nlo = ~lo + 1ULL;
  const unsigned long long nhi = ~hi + (nlo == 0ULL ? 1ULL : 0ULL);
  return -from_fixed128(nlo, nhi, scale);
}

// exponent such that bound * 2^scale <= 2^118 (ten bits of headroom below 2^128)
__device__ __forceinline__ int fixed_scale_for(double bound) {
  if (!(bound > 0.0)) return 0;
  int e;
  frexp(bound, &e);  // bound < 2^e
  return 118 - e;
}

// ------------------------------------------------------ photon counts
// photons made for one cell energy (source.h:229-243): at least one
__device__ __forceinline__ uint32_t photons_for(unsigned long long n_user, double E, double total_E) {
  if (!(E > 0.0)) return 0u;
  const uint32_t t = (uint32_t)(int)((double)n_user * E / total_E);
  return t == 0u ? 1u : t;
}

}  // namespace bgs
