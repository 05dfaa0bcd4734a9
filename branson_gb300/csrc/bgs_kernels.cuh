// Device helpers shared by the kernels and the host launcher declarations.
#pragma once

#include "bgs_fixmath.cuh"
#include "bgs_internal.cuh"

namespace bgs {

// node array of cell g (cell.h:325): (x_lo, x_hi, y_lo, y_hi, z_lo, z_hi)
__device__ __forceinline__ void cell_nodes(const MeshDev &m, uint32_t g, double n[6]) {
  uint32_t i, j, k;
  cell_coords(m, g, i, j, k);
  n[0] = m.x[i];
  n[1] = m.x[i + 1];
  n[2] = m.y[j];
  n[3] = m.y[j + 1];
  n[4] = m.z[k];
  n[5] = m.z[k + 1];
}

// Cell::get_volume (cell.h:188-191)
__device__ __forceinline__ double cell_volume(const double n[6]) {
  return (n[1] - n[0]) * (n[3] - n[2]) * (n[5] - n[4]);
}

// x^n for a small integer n >= 0 (the temperature powers of
// calculate_photon_energy), rounded once: the running product is kept as an
// unevaluated double-double sum with exact products (Dekker's TwoProduct
// via fma), so the result is the correctly rounded power except when the
// exact value lies within ~n*2^-105 relative of a rounding boundary.  Zero,
// non-finite and out-of-range arguments take pow.
__device__ __forceinline__ double pow_small_int_rn(double x, int n) {
  if (n == 0) return 1.0;
  if (x == 0.0) return (n & 1) ? x : 0.0;  // pow(+-0, n > 0)
  if (!(x > 0.0) || !isfinite(x) || x > 1e60 || x < 1e-60) return pow(x, (double)n);
  double ph = x, pl = 0.0;
  for (int i = 1; i < n; ++i) {
    const double p = __dmul_rn(ph, x);
    const double e = __fma_rn(ph, x, -p);   // ph*x - p, exact
    const double l = __fma_rn(pl, x, e);
    const double s = __dadd_rn(p, l);
    pl = __dsub_rn(l, __dsub_rn(s, p));     // |p| >= |l|: exact error of s
    ph = s;
  }
  return ph;
}

// x^3 and x^4 as pow_small_int_rn(x, 3) and (x, 4) return them: the fourth
// power continues the third's double-double product
__device__ __forceinline__ void pow34_rn(double x, double &p3, double &p4) {
  if (x == 0.0 || !(x > 0.0) || !isfinite(x) || x > 1e60 || x < 1e-60) {
    p3 = pow_small_int_rn(x, 3);
    p4 = pow_small_int_rn(x, 4);
    return;
  }
  double ph = x, pl = 0.0;
  for (int i = 1; i < 4; ++i) {
    const double p = __dmul_rn(ph, x);
    const double e = __fma_rn(ph, x, -p);
    const double l = __fma_rn(pl, x, e);
    const double s = __dadd_rn(p, l);
    pl = __dsub_rn(l, __dsub_rn(s, p));
    ph = s;
    if (i == 2) p3 = ph;
  }
  p4 = ph;
}

// pow(x, c) with the small-integer exponents of the decks done exactly
__device__ __forceinline__ double pow_deck(double x, double c) {
  const int n = (int)c;
  if ((double)n == c && n >= 0 && n <= 8) return pow_small_int_rn(x, n);
  return pow(x, c);
}

// RN(1/b) for div_recip (bgs_physics.cuh), or 0 when |b| is outside
// [2^-900, 2^900], where the division must be done directly
__device__ __forceinline__ double recip_for_div(double b) {
  const double ab = fabs(b);
  return (ab >= 0x1p-900 && ab <= 0x1p900) ? 1.0 / b : 0.0;
}

// per-cell transport coefficients (see CellXS) and the CDF step of
// sample_emission_group's walk, op_a(g) * 1/(op_a(0)*N) with all groups
// equal (sampling_functions.h:132-135, cell.h:260-266)
__device__ __forceinline__ void set_cell_xs(const CellsDev &c, uint32_t g, double op_a, double op_s,
                                            double f, uint32_t n_groups) {
  CellXS x;
  x.sig_eff = (1.0 - f) * op_a + op_s;
  x.neg_saf = -op_a * f;
  // op_s / sigma_eff; a zero op_s over a positive finite sigma_eff is op_s itself
  x.p_scat = (op_s == 0.0 && x.sig_eff > 0.0 && x.sig_eff < 1.7976931348623157e308) ? op_s
                                                                                   : op_s / x.sig_eff;
  x.inv_se = recip_for_div(x.sig_eff);
  c.xs[g] = x;
  c.inv_saf[g] = 1.0 / (op_a * f);
  // read only by the multigroup resample (sample_group)
  if (n_groups > 1) {
    const double norm_factor = 1.0 / (op_a * (double)n_groups);
    c.group_v[g] = op_a * norm_factor;
  } else {
    c.group_v[g] = 1.0;
  }
}

// ---------------------------------------------------------------- launchers
void launch_init_cells(const MeshDev &m, const CellsDev &c, cudaStream_t s);
__host__ __device__ uint32_t energy_parts(uint32_t n_cells);
void launch_cell_energy(const MeshDev &m, const CellsDev &c, uint32_t step, double dt, double *mat_E,
                        double *part, DeviceDiag *d, unsigned long long n_user, cudaStream_t s,
                        const double *op_a_in = nullptr);
void launch_check_counts(const MeshDev &m, const CellsDev &c, DeviceDiag *d, uint32_t step, cudaStream_t s);
void launch_cell_xs(const MeshDev &m, const CellsDev &c, cudaStream_t s);
uint32_t scan_tiles_needed(uint64_t n);
void launch_scan_counts(const uint32_t *cnt, const uint32_t *cnt2, uint32_t n,
                        unsigned long long *out, unsigned long long *tile_sum, cudaStream_t s);
void launch_scan_flags(const uint8_t *desc, uint8_t want, uint32_t capacity,
                       const unsigned long long *n_dev, unsigned long long *out,
                       unsigned long long *tile_sum, cudaStream_t s);
void launch_bank_bounds(const Bank &b, unsigned long long *max_bits, DeviceDiag *d, int n_sm,
                        cudaStream_t s);
void launch_tally_to_double(const MeshDev &m, const CellsDev &c, DeviceDiag *d, double *abs_out,
                           double *track_out, cudaStream_t s);
void launch_update_temperature(const MeshDev &m, const CellsDev &c, DeviceDiag *d, double dt,
                               const double *abs_in, const double *track_in, double *mat_part,
                               cudaStream_t s);
uint32_t update_temperature_parts(uint32_t n_cells);

void launch_plan_bank(const MeshDev &m, const CellsDev &c, DeviceDiag *d, uint32_t step,
                      unsigned long long capacity, cudaStream_t s);
void launch_source(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d, uint32_t seed,
                   uint32_t step, double dt, int n_sm, cudaStream_t s);

struct TransportLaunch {
  int blocks, threads;
};
// persistent grid of the history kernel for a block size of 64, 128 or 256
TransportLaunch transport_launch_shape(int n_sm, int threads = 128);
void launch_transport_history(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d,
                              uint32_t seed, const TransportLaunch &shape, cudaStream_t s);
// history transport of bank entries [first, first + count) with their own
// work counter (zeroed by the caller)
void launch_transport_history_range(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d,
                                    uint32_t seed, unsigned long long first, unsigned long long count,
                                    unsigned long long *queue, const TransportLaunch &shape, cudaStream_t s);
void launch_census(const Bank &from, const Bank &to, DeviceDiag *d, const unsigned long long *off,
                   double next_dt, int n_sm, cudaStream_t s);
void launch_transport_resume(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d,
                             uint32_t seed, const EventState &es, const TransportLaunch &shape,
                             cudaStream_t s);
// event mode: one stage round (advance, scatter, boundary, rotate) per call
void launch_event_init(const EventState &es, DeviceDiag *d, cudaStream_t s);
void launch_event_round(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d, uint32_t seed,
                        const EventState &es, bool first, int n_sm, cudaStream_t s);

// problem of work item w: the last p with item_off[p] <= w (n problems),
// searched in [lo, n) (item_off[lo] <= w)
__device__ __forceinline__ uint32_t problem_of(const unsigned long long *item_off, uint32_t n,
                                               unsigned long long w, uint32_t lo = 0) {
  uint32_t hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (item_off[mid] <= w) lo = mid; else hi = mid;
  }
  return lo;
}

// Many independent problems stepped together (bgs_batch.cu): one problem's
// view for the batched launches, in device memory.  Every batched kernel
// takes the view table and runs problem blockIdx.y; the step's parameters
// live in the table, so one recorded launch sequence serves every step.
struct ProblemView {
  MeshDev m;
  CellsDev c;
  DeviceDiag *d;
  Bank from, to;             // this step's bank and the bank the census goes to
  double *mat_E, *energy_part, *abs, *track, *mat_part;
  unsigned long long *tile_cells, *off_bank, *tile_bank, *maxbits;
  unsigned long long n_user, seed_hi;
  uint32_t capacity, step;
  double dt, next_dt;
};
TransportLaunch batch_launch_shape(int n_sm);
// per-problem block counts of the batched launches
struct BatchGrid {
  uint32_t n;              // problems (gridDim.y)
  uint32_t cells;          // blocks per problem over cells
  uint32_t photons;        // blocks per problem over bank entries
  uint32_t cell_tiles;     // scan tiles over the largest mesh
  uint32_t bank_tiles;     // scan tiles over the largest bank capacity
};
// phases of one batched step, in order (bgs_mesh.cu, bgs_source.cu, bgs_batch.cu, bgs_transport.cu)
void launch_batch_begin(const ProblemView *v, const BatchGrid &g, cudaStream_t s);
void launch_batch_energy(const ProblemView *v, const BatchGrid &g, cudaStream_t s);
void launch_batch_source(const ProblemView *v, const BatchGrid &g, cudaStream_t s);
void launch_batch_bounds(const ProblemView *v, const BatchGrid &g, cudaStream_t s);
// item offsets: exclusive prefix sum of every problem's n_bank (n+1 entries)
void launch_batch_items(const ProblemView *v, uint32_t n, unsigned long long *item_off,
                        unsigned long long *work_counter, cudaStream_t s);
void launch_transport_batched(const ProblemView *v, uint32_t n, const unsigned long long *item_off,
                              unsigned long long *work_counter, const TransportLaunch &shape, bool gray,
                              cudaStream_t s);
void launch_batch_census_scan(const ProblemView *v, const BatchGrid &g, cudaStream_t s);
void launch_batch_census(const ProblemView *v, const BatchGrid &g, cudaStream_t s);
void launch_batch_finish(const ProblemView *v, const BatchGrid &g, cudaStream_t s);
// every problem's DeviceDiag gathered into out[0..n) (one copy to the host instead of n)
void launch_batch_diag_gather(const ProblemView *v, uint32_t n, DeviceDiag *out, cudaStream_t s);

// adjoint replay of a saved photon bank (bgs_adjoint.cu)
TransportLaunch adjoint_launch_shape(int n_sm);
void launch_adjoint_cells(const CellsDev &c, uint32_t n_cells, AdjCell *adj, double *src,
                          unsigned long long *coef_max_bits, cudaStream_t s);
void launch_adjoint_set_w(uint32_t n_cells, AdjCell *adj, const double *w, cudaStream_t s);
// the replay passes over n problems; item_off (device, n+1 entries) is the
// exclusive prefix sum of the problems' saved histories
void launch_adjoint_replay(const AdjProblem *probs, uint32_t n, const unsigned long long *item_off,
                           const AdjShared &a, const TransportLaunch &shape, cudaStream_t s);
void launch_adjoint_grad_to_double(uint32_t n_cells, const unsigned long long *grad, int scale, double *out,
                                   cudaStream_t s);

}  // namespace bgs
