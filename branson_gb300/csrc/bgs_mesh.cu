// Per-cell physics of the replicated step: opacity / Fleck factor / source
// energies (Mesh::calculate_photon_energy, mesh.h:237-323), photon counts
// and their prefix sums (source.h:225-245), and the tally reduce fused with
// the temperature update (replicated_driver.h:90-96 + Mesh::update_temperature,
// mesh.h:327-423).
//
// All of this is O(cells) work that is HBM/latency bound and small next to
// transport; the one serial piece is the cell-order floating-point sum of the
// source energies, kept serial because the photon counts int(n*E/total)
// depend on its exact rounding.
#include "bgs_kernels.cuh"

namespace bgs {

// ---------------------------------------------------------------------------
// Cell::get_source_face over the structured mesh (cell.h:69-76): the first
// face (X-, X+, Y-, Y+, Z-, Z+) that is a domain face with a SOURCE condition.
__global__ void k_init_cells(MeshDev m, CellsDev c) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= m.n_cells) return;
  const uint32_t i = g % m.ngx, j = (g / m.ngx) % m.ngy, k = g / (m.ngx * m.ngy);
  const bool at_face[6] = {i == 0, i + 1 == m.ngx, j == 0, j + 1 == m.ngy, k == 0, k + 1 == m.ngz};
  int sf = -1;
  for (int f = 0; f < 6; ++f)
    if (at_face[f] && m.bc[f] == SOURCE) { sf = f; break; }
  c.source_face[g] = (int8_t)sf;
  const double *r = m.regions + 8 * (size_t)m.region[g];
  c.T_e[g] = r[6];   // Mesh::initialize_physical_properties (mesh.h:426-439)
  c.T_r[g] = r[7];
  c.T_s[g] = sf != -1 ? m.T_source : 0.0;
}

// Cell::get_face_area (cell.h:83-100)
__device__ __forceinline__ double face_area(const double n[6], int face) {
  if (face == 0 || face == 1) return __dmul_rn(__dsub_rn(n[3], n[2]), __dsub_rn(n[5], n[4]));
  if (face == 2 || face == 3) return __dmul_rn(__dsub_rn(n[1], n[0]), __dsub_rn(n[5], n[4]));
  if (face == 4 || face == 5) return __dmul_rn(__dsub_rn(n[1], n[0]), __dsub_rn(n[3], n[2]));
  return -1.0;
}

// Mesh::calculate_photon_energy per cell (mesh.h:253-287), one rank
// (replicated factor 1).  Also derives the transport table.
__device__ __forceinline__ void cell_energy_body(const MeshDev &m, const CellsDev &c, uint32_t step, double dt,
                                                 double *mat_E, const double *op_a_in, uint32_t bx, uint32_t nbx) {
  for (uint32_t g = bx * blockDim.x + threadIdx.x; g < m.n_cells; g += nbx * blockDim.x) {
    double n[6];
    cell_nodes(m, g, n);
    const double vol = cell_volume(n);
    const double *r = m.regions + 8 * (size_t)m.region[g];
    const double cV = r[0], rho = r[1], A = r[2], B = r[3], Cx = r[4], S = r[5];
    const double T = c.T_e[g], Tr = c.T_r[g], Ts = c.T_s[g];
    const double rf = 1.0;
    // Region::get_absorption_opacity (region.h:44-46), or the caller's
    // per-cell opacity when it supplies one (the adjoint forward)
    const double op_a = op_a_in ? op_a_in[g] : A + B * pow_deck(T, Cx);
    const double op_s = S;
    double T3, T4;
    pow34_rn(T, T3, T4);
    const double f = 1.0 / (1.0 + dt * op_a * kC * (4.0 * kA * T3 / (cV * rho)));
    c.op_a[g] = op_a;
    c.op_s[g] = op_s;
    c.f[g] = f;
    c.em_E[g] = rf * dt * vol * f * op_a * kA * kC * T4;
    c.ce_E[g] = (step > 1) ? 0.0 : rf * vol * kA * pow_small_int_rn(Tr, 4);
    c.so_E[g] = rf * 0.25 * kA * kC * face_area(n, c.source_face[g]) * pow_small_int_rn(Ts, 4) * dt;
    mat_E[g] = T * cV * vol * rho;
    set_cell_xs(c, g, op_a, op_s, f, m.n_groups);
  }
}

__global__ void k_cell_energy(MeshDev m, CellsDev c, uint32_t step, double dt, double *mat_E,
                              const double *op_a_in) {
  cell_energy_body(m, c, step, dt, mat_E, op_a_in, blockIdx.x, gridDim.x);
}

// Transport table from op_a, op_s, f already in the cell arrays (the
// drop-in path, where the caller supplies the opacities).
__global__ void k_cell_xs(MeshDev m, CellsDev c) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= m.n_cells) return;
  set_cell_xs(c, g, c.op_a[g], c.op_s[g], c.f[g], m.n_groups);
}

// The cell-order sums of calculate_photon_energy (mesh.h:282-287).  The
// upstream total is a left-to-right floating-point sum, and the photon
// counts int(n_user*E/total) (source.h:229-243) depend on its rounding.  A
// serial FP64 chain is very slow on one GPU lane, so the total is first
// formed by a deterministic tree sum; every cell count is then checked
// against the rounding-error bound of the serial sum, and only if some count
// could differ (an integer inside the error window of n_user*E/total) does
// the serial sum run (k_serial_total).  Either way the counts equal the
// upstream ones.
constexpr int kSumThreads = 256;

__device__ __forceinline__ void energy_partials_body(const MeshDev &m, const CellsDev &c, const double *mat_E,
                                                     double *part, uint32_t bx, uint32_t nbx) {
  __shared__ double s[5][kSumThreads];
  const uint32_t parts = (m.n_cells + kSumThreads - 1) / kSumThreads;
  for (uint32_t b = bx; b < parts; b += nbx) {
    const uint32_t g = b * kSumThreads + threadIdx.x;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (g < m.n_cells) {
      v[0] = c.so_E[g] + c.ce_E[g] + c.em_E[g];  // the upstream per-cell term
      v[1] = c.em_E[g];
      v[2] = c.ce_E[g];
      v[3] = c.so_E[g];
      v[4] = mat_E[g];
    }
    __syncthreads();
    for (int q = 0; q < 5; ++q) s[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int o = kSumThreads / 2; o > 0; o >>= 1) {
      if (threadIdx.x < (unsigned)o)
        for (int q = 0; q < 5; ++q) s[q][threadIdx.x] += s[q][threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x < 5) part[5 * (size_t)b + threadIdx.x] = s[threadIdx.x][0];
  }
}

__global__ void __launch_bounds__(kSumThreads) k_energy_partials(MeshDev m, CellsDev c, const double *mat_E,
                                                                 double *part) {
  energy_partials_body(m, c, mat_E, part, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void energy_finish_body(const double *part, uint32_t n_parts, DeviceDiag *d) {
  // one warp: lane q < 5 sums column q in block order (deterministic)
  const int q = threadIdx.x;
  if (q >= 5) return;
  double acc = 0.0;
  for (uint32_t b = 0; b < n_parts; ++b) acc += part[5 * (size_t)b + q];
  if (q == 0) { d->total_photon_E = acc; d->serial_needed = 0; }
  if (q == 1) d->emission_E = acc;
  if (q == 2) d->census_cell_E = acc;
  if (q == 3) d->source_E = acc;
  if (q == 4) d->pre_mat_E = acc;
}

__global__ void k_energy_finish(const double *part, uint32_t n_parts, DeviceDiag *d) {
  energy_finish_body(part, n_parts, d);
}

// could int(n_user*E/total_serial) differ from int(n_user*E/total_tree)?
// photons_for(n_user, E, total) from one quotient, and whether the count
// could differ under the serial sum: q's window of the total's error bound
// holds an integer boundary (counts 0 and 1 both become one photon)
__device__ __forceinline__ uint32_t count_checked(unsigned long long n_user, double E, double total, double window,
                                                  bool &ambiguous) {
  if (!(E > 0.0)) return 0u;
  const double q = (double)n_user * E / total;
  const double lo = q - q * window, hi = q + q * window;
  if (!(hi < 2.0) && floor(lo) != floor(hi)) ambiguous = true;
  const uint32_t t = (uint32_t)(int)q;
  return t == 0u ? 1u : t;
}

// counts from the tree total, flagging the step when any could differ
__device__ __forceinline__ void counts_check_body(const MeshDev &m, const CellsDev &c, DeviceDiag *d,
                                                  unsigned long long n_user, uint32_t step, uint32_t bx,
                                                  uint32_t nbx) {
  const double total = d->total_photon_E;
  // |serial - exact| <= (n-1) u sum, |tree - exact| <= (log2 n + 1) u sum,
  // plus the rounding of n*E/total: a window of (n + 64) u, doubled
  const double window = 2.0 * ((double)m.n_cells + 64.0) * 1.1102230246251565e-16;
  bool amb = false;
  for (uint32_t g = bx * blockDim.x + threadIdx.x; g < m.n_cells; g += nbx * blockDim.x) {
    c.n_em[g] = count_checked(n_user, c.em_E[g], total, window, amb);
    c.n_so[g] = count_checked(n_user, c.so_E[g], total, window, amb);
    c.n_ce[g] = step == 1 ? count_checked(n_user, c.ce_E[g], total, window, amb) : 0u;
  }
  if (amb) d->serial_needed = 1;
}

__global__ void k_counts_check(MeshDev m, CellsDev c, DeviceDiag *d, unsigned long long n_user,
                               uint32_t step) {
  counts_check_body(m, c, d, n_user, step, blockIdx.x, gridDim.x);
}

// the upstream serial sum, run only when a count is ambiguous; one block
// stages the per-cell terms in shared memory, thread 0 keeps the add chain
__device__ __forceinline__ void serial_total_body(const MeshDev &m, const CellsDev &c, DeviceDiag *d) {
  if (!d->serial_needed) return;
  constexpr int kChunk = 2048;
  __shared__ double s_t[kChunk];
  double total = 0.0;
  for (uint32_t base = 0; base < m.n_cells; base += kChunk) {
    const uint32_t cnt = min((uint32_t)kChunk, m.n_cells - base);
    for (uint32_t t = threadIdx.x; t < cnt; t += blockDim.x) {
      const uint32_t g = base + t;
      s_t[t] = c.so_E[g] + c.ce_E[g] + c.em_E[g];
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (uint32_t t = 0; t < cnt; ++t) total += s_t[t];
    __syncthreads();
  }
  if (threadIdx.x == 0) d->total_photon_E = total;
}

__global__ void k_serial_total(MeshDev m, CellsDev c, DeviceDiag *d) { serial_total_body(m, c, d); }

// photons per cell for emission, boundary source and (step 1) initial
// census from the serial total, when the checked counts were ambiguous
__device__ __forceinline__ void recount_body(const MeshDev &m, const CellsDev &c, const DeviceDiag *d,
                                             unsigned long long n_user, uint32_t step, uint32_t bx, uint32_t nbx) {
  if (!d->serial_needed) return;
  const double total = d->total_photon_E;
  for (uint32_t g = bx * blockDim.x + threadIdx.x; g < m.n_cells; g += nbx * blockDim.x) {
    c.n_em[g] = photons_for(n_user, c.em_E[g], total);
    c.n_so[g] = photons_for(n_user, c.so_E[g], total);
    c.n_ce[g] = step == 1 ? photons_for(n_user, c.ce_E[g], total) : 0u;
  }
}

__global__ void k_recount(MeshDev m, CellsDev c, const DeviceDiag *d, unsigned long long n_user,
                          uint32_t step) {
  recount_body(m, c, d, n_user, step, blockIdx.x, gridDim.x);
}

// counts supplied by the caller (frozen across perturbed runs) must give every
// cell with energy at least one photon and none to a cell without
__global__ void k_check_counts(MeshDev m, CellsDev c, DeviceDiag *d, uint32_t step) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= m.n_cells) return;
  bool bad = (c.em_E[g] > 0.0) != (c.n_em[g] > 0u) || (c.so_E[g] > 0.0) != (c.n_so[g] > 0u);
  if (step == 1) bad |= (c.ce_E[g] > 0.0) != (c.n_ce[g] > 0u);
  else bad |= c.n_ce[g] != 0u;
  if (bad) {
    atomicOr(&d->flags, (uint32_t)FLAG_BAD_COUNTS);
    atomicCAS(&d->bad_counts_cell, 0u, g + 1u);
  }
}

void launch_check_counts(const MeshDev &m, const CellsDev &c, DeviceDiag *d, uint32_t step, cudaStream_t s) {
  k_check_counts<<<(m.n_cells + 255) / 256, 256, 0, s>>>(m, c, d, step);
}

// ---------------------------------------------------------------------------
// Exclusive prefix sum of uint32 counts into uint64 offsets (n+1 entries),
// three passes: per-block scan, scan of block totals, add.
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename Pred>
__device__ __forceinline__ void scan_tile(uint32_t n, uint32_t tile, Pred value,
                                          unsigned long long *out, unsigned long long *tile_sum) {
  __shared__ unsigned long long s_warp[kScanThreads / 32];
  const uint32_t base = tile * kScanTile + threadIdx.x * kScanItems;
  unsigned long long v[kScanItems];
  unsigned long long run = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    const uint32_t idx = base + q;
    v[q] = idx < n ? (unsigned long long)value(idx) : 0ULL;
    run += v[q];
  }
  // inclusive warp scan of the per-thread totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long incl = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < kScanThreads / 32 ? s_warp[lane] : 0ULL;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < kScanThreads / 32) s_warp[lane] = w;
  }
  __syncthreads();
  unsigned long long excl = incl - run + (warp > 0 ? s_warp[warp - 1] : 0ULL);
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    const uint32_t idx = base + q;
    if (idx < n) out[idx] = excl;
    excl += v[q];
  }
  if (threadIdx.x == kScanThreads - 1) tile_sum[tile] = excl;
}

__device__ __forceinline__ void scan_counts_body(const uint32_t *cnt, const uint32_t *cnt2, uint32_t n,
                                                 unsigned long long *out, unsigned long long *tile_sum,
                                                 uint32_t bx, uint32_t nbx) {
  const uint32_t tiles = n > 0 ? (uint32_t)((n + kScanTile - 1) / kScanTile) : 1u;
  for (uint32_t t = bx; t < tiles; t += nbx) {
    __syncthreads();
    if (cnt2)
      scan_tile(n, t, [cnt, cnt2](uint32_t i) { return cnt[i] + cnt2[i]; }, out, tile_sum);
    else
      scan_tile(n, t, [cnt](uint32_t i) { return cnt[i]; }, out, tile_sum);
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_counts(const uint32_t *cnt, const uint32_t *cnt2,
                                                              uint32_t n, unsigned long long *out,
                                                              unsigned long long *tile_sum) {
  scan_counts_body(cnt, cnt2, n, out, tile_sum, blockIdx.x, gridDim.x);
}

// flags of a bank whose live length *n_dev is only known on the device; the
// tiles cover the capacity and tiles past the end only zero their sums
__device__ __forceinline__ void scan_flags_body(const uint8_t *desc, uint8_t want, const unsigned long long *n_dev,
                                                uint32_t capacity, unsigned long long *out,
                                                unsigned long long *tile_sum, uint32_t bx, uint32_t nbx) {
  const unsigned long long n = *n_dev;
  const uint32_t tiles = capacity > 0 ? (uint32_t)((capacity + kScanTile - 1) / kScanTile) : 1u;
  for (uint32_t t = bx; t < tiles; t += nbx) {
    if ((unsigned long long)t * kScanTile >= n) {
      if (threadIdx.x == 0) tile_sum[t] = 0ULL;
      continue;
    }
    __syncthreads();
    scan_tile((uint32_t)n, t, [desc, want](uint32_t i) { return desc[i] == want ? 1u : 0u; }, out, tile_sum);
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_flags(const uint8_t *desc, uint8_t want,
                                                             const unsigned long long *n_dev, uint32_t capacity,
                                                             unsigned long long *out,
                                                             unsigned long long *tile_sum) {
  scan_flags_body(desc, want, n_dev, capacity, out, tile_sum, blockIdx.x, gridDim.x);
}

// exclusive scan of tile sums in one block (sequential over chunks)
__device__ __forceinline__ void scan_tiles_body(unsigned long long *tile_sum, uint32_t n_tiles,
                                                unsigned long long *total_out) {
  __shared__ unsigned long long s[1024];
  unsigned long long carry = 0;
  for (uint32_t base = 0; base < n_tiles; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    const unsigned long long v = i < n_tiles ? tile_sum[i] : 0ULL;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const unsigned long long t = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0ULL;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n_tiles) tile_sum[i] = carry + s[threadIdx.x] - v;
    const unsigned long long chunk_total = s[1023];
    __syncthreads();
    carry += chunk_total;
  }
  if (threadIdx.x == 0 && total_out) *total_out = carry;
}

__global__ void __launch_bounds__(1024) k_scan_tiles(unsigned long long *tile_sum, uint32_t n_tiles,
                                                     unsigned long long *total_out) {
  scan_tiles_body(tile_sum, n_tiles, total_out);
}

__device__ __forceinline__ void scan_add_body(unsigned long long *out, uint32_t n, const unsigned long long *n_dev,
                                              const unsigned long long *tile_sum, const unsigned long long *total,
                                              uint32_t bx, uint32_t nbx) {
  if (n_dev) n = (uint32_t)*n_dev;
  for (uint32_t i = bx * blockDim.x + threadIdx.x; i < n; i += nbx * blockDim.x) out[i] += tile_sum[i / kScanTile];
  if (bx == 0 && threadIdx.x == 0) out[n] = *total;
}

__global__ void k_scan_add(unsigned long long *out, uint32_t n, const unsigned long long *n_dev,
                           const unsigned long long *tile_sum, const unsigned long long *total) {
  scan_add_body(out, n, n_dev, tile_sum, total, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// Fixed-point scale for a bank of photons: the bound from the largest photon
// energy (an order-independent maximum, so the scale and hence the tallies
// are deterministic).
__device__ __forceinline__ void bank_bounds_body(const Bank &b, const DeviceDiag *d, unsigned long long *max_bits,
                                                 uint32_t bx, uint32_t nbx) {
  const unsigned long long n = d->n_bank;
  unsigned long long mE = 0;
  for (unsigned long long i = bx * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)nbx * blockDim.x)
    mE = max(mE, (unsigned long long)__double_as_longlong(fabs(b.E[i])));
  for (int o = 16; o > 0; o >>= 1) mE = max(mE, __shfl_down_sync(0xffffffffu, mE, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&max_bits[0], mE);
}

__global__ void k_bank_bounds(Bank b, const DeviceDiag *d, unsigned long long *max_bits) {
  bank_bounds_body(b, d, max_bits, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void set_scales_body(DeviceDiag *d, const unsigned long long *max_bits) {
  const double maxE = __longlong_as_double((long long)max_bits[0]);
  const double n = (double)(d->n_bank > 0 ? d->n_bank : 1ULL);
  // absorbed energy of a history (and any of its parts) <= its starting
  // energy (transport_photon :74-82)
  const double bound_abs = 2.0 * maxE * n + 1e-300;
  d->scale_abs = fixed_scale_for(bound_abs);
}

__global__ void k_set_scales(DeviceDiag *d, const unsigned long long *max_bits) { set_scales_body(d, max_bits); }

// ---------------------------------------------------------------------------
// 128-bit values as three 43-bit limbs so block sums of up to 2^21 terms
// are exact in 64-bit adds.
struct Limbs { unsigned long long a0, a1, a2; };
__device__ __forceinline__ Limbs limbs_of(unsigned long long lo, unsigned long long hi) {
  const unsigned long long M = (1ULL << 43) - 1ULL;
  return {lo & M, ((lo >> 43) | (hi << 21)) & M, hi >> 22};
}
__device__ __forceinline__ void limbs_to128(const Limbs &l, unsigned long long &lo,
                                            unsigned long long &hi) {
  // value = a0 + a1*2^43 + a2*2^86
  lo = l.a0;
  hi = 0;
  const unsigned long long t1 = l.a1 << 43;
  const unsigned long long o = lo;
  lo += t1;
  hi += (lo < o) ? 1ULL : 0ULL;
  hi += l.a1 >> 21;
  hi += l.a2 << 22;
}

__device__ __forceinline__ Limbs block_sum_limbs(Limbs v) {
  __shared__ unsigned long long s[3][32];
  for (int o = 16; o > 0; o >>= 1) {
    v.a0 += __shfl_down_sync(0xffffffffu, v.a0, o);
    v.a1 += __shfl_down_sync(0xffffffffu, v.a1, o);
    v.a2 += __shfl_down_sync(0xffffffffu, v.a2, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) { s[0][warp] = v.a0; s[1][warp] = v.a1; s[2][warp] = v.a2; }
  __syncthreads();
  Limbs r{0, 0, 0};
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    r.a0 = lane < nw ? s[0][lane] : 0ULL;
    r.a1 = lane < nw ? s[1][lane] : 0ULL;
    r.a2 = lane < nw ? s[2][lane] : 0ULL;
    for (int o = 16; o > 0; o >>= 1) {
      r.a0 += __shfl_down_sync(0xffffffffu, r.a0, o);
      r.a1 += __shfl_down_sync(0xffffffffu, r.a1, o);
      r.a2 += __shfl_down_sync(0xffffffffu, r.a2, o);
    }
  }
  return r;  // valid in thread 0
}

__device__ void block_add128(unsigned long long lo, unsigned long long hi, unsigned long long *dst) {
  Limbs t = block_sum_limbs(limbs_of(lo, hi));
  if (threadIdx.x == 0) {
    unsigned long long l, h;
    limbs_to128(t, l, h);
    atomic_add128(&dst[0], &dst[1], l, h);
  }
}

// ---------------------------------------------------------------------------
// Tally -> double per cell (the values replicated_transport copies out to
// rank_abs_E / rank_track_E, replicated_transport.h:135-140) with the total
// absorbed energy summed exactly from the fixed-point integers.
__device__ __forceinline__ void tally_to_double_body(const MeshDev &m, const CellsDev &c, DeviceDiag *d,
                                                     double *abs_out, double *track_out, uint32_t bx, uint32_t nbx) {
  const uint32_t rounds = (m.n_cells + blockDim.x - 1) / blockDim.x;
  for (uint32_t r = bx; r < rounds; r += nbx) {
    const uint32_t g = r * blockDim.x + threadIdx.x;
    unsigned long long alo = 0, ahi = 0;
    if (g < m.n_cells) {
      const TallyCell t = c.tally[g];
      abs_out[g] = from_fixed128(t.abs_lo, t.abs_hi, d->scale_abs);
      // track_E = (abs - dep) / (sigma_a f), by the cell's RN(1/(sigma_a f));
      // a cell that absorbed nothing has none (TallyCell)
      const unsigned long long vlo = t.abs_lo - t.dep_lo;
      const unsigned long long vhi = t.abs_hi - t.dep_hi - (t.abs_lo < t.dep_lo ? 1ULL : 0ULL);
      track_out[g] = (vlo | vhi) ? from_fixed128(vlo, vhi, d->scale_abs) * c.inv_saf[g] : 0.0;
      alo = t.abs_lo;
      ahi = t.abs_hi;
    }
    block_add128(alo, ahi, d->sum_abs);
  }
}

__global__ void k_tally_to_double(MeshDev m, CellsDev c, DeviceDiag *d, double *abs_out,
                                  double *track_out) {
  tally_to_double_body(m, c, d, abs_out, track_out, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void tally_total_body(DeviceDiag *d) {
  d->absorbed_E = from_fixed128(d->sum_abs[0], d->sum_abs[1], d->scale_abs);
}

__global__ void k_tally_total(DeviceDiag *d) { tally_total_body(d); }

// Mesh::update_temperature (mesh.h:349-362) per cell and a deterministic
// block-ordered sum of the post-step material energy (parts of 256 cells).
constexpr uint32_t kTempThreads = 256;

__device__ __forceinline__ void update_temperature_body(const MeshDev &m, const CellsDev &c, double dt,
                                                        const double *abs_in, const double *track_in,
                                                        double *mat_part, uint32_t bx, uint32_t nbx) {
  __shared__ double s[kTempThreads];
  const uint32_t parts = (m.n_cells + kTempThreads - 1) / kTempThreads;
  for (uint32_t b = bx; b < parts; b += nbx) {
    const uint32_t g = b * kTempThreads + threadIdx.x;
    double matE = 0.0;
    if (g < m.n_cells) {
      double n[6];
      cell_nodes(m, g, n);
      const double vol = cell_volume(n);
      const double *r = m.regions + 8 * (size_t)m.region[g];
      const double cV = r[0], rho = r[1];
      const double T = c.T_e[g];
      const double T_new = T + (abs_in[g] - c.em_E[g]) / (cV * vol * rho);
      // x^(1/4) (mesh.h:358), square roots on the integer pipe (bit-identical)
      c.T_r_diag[g] = fix::sqrt_rn(fix::sqrt_rn(track_in[g] / (vol * dt * kA * kC)));
      c.T_e[g] = T_new;
      matE = T_new * cV * vol * rho;
    }
    __syncthreads();
    s[threadIdx.x] = matE;
    __syncthreads();
    for (int o = kTempThreads / 2; o > 0; o >>= 1) {
      if (threadIdx.x < (unsigned)o) s[threadIdx.x] += s[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) mat_part[b] = s[0];
  }
}

__global__ void __launch_bounds__(kTempThreads) k_update_temperature(MeshDev m, CellsDev c, double dt,
                                                                    const double *abs_in, const double *track_in,
                                                                    double *mat_part) {
  update_temperature_body(m, c, dt, abs_in, track_in, mat_part, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void finish_temperature_body(DeviceDiag *d, const double *mat_part, uint32_t n_parts) {
  if (threadIdx.x != 0) return;
  double s = 0.0;
  for (uint32_t i = 0; i < n_parts; ++i) s += mat_part[i];
  d->post_mat_E = s;
}

__global__ void k_finish_temperature(DeviceDiag *d, const double *mat_part, uint32_t n_parts) {
  if (blockIdx.x != 0) return;
  finish_temperature_body(d, mat_part, n_parts);
}

// ---------------------------------------------------------------------------
// host launchers
void launch_init_cells(const MeshDev &m, const CellsDev &c, cudaStream_t s) {
  k_init_cells<<<(m.n_cells + 255) / 256, 256, 0, s>>>(m, c);
}

__host__ __device__ uint32_t energy_parts(uint32_t n_cells) { return (n_cells + kSumThreads - 1) / kSumThreads; }

void launch_cell_energy(const MeshDev &m, const CellsDev &c, uint32_t step, double dt, double *mat_E,
                        double *part, DeviceDiag *d, unsigned long long n_user, cudaStream_t s,
                        const double *op_a_in) {
  const uint32_t blocks = (m.n_cells + 255) / 256;
  const uint32_t parts = energy_parts(m.n_cells);
  k_cell_energy<<<blocks, 256, 0, s>>>(m, c, step, dt, mat_E, op_a_in);
  k_energy_partials<<<parts, kSumThreads, 0, s>>>(m, c, mat_E, part);
  k_energy_finish<<<1, 32, 0, s>>>(part, parts, d);
  k_counts_check<<<blocks, 256, 0, s>>>(m, c, d, n_user, step);
  k_serial_total<<<1, 256, 0, s>>>(m, c, d);
  k_recount<<<blocks, 256, 0, s>>>(m, c, d, n_user, step);
}

void launch_cell_xs(const MeshDev &m, const CellsDev &c, cudaStream_t s) {
  k_cell_xs<<<(m.n_cells + 255) / 256, 256, 0, s>>>(m, c);
}

uint32_t scan_tiles_needed(uint64_t n) { return (uint32_t)((n + kScanTile - 1) / kScanTile); }

void launch_scan_counts(const uint32_t *cnt, const uint32_t *cnt2, uint32_t n, unsigned long long *out,
                        unsigned long long *tile_sum, cudaStream_t s) {
  const uint32_t tiles = scan_tiles_needed(n) > 0 ? scan_tiles_needed(n) : 1;
  k_scan_counts<<<tiles, kScanThreads, 0, s>>>(cnt, cnt2, n, out, tile_sum);
  k_scan_tiles<<<1, 1024, 0, s>>>(tile_sum, tiles, tile_sum + tiles);
  k_scan_add<<<(n + 256) / 256, 256, 0, s>>>(out, n, nullptr, tile_sum, tile_sum + tiles);
}

void launch_scan_flags(const uint8_t *desc, uint8_t want, uint32_t capacity,
                       const unsigned long long *n_dev, unsigned long long *out,
                       unsigned long long *tile_sum, cudaStream_t s) {
  const uint32_t tiles = scan_tiles_needed(capacity) > 0 ? scan_tiles_needed(capacity) : 1;
  k_scan_flags<<<tiles, kScanThreads, 0, s>>>(desc, want, n_dev, capacity, out, tile_sum);
  k_scan_tiles<<<1, 1024, 0, s>>>(tile_sum, tiles, tile_sum + tiles);
  k_scan_add<<<(capacity + 256) / 256, 256, 0, s>>>(out, capacity, n_dev, tile_sum, tile_sum + tiles);
}

void launch_bank_bounds(const Bank &b, unsigned long long *max_bits, DeviceDiag *d, int n_sm,
                        cudaStream_t s) {
  cudaMemsetAsync(max_bits, 0, 2 * sizeof(unsigned long long), s);
  k_bank_bounds<<<n_sm * 4, 256, 0, s>>>(b, d, max_bits);
  k_set_scales<<<1, 1, 0, s>>>(d, max_bits);
}

void launch_tally_to_double(const MeshDev &m, const CellsDev &c, DeviceDiag *d, double *abs_out,
                           double *track_out, cudaStream_t s) {
  cudaMemsetAsync(d->sum_abs, 0, sizeof(d->sum_abs), s);
  k_tally_to_double<<<(m.n_cells + 255) / 256, 256, 0, s>>>(m, c, d, abs_out, track_out);
  k_tally_total<<<1, 1, 0, s>>>(d);
}

void launch_update_temperature(const MeshDev &m, const CellsDev &c, DeviceDiag *d, double dt,
                               const double *abs_in, const double *track_in, double *mat_part,
                               cudaStream_t s) {
  const uint32_t blocks = (m.n_cells + 255) / 256;
  k_update_temperature<<<blocks, 256, 0, s>>>(m, c, dt, abs_in, track_in, mat_part);
  k_finish_temperature<<<1, 32, 0, s>>>(d, mat_part, blocks);
}

uint32_t update_temperature_parts(uint32_t n_cells) { return (n_cells + 255) / 256; }

__device__ __forceinline__ uint32_t update_temperature_parts_dev(uint32_t n_cells) {
  return (n_cells + kTempThreads - 1) / kTempThreads;
}

// ---------------------------------------------------------------------------
// Batched launches: the same bodies, problem blockIdx.y of the view table.
__global__ void k_b_begin(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  unsigned long long *t = reinterpret_cast<unsigned long long *>(P.c.tally);
  const size_t words = 4 * (size_t)P.m.n_cells;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
    t[i] = 0ULL;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.maxbits[0] = 0ULL;
    P.maxbits[1] = 0ULL;
    DeviceDiag *d = P.d;
    d->sum_abs[0] = d->sum_abs[1] = 0ULL;
    d->sum_census[0] = d->sum_census[1] = 0ULL;
    d->sum_exit[0] = d->sum_exit[1] = 0ULL;
  }
}

__global__ void __launch_bounds__(256) k_b_cell_energy(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  cell_energy_body(P.m, P.c, P.step, P.dt, P.mat_E, nullptr, blockIdx.x, gridDim.x);
}
__global__ void __launch_bounds__(kSumThreads) k_b_energy_partials(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  energy_partials_body(P.m, P.c, P.mat_E, P.energy_part, blockIdx.x, gridDim.x);
}
__global__ void k_b_energy_finish(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  energy_finish_body(P.energy_part, energy_parts(P.m.n_cells), P.d);
}
__global__ void __launch_bounds__(256) k_b_counts_check(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  counts_check_body(P.m, P.c, P.d, P.n_user, P.step, blockIdx.x, gridDim.x);
}
__global__ void __launch_bounds__(256) k_b_serial_total(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  serial_total_body(P.m, P.c, P.d);
}
__global__ void __launch_bounds__(256) k_b_recount(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  recount_body(P.m, P.c, P.d, P.n_user, P.step, blockIdx.x, gridDim.x);
}
// which: 0 = emission + source counts into off_new, 1 = census counts into off_ce
__global__ void __launch_bounds__(kScanThreads) k_b_scan_counts(const ProblemView *v, int which) {
  const ProblemView &P = v[blockIdx.y];
  if (which == 0)
    scan_counts_body(P.c.n_em, P.c.n_so, P.m.n_cells, P.c.off_new, P.tile_cells, blockIdx.x, gridDim.x);
  else
    scan_counts_body(P.c.n_ce, nullptr, P.m.n_cells, P.c.off_ce, P.tile_cells, blockIdx.x, gridDim.x);
}
__device__ __forceinline__ uint32_t tiles_of(uint64_t n) {
  return n > 0 ? (uint32_t)((n + kScanTile - 1) / kScanTile) : 1u;
}
// which: 0/1 as above, 2 = census flags over the bank capacity
__global__ void __launch_bounds__(1024) k_b_scan_tiles(const ProblemView *v, int which) {
  const ProblemView &P = v[blockIdx.y];
  const uint32_t tiles = which == 2 ? tiles_of(P.capacity) : tiles_of(P.m.n_cells);
  unsigned long long *ts = which == 2 ? P.tile_bank : P.tile_cells;
  scan_tiles_body(ts, tiles, ts + tiles);
}
__global__ void __launch_bounds__(256) k_b_scan_add(const ProblemView *v, int which) {
  const ProblemView &P = v[blockIdx.y];
  if (which == 2) {
    const uint32_t tiles = tiles_of(P.capacity);
    scan_add_body(P.off_bank, P.capacity, &P.d->n_bank, P.tile_bank, P.tile_bank + tiles, blockIdx.x, gridDim.x);
  } else {
    const uint32_t tiles = tiles_of(P.m.n_cells);
    unsigned long long *out = which == 0 ? P.c.off_new : P.c.off_ce;
    scan_add_body(out, P.m.n_cells, nullptr, P.tile_cells, P.tile_cells + tiles, blockIdx.x, gridDim.x);
  }
}
__global__ void __launch_bounds__(kScanThreads) k_b_scan_flags(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  scan_flags_body(P.from.desc, CENSUS, &P.d->n_bank, P.capacity, P.off_bank, P.tile_bank, blockIdx.x, gridDim.x);
}
__global__ void __launch_bounds__(256) k_b_bank_bounds(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  bank_bounds_body(P.from, P.d, P.maxbits, blockIdx.x, gridDim.x);
}
__global__ void k_b_set_scales(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  if (threadIdx.x == 0) set_scales_body(P.d, P.maxbits);
}
__global__ void __launch_bounds__(256) k_b_tally_to_double(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  tally_to_double_body(P.m, P.c, P.d, P.abs, P.track, blockIdx.x, gridDim.x);
}
__global__ void k_b_tally_total(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  if (threadIdx.x == 0) tally_total_body(P.d);
}
__global__ void __launch_bounds__(kTempThreads) k_b_update_temperature(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  update_temperature_body(P.m, P.c, P.dt, P.abs, P.track, P.mat_part, blockIdx.x, gridDim.x);
}
__global__ void k_b_finish_temperature(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  finish_temperature_body(P.d, P.mat_part, update_temperature_parts_dev(P.m.n_cells));
}

void launch_batch_begin(const ProblemView *v, const BatchGrid &g, cudaStream_t s) {
  k_b_begin<<<dim3(g.cells, g.n), 256, 0, s>>>(v);
}

void launch_batch_energy(const ProblemView *v, const BatchGrid &g, cudaStream_t s) {
  k_b_cell_energy<<<dim3(g.cells, g.n), 256, 0, s>>>(v);
  k_b_energy_partials<<<dim3(g.cells, g.n), kSumThreads, 0, s>>>(v);
  k_b_energy_finish<<<dim3(1, g.n), 32, 0, s>>>(v);
  k_b_counts_check<<<dim3(g.cells, g.n), 256, 0, s>>>(v);
  k_b_serial_total<<<dim3(1, g.n), 256, 0, s>>>(v);
  k_b_recount<<<dim3(g.cells, g.n), 256, 0, s>>>(v);
  for (int which = 0; which < 2; ++which) {
    k_b_scan_counts<<<dim3(g.cell_tiles, g.n), kScanThreads, 0, s>>>(v, which);
    k_b_scan_tiles<<<dim3(1, g.n), 1024, 0, s>>>(v, which);
    k_b_scan_add<<<dim3(g.cells, g.n), 256, 0, s>>>(v, which);
  }
}

void launch_batch_bounds(const ProblemView *v, const BatchGrid &g, cudaStream_t s) {
  k_b_bank_bounds<<<dim3(g.photons, g.n), 256, 0, s>>>(v);
  k_b_set_scales<<<dim3(1, g.n), 32, 0, s>>>(v);
}

// census flags and offsets (before the census copy)
void launch_batch_census_scan(const ProblemView *v, const BatchGrid &g, cudaStream_t s) {
  k_b_scan_flags<<<dim3(g.bank_tiles, g.n), kScanThreads, 0, s>>>(v);
  k_b_scan_tiles<<<dim3(1, g.n), 1024, 0, s>>>(v, 2);
  k_b_scan_add<<<dim3(g.photons, g.n), 256, 0, s>>>(v, 2);
}

void launch_batch_finish(const ProblemView *v, const BatchGrid &g, cudaStream_t s) {
  k_b_tally_to_double<<<dim3(g.cells, g.n), 256, 0, s>>>(v);
  k_b_tally_total<<<dim3(1, g.n), 32, 0, s>>>(v);
  k_b_update_temperature<<<dim3(g.cells, g.n), kTempThreads, 0, s>>>(v);
  k_b_finish_temperature<<<dim3(1, g.n), 32, 0, s>>>(v);
}

static_assert(sizeof(DeviceDiag) % sizeof(unsigned long long) == 0, "DeviceDiag is copied in 8-byte words");
__global__ void k_b_diag_gather(const ProblemView *v, DeviceDiag *out) {
  const unsigned long long *from = reinterpret_cast<const unsigned long long *>(v[blockIdx.x].d);
  unsigned long long *to = reinterpret_cast<unsigned long long *>(out + blockIdx.x);
  for (uint32_t k = threadIdx.x; k < sizeof(DeviceDiag) / sizeof(unsigned long long); k += blockDim.x) to[k] = from[k];
}

void launch_batch_diag_gather(const ProblemView *v, uint32_t n, DeviceDiag *out, cudaStream_t s) {
  k_b_diag_gather<<<n, 32, 0, s>>>(v, out);
}

}  // namespace bgs
