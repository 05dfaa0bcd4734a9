// Census population control: comb_photons (census_functions.h:48-93) on the
// census a step left in the current bank.
//
// Upstream walks the census list once with one RNG: the comb energy is the
// list's left-to-right energy sum over max_census_photons; photon k takes
// the RNG's k-th draw and survives when it exceeds 1 - E/comb_E or when the
// photon is the only one left in its cell; survivors carry the comb energy,
// and then every survivor of a cell gets an equal share of the cell's
// energy defect (the cell's census energy, summed in list order, minus the
// comb energies handed out in it).
//
// On the device the only sequential pieces are the sums, which are kept in
// upstream order so the result is the same bits: the list total is one add
// chain (one block, staged through shared memory), and every cell runs the
// upstream loop over its own photons in list order.  A cell's photons are
// found by a stable radix sort of (cell, list position) pairs, the draw of
// photon k is Threefry at counter + k, so cells are independent.  Survivors
// are compacted stably into the other bank, which becomes current.
#include <cub/device/device_radix_sort.cuh>

#include "bgs_context.cuh"

namespace bgs {
namespace {

constexpr int kCombThreads = 256;
constexpr uint32_t kNoPhoton = 0xFFFFFFFFu;

// positions and cells of the census list, the radix sort's input
__global__ void k_comb_keys(const uint32_t *cell, uint32_t n, uint32_t *keys, uint32_t *pos) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    keys[k] = cell[k];
    pos[k] = k;
  }
}

// first and last sorted slot of every cell that holds census photons
__global__ void k_comb_bounds(const uint32_t *keys, uint32_t n, uint32_t *first, uint32_t *last) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const uint32_t c = keys[j];
    if (j == 0 || keys[j - 1] != c) first[c] = j;
    if (j + 1 == n || keys[j + 1] != c) last[c] = j;
  }
}

// get_photon_list_E (census_functions.h:40-46) as one add chain in list
// order, and the comb energy; also clears the census energy sum
__global__ void __launch_bounds__(kCombThreads) k_comb_total(const double *E, uint32_t n, double max_census,
                                                           double *comb, DeviceDiag *d) {
  constexpr int kChunk = 2048;
  __shared__ double s_e[kChunk];
  double total = 0.0;
  for (uint32_t base = 0; base < n; base += kChunk) {
    const uint32_t cnt = min((uint32_t)kChunk, n - base);
    for (uint32_t t = threadIdx.x; t < cnt; t += blockDim.x) s_e[t] = E[base + t];
    __syncthreads();
    if (threadIdx.x == 0)
      for (uint32_t t = 0; t < cnt; ++t) total += s_e[t];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    comb[0] = total;
    comb[1] = total / max_census;
    d->sum_census[0] = d->sum_census[1] = 0ULL;
  }
}

// the upstream loops of comb_photons restricted to one cell, over its
// photons in list order: the cell's energy, the survival decisions (draw k
// of the comb RNG for list position k), then the energy defect shared among
// the survivors.  Decisions are written to the census descriptors (CENSUS
// kept, KILLED combed away), survivor energies in place.
__global__ void k_comb_cells(Bank b, const uint32_t *pos, const uint32_t *first, const uint32_t *last,
                             uint32_t n_cells, const double *comb, unsigned long long seed_hi,
                             unsigned long long stream, unsigned long long counter) {
  const double comb_E = comb[1];
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += gridDim.x * blockDim.x) {
    const uint32_t j0 = first[c];
    if (j0 == kNoPhoton) continue;
    const uint32_t j1 = last[c];
    double cell_E = 0.0;
    for (uint32_t j = j0; j <= j1; ++j) cell_E += b.E[pos[j]];
    uint32_t count = j1 - j0 + 1;
    double corrected = 0.0;
    for (uint32_t j = j0; j <= j1; ++j) {
      const uint32_t k = pos[j];
      const double p_kill = 1.0 - b.E[k] / comb_E;
      const double u = u01_from_bits(threefry2x64_20_w0(counter + k, seed_hi, stream));
      if (u > p_kill || count == 1) {
        b.desc[k] = CENSUS;
        corrected += comb_E;
      } else {
        b.desc[k] = KILLED;
        --count;
      }
    }
    const double share = (cell_E - corrected) / (double)count;
    for (uint32_t j = j0; j <= j1; ++j) {
      const uint32_t k = pos[j];
      if (b.desc[k] == CENSUS) b.E[k] = comb_E + share;
    }
  }
}

// survivors copied stably into the other bank; their energy summed exactly
// in the census fixed point
__global__ void __launch_bounds__(kCombThreads) k_comb_copy(Bank from, Bank to, uint32_t n,
                                                          const unsigned long long *off, DeviceDiag *d) {
  const int sa = d->scale_abs;
  unsigned long long lo = 0, hi = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (from.desc[i] != CENSUS) continue;
    const unsigned long long j = off[i];
    to.px[j] = from.px[i]; to.py[j] = from.py[i]; to.pz[j] = from.pz[i];
    to.dx[j] = from.dx[i]; to.dy[j] = from.dy[i]; to.dz[j] = from.dz[i];
    to.E[j] = from.E[i]; to.E0[j] = from.E0[i]; to.life[j] = from.life[i];
    to.cell[j] = from.cell[i]; to.group[j] = from.group[i];
    to.desc[j] = CENSUS; to.stype[j] = from.stype[i];
    to.stream[j] = from.stream[i]; to.ctr[j] = from.ctr[i];
    unsigned long long vlo, vhi;
    if (to_fixed128(from.E[i], sa, vlo, vhi)) {
      lo += vlo;
      hi += vhi + (lo < vlo ? 1ULL : 0ULL);
    } else {
      atomicOr(&d->flags, (uint32_t)FLAG_TALLY_RANGE);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long l2 = __shfl_down_sync(0xffffffffu, lo, o);
    const unsigned long long h2 = __shfl_down_sync(0xffffffffu, hi, o);
    lo += l2;
    hi += h2 + (lo < l2 ? 1ULL : 0ULL);
  }
  if ((threadIdx.x & 31u) == 0 && (lo | hi)) atomic_add128(&d->sum_census[0], &d->sum_census[1], lo, hi);
}

// the combed census is the head of the next step's bank
__global__ void k_comb_finish(DeviceDiag *d, const unsigned long long *off, uint32_t n) {
  const unsigned long long kept = off[n];
  d->n_census_out = kept;
  d->n_census_in = kept;
  d->census_E = from_fixed128(d->sum_census[0], d->sum_census[1], d->scale_abs);
  d->census_E_in = d->census_E;
}

int grid_for(uint64_t n, int n_sm) {
  const uint64_t want = (n + kCombThreads - 1) / kCombThreads;
  const uint64_t cap = (uint64_t)n_sm * 8;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

// sort buffers sized for n census photons and the mesh's cells (kept
// between calls, grown on demand)
int comb_scratch(bgs_context *ctx, uint32_t n) {
  const uint32_t n_cells = ctx->mesh.n_cells;
  size_t temp = 0;
  if (cub::DeviceRadixSort::SortPairs(nullptr, temp, (const uint32_t *)nullptr, (uint32_t *)nullptr,
                                      (const uint32_t *)nullptr, (uint32_t *)nullptr, (int)n, 0, 32,
                                      ctx->stream) != cudaSuccess)
    return fail(ctx, BGS_ERR_CUDA, "radix sort size query failed");
  if (n <= ctx->comb_cap && n_cells <= ctx->comb_cells_cap && temp <= ctx->comb_temp_bytes) return BGS_OK;
  free_list(ctx->comb_allocs);
  ctx->comb_cap = ctx->comb_cells_cap = 0;
  ctx->comb_temp_bytes = 0;
  int rc;
  if ((rc = dev_alloc(ctx, ctx->comb_allocs, &ctx->comb_keys, 2 * (size_t)n)) ||
      (rc = dev_alloc(ctx, ctx->comb_allocs, &ctx->comb_pos, 2 * (size_t)n)) ||
      (rc = dev_alloc(ctx, ctx->comb_allocs, &ctx->comb_first, 2 * (size_t)n_cells)) ||
      (rc = dev_alloc(ctx, ctx->comb_allocs, &ctx->comb_scalars, 2)) ||
      (rc = dev_alloc(ctx, ctx->comb_allocs, &ctx->comb_temp, temp)))
    return rc;
  ctx->comb_cap = n;
  ctx->comb_cells_cap = n_cells;
  ctx->comb_temp_bytes = temp;
  return BGS_OK;
}

}  // namespace
}  // namespace bgs

extern "C" {

int bgs_comb_census(bgs_context *ctx, int64_t max_census_photons, uint32_t seed, uint64_t stream,
                    uint64_t *rng_counter, uint64_t *n_census) {
  if (!ctx || !rng_counter) return BGS_ERR_INVALID;
  if (!ctx->has_mesh) return fail(ctx, BGS_ERR_STATE, "no mesh");
  if (max_census_photons <= 0)
    return fail(ctx, BGS_ERR_INVALID, "max_census_photons must be positive (got %lld)",
                (long long)max_census_photons);
  if (!ctx->bank_is_census) return fail(ctx, BGS_ERR_STATE, "the bank does not hold a census");
  int rc = set_device(ctx);
  if (rc) return rc;
  if ((rc = read_diag(ctx))) return rc;
  const unsigned long long n64 = ctx->h_diag->n_census_in;
  if (n64 > 0xFFFFFFFEull) return fail(ctx, BGS_ERR_CAPACITY, "census of %llu photons is too large", n64);
  const uint32_t n = (uint32_t)n64;
  if (n == 0) {
    if (n_census) *n_census = 0;
    return BGS_OK;
  }
  if ((rc = comb_scratch(ctx, n))) return rc;
  cudaStream_t s = ctx->stream;
  Bank &from = ctx->bank[ctx->cur];
  Bank &to = ctx->bank[1 - ctx->cur];
  const uint32_t n_cells = ctx->mesh.n_cells;
  uint32_t *keys_in = ctx->comb_keys, *keys_out = ctx->comb_keys + n;
  uint32_t *pos_in = ctx->comb_pos, *pos_out = ctx->comb_pos + n;
  uint32_t *first = ctx->comb_first, *last = ctx->comb_first + n_cells;
  k_comb_keys<<<grid_for(n, ctx->n_sm), kCombThreads, 0, s>>>(from.cell, n, keys_in, pos_in);
  BGS_LAUNCHED(ctx, 1);
  int end_bit = 1;
  while (end_bit < 32 && (1ull << end_bit) < n_cells) ++end_bit;
  size_t temp = ctx->comb_temp_bytes;
  BGS_CUDA(ctx, cub::DeviceRadixSort::SortPairs(ctx->comb_temp, temp, keys_in, keys_out, pos_in, pos_out, (int)n,
                                                0, end_bit, s));
  BGS_CUDA(ctx, cudaMemsetAsync(first, 0xFF, (size_t)n_cells * sizeof(uint32_t), s));
  k_comb_bounds<<<grid_for(n, ctx->n_sm), kCombThreads, 0, s>>>(keys_out, n, first, last);
  k_comb_total<<<1, kCombThreads, 0, s>>>(from.E, n, (double)max_census_photons, ctx->comb_scalars, ctx->d_diag);
  k_comb_cells<<<grid_for(n_cells, ctx->n_sm), kCombThreads, 0, s>>>(
      from, pos_out, first, last, n_cells, ctx->comb_scalars, (unsigned long long)seed << 32, stream, *rng_counter);
  BGS_LAUNCHED(ctx, 3);
  launch_scan_flags(from.desc, CENSUS, (uint32_t)ctx->capacity, &ctx->d_diag->n_census_in, ctx->d_off_bank,
                    ctx->d_tile_bank, s);
  BGS_LAUNCHED(ctx, 3);
  k_comb_copy<<<grid_for(n, ctx->n_sm), kCombThreads, 0, s>>>(from, to, n, ctx->d_off_bank, ctx->d_diag);
  k_comb_finish<<<1, 1, 0, s>>>(ctx->d_diag, ctx->d_off_bank, n);
  BGS_LAUNCHED(ctx, 2);
  ctx->cur = 1 - ctx->cur;
  if ((rc = read_diag(ctx))) return rc;
  *rng_counter += n;  // one draw per census photon
  if (n_census) *n_census = ctx->h_diag->n_census_in;
  return check_flags(ctx, ctx->h_diag->flags);
}

}  // extern "C"
