// History-based IMC transport on sm_103a (transport_photon,
// history_based_transport.h:33-141) and census post-processing
// (post_process_photons, post_process_functions.h:33-109).
//
// Execution model: a persistent grid sized to the SM count; each warp pulls
// histories from a device-side queue, one per lane, and refills a lane the
// moment its history ends (warp-aggregated atomic on the queue head), so a
// warp advances 32 live histories one segment per loop trip instead of
// waiting for its longest history.  Photon state stays in registers for the
// whole history; the bank (structure of arrays) is read once at pickup and
// written once at the end.  Per-cell tallies are 128-bit fixed-point integer
// atomics flushed when a history leaves a cell or ends, exactly where the
// upstream loop flushes its thread-local tallies, so the sums are exact and
// independent of thread order.
//
// Arithmetic is FP64 in the upstream operation order (the translation unit
// is built without FMA contraction); the per-cell coefficients come from the
// CellXS table, formed with the same expressions as the upstream loop.
#include "bgs_fixmath.cuh"
#include "bgs_kernels.cuh"

namespace bgs {

constexpr int kTransportThreads = 128;
// Build-time choices for the per-segment arithmetic (see the header comment
// of bgs_fixmath.cuh): integer or FP64 for the divisions, the square root
// and sin/cos, and the minimum number of resident blocks per SM.
#ifndef BGS_INT_DIV
#define BGS_INT_DIV 0
#endif
#ifndef BGS_INT_SQRT
#define BGS_INT_SQRT 1
#endif
#ifndef BGS_INT_SINCOS
#define BGS_INT_SINCOS 1
#endif
#ifndef BGS_MIN_BLOCKS
#define BGS_MIN_BLOCKS 5
#endif
#ifndef BGS_INT_DIV_DS
#define BGS_INT_DIV_DS 0  // -log(u)/sigma_eff by the exact integer division (per-cell reciprocal)
#endif
#ifndef BGS_SPEC_DRAWS
#define BGS_SPEC_DRAWS 0  // draw the scattering angles with the collision distance (3 at once)
#endif

__device__ __forceinline__ double seg_div(double a, double b, unsigned long long rb) {
#if BGS_INT_DIV
  return fix::div_rn(a, b, rb);
#else
  (void)rb;
  return a / b;
#endif
}
__device__ __forceinline__ double seg_sqrt(double x) {
#if BGS_INT_SQRT
  return fix::sqrt_rn(x);
#else
  return sqrt(x);
#endif
}
__device__ __forceinline__ void seg_sincos(double phi, double *s, double *c) {
#if BGS_INT_SINCOS
  fix::sincos_phi(phi, s, c);
#else
  sincos(phi, s, c);
#endif
}

struct Lane {
  double px, py, pz, dx, dy, dz, E, E0, life, inv_E0;
  unsigned long long rbx, rby, rbz;  // divisor reciprocals of the direction cosines
  double n0, n1, n2, n3, n4, n5;  // nodes of the current cell
  double thr_abs, thr_trk;
  unsigned long long idx;
  Rng rng;
  uint32_t cell, group, ci, cj, ck, segs;
};

__device__ __forceinline__ void load_nodes(const MeshDev &m, Lane &L) {
  L.n0 = m.x[L.ci]; L.n1 = m.x[L.ci + 1];
  L.n2 = m.y[L.cj]; L.n3 = m.y[L.cj + 1];
  L.n4 = m.z[L.ck]; L.n5 = m.z[L.ck + 1];
}

__device__ __forceinline__ void flush_tally(const CellsDev &c, const DeviceDiag *d, uint32_t cell,
                                            double a, double t, uint32_t &flags, int sa, int st) {
  unsigned long long lo, hi;
  TallyCell *tc = &c.tally[cell];
  if (a != 0.0) {
    if (to_fixed128(a, sa, lo, hi)) atomic_add128(&tc->abs_lo, &tc->abs_hi, lo, hi);
    else flags |= (a == a) ? FLAG_TALLY_RANGE : FLAG_NAN;
  }
  if (t != 0.0) {
    if (to_fixed128(t, st, lo, hi)) atomic_add128(&tc->trk_lo, &tc->trk_hi, lo, hi);
    else flags |= (t == t) ? FLAG_TALLY_RANGE : FLAG_NAN;
  }
}

__device__ __forceinline__ void direction_recips(Lane &L) {

#if BGS_INT_DIV
  L.rbx = fix::divisor_recip(L.dx);
  L.rby = fix::divisor_recip(L.dy);
  L.rbz = fix::divisor_recip(L.dz);
#else
  (void)L;
#endif
}

__device__ __forceinline__ void store_end(const Bank &b, const Lane &L, uint8_t desc) {
  const unsigned long long i = L.idx;
  b.px[i] = L.px; b.py[i] = L.py; b.pz[i] = L.pz;
  b.dx[i] = L.dx; b.dy[i] = L.dy; b.dz[i] = L.dz;
  b.E[i] = L.E; b.life[i] = L.life;
  b.cell[i] = L.cell; b.group[i] = L.group;
  b.desc[i] = desc; b.ctr[i] = L.rng.ctr;
}

// sample_emission_group, Cell version (sampling_functions.h:126-138) with
// all groups at the same opacity: walk the CDF in steps of v; a walk that
// would run past the last group stays in the last group.
__device__ __forceinline__ uint32_t sample_group(Rng &r, double v, uint32_t n_groups) {
  double cdf = r.next();
  int g = -1;
  while (cdf > 0) {
    ++g;
    cdf -= v;
    if ((uint32_t)g == n_groups - 1) break;
  }
  return g < 0 ? 0u : (uint32_t)g;
}

__global__ void __launch_bounds__(kTransportThreads, BGS_MIN_BLOCKS)
    k_transport_history(MeshDev m, CellsDev c, Bank b, DeviceDiag *d, unsigned long long seed_hi) {
  const unsigned long long n = d->n_bank;
  const int sa = d->scale_abs, st = d->scale_track;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lanemask_lt = (1u << lane) - 1u;
  uint32_t flags = 0;
  unsigned long long seg_total = 0;
  Lane L;
  bool active = false, done = false;

  while (true) {
    // ---- refill lanes whose history ended
    const unsigned need = __ballot_sync(0xffffffffu, !active && !done);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) base = atomicAdd(&d->work_counter, (unsigned long long)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!active && !done) {
        const unsigned long long i = base + __popc(need & lanemask_lt);
        if (i < n) {
          L.idx = i;
          L.px = b.px[i]; L.py = b.py[i]; L.pz = b.pz[i];
          L.dx = b.dx[i]; L.dy = b.dy[i]; L.dz = b.dz[i];
          L.E = b.E[i]; L.E0 = b.E0[i]; L.life = b.life[i];
          L.cell = b.cell[i]; L.group = b.group[i];
          L.rng.stream = b.stream[i]; L.rng.ctr = b.ctr[i]; L.rng.hi = seed_hi;
          L.thr_abs = 0.0; L.thr_trk = 0.0; L.segs = 0;
          L.inv_E0 = 1.0 / L.E0;
          direction_recips(L);
          if (L.cell < m.n_cells) {
            L.ci = L.cell % m.ngx; L.cj = (L.cell / m.ngx) % m.ngy; L.ck = L.cell / (m.ngx * m.ngy);
            load_nodes(m, L);
            active = true;
          } else {
            flags |= FLAG_BAD_CELL;
            b.desc[i] = KILLED;
          }
        } else {
          done = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, !active)) break;
    if (!active) continue;

    // ---- one segment of transport_photon (history_based_transport.h:55-139)
    ++L.segs;
    ++seg_total;
    const CellXS xs = c.xs[L.cell];
    // -log(u) / sigma_eff with the integer, correctly rounded -log (bgs_fixmath.cuh)
    // (divisions are the exact integer div_rn: bitwise the IEEE quotient)
#if BGS_SPEC_DRAWS
    // the collision draw and, speculatively, the two angle draws that a
    // scatter would take next: three independent Threefry evaluations
    unsigned long long w_mu = 0, w_phi = 0;
    unsigned long long m_ds = 0;
    if (xs.sig_eff > 0.0) {
      const unsigned long long w0 = L.rng.peek(0);
      w_mu = L.rng.peek(1);
      w_phi = L.rng.peek(2);
      L.rng.skip();
      m_ds = (w0 >> 11) | 1ULL;
    }
    const double dist_to_scatter =
        (xs.sig_eff > 0.0) ? fix::div_rn(fix::neg_log_u53(m_ds), xs.sig_eff, xs.rb_sig) : 1.0e100;
#elif BGS_INT_DIV_DS
    const double dist_to_scatter =
        (xs.sig_eff > 0.0) ? fix::div_rn(fix::neg_log_u53(L.rng.next_m53()), xs.sig_eff, xs.rb_sig)
                           : 1.0e100;
#else
    const double dist_to_scatter =
        (xs.sig_eff > 0.0) ? fix::neg_log_u53(L.rng.next_m53()) / xs.sig_eff : 1.0e100;
#endif
    // Cell::get_distance_to_boundary (cell.h:117-132)
    double dist_to_boundary = 1.0e16;
    uint32_t surface_cross = 0;
    const bool posx = 0.0 < L.dx, posy = 0.0 < L.dy, posz = 0.0 < L.dz;
    const double numx = (posx ? L.n1 : L.n0) - L.px;
    const double numy = (posy ? L.n3 : L.n2) - L.py;
    const double numz = (posz ? L.n5 : L.n4) - L.pz;
    {
      double dist = seg_div(numx, L.dx, L.rbx);
      if (dist < dist_to_boundary) { dist_to_boundary = dist; surface_cross = posx ? 1u : 0u; }
      dist = seg_div(numy, L.dy, L.rby);
      if (dist < dist_to_boundary) { dist_to_boundary = dist; surface_cross = posy ? 3u : 2u; }
      dist = seg_div(numz, L.dz, L.rbz);
      if (dist < dist_to_boundary) { dist_to_boundary = dist; surface_cross = posz ? 5u : 4u; }
    }
    const double dist_to_census = L.life;
    // std::min(a, b) == (b < a) ? b : a; the event tests that follow
    // (dist_to_event == dist_to_scatter, then == dist_to_boundary) are the
    // same comparisons read back
    const bool census_first = dist_to_census < dist_to_boundary;
    const double inner = census_first ? dist_to_census : dist_to_boundary;
    const bool inner_first = inner < dist_to_scatter;
    const double dist_to_event = inner_first ? inner : dist_to_scatter;

    const double absorbed_E = L.E * (1.0 - fix::exp_neg(-(xs.neg_saf * dist_to_event)));
    L.thr_abs += absorbed_E;
    L.thr_trk += absorbed_E * xs.inv_saf;
    L.E = L.E - absorbed_E;
    L.px += L.dx * dist_to_event;  // Photon::move (photon.h:109-114)
    L.py += L.dy * dist_to_event;
    L.pz += L.dz * dist_to_event;
    L.life -= dist_to_event;

    // below_cutoff: E/E0 < 0.01 (photon.h:47-49), decided from E*(1/E0) and
    // settled with the exact quotient only within a few ulps of the threshold
    const double frac = L.E * L.inv_E0;
    bool killed = frac < kCutoff;
    if (fabs(frac - kCutoff) <= 4.0e-18) killed = L.E / L.E0 < kCutoff;
    if (killed || L.segs >= kMaxSegmentsPerHistory) {
      if (!killed) flags |= FLAG_SEGMENT_LIMIT;
      L.thr_abs += L.E;
      flush_tally(c, d, L.cell, L.thr_abs, L.thr_trk, flags, sa, st);
      store_end(b, L, KILLED);
      active = false;
    } else if (!inner_first) {  // dist_to_event == dist_to_scatter
      // get_uniform_angle (sampling_functions.h:57-70)
#if BGS_SPEC_DRAWS
      const double mu = mu_from_m53((w_mu >> 11) | 1ULL);
      const double phi = u01_from_bits(w_phi) * 2.0 * kPi;
      L.rng.skip();
      L.rng.skip();
#else
      const double mu = mu_from_m53(L.rng.next_m53());
      const double phi = L.rng.next() * 2.0 * kPi;
#endif
      const double sin_theta = seg_sqrt(1.0 - mu * mu);
      double sp, cp;
      seg_sincos(phi, &sp, &cp);
      L.dx = sin_theta * cp;
      L.dy = sin_theta * sp;
      L.dz = mu;
      direction_recips(L);
      // effective-scatter test and group resample (history_based_transport.h:97-98):
      // with sigma_s = 0 the test u > 0 always passes, and with one group the
      // walk always ends in group 0, so those draws only advance the counter
      bool resample;
      if (xs.p_scat > 0.0) resample = L.rng.next() > xs.p_scat;
      else { L.rng.skip(); resample = true; }
      if (resample) {
        if (m.n_groups > 1) L.group = sample_group(L.rng, c.group_v[L.cell], m.n_groups);
        else { L.rng.skip(); L.group = 0; }
      }
    } else if (!census_first) {  // dist_to_event == dist_to_boundary
      // structured-mesh face: interior faces are ELEMENT (proto_mesh.h:156-202)
      bool interior;
      switch (surface_cross) {
        case 0: interior = L.ci > 0; break;
        case 1: interior = L.ci + 1 < m.ngx; break;
        case 2: interior = L.cj > 0; break;
        case 3: interior = L.cj + 1 < m.ngy; break;
        case 4: interior = L.ck > 0; break;
        default: interior = L.ck + 1 < m.ngz; break;
      }
      const int bc = interior ? ELEMENT : m.bc[surface_cross];
      if (bc == ELEMENT) {
        flush_tally(c, d, L.cell, L.thr_abs, L.thr_trk, flags, sa, st);
        L.thr_abs = 0.0;
        L.thr_trk = 0.0;
        switch (surface_cross) {
          case 0: --L.ci; L.cell -= 1; break;
          case 1: ++L.ci; L.cell += 1; break;
          case 2: --L.cj; L.cell -= m.ngx; break;
          case 3: ++L.cj; L.cell += m.ngx; break;
          case 4: --L.ck; L.cell -= m.ngx * m.ngy; break;
          default: ++L.ck; L.cell += m.ngx * m.ngy; break;
        }
        load_nodes(m, L);
      } else if (bc == VACUUM || bc == SOURCE || bc == PROCESSOR) {
        flush_tally(c, d, L.cell, L.thr_abs, L.thr_trk, flags, sa, st);
        store_end(b, L, bc == PROCESSOR ? PASS : EXIT);
        active = false;
      } else {  // REFLECT: Photon::reflect (photon.h:151-155)
        if (surface_cross < 2) L.dx = -L.dx;
        else if (surface_cross < 4) L.dy = -L.dy;
        else L.dz = -L.dz;
      }
    } else {  // dist_to_event == dist_to_census
      flush_tally(c, d, L.cell, L.thr_abs, L.thr_trk, flags, sa, st);
      store_end(b, L, CENSUS);
      active = false;
    }
  }

  // ---- per-warp totals
  for (int o = 16; o > 0; o >>= 1) {
    seg_total += __shfl_down_sync(0xffffffffu, seg_total, o);
    flags |= __shfl_down_sync(0xffffffffu, flags, o);
  }
  if (lane == 0) {
    atomicAdd(&d->n_segments, seg_total);
    if (flags) atomicOr(&d->flags, flags);
  }
}

// ---------------------------------------------------------------------------
// post_process_photons (post_process_functions.h:62-109): census photons
// copied in bank order into the other bank with life_dx = c*next_dt (the
// end state in the source bank gets the same reset, as upstream, where the
// reset happens in place before the copy), census and exit energies summed
// exactly in fixed point.
__device__ __forceinline__ void block_sum128(unsigned long long lo, unsigned long long hi,
                                             unsigned long long *dst);

__global__ void k_census(Bank from, Bank to, DeviceDiag *d, const unsigned long long *off,
                         double next_dt) {
  const unsigned long long n = d->n_bank;
  const int sa = d->scale_abs;
  const double life = kC * next_dt;
  unsigned long long c_lo = 0, c_hi = 0, e_lo = 0, e_hi = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const uint8_t desc = from.desc[i];
    unsigned long long lo, hi;
    if (desc == CENSUS) {
      const unsigned long long j = off[i];
      from.life[i] = life;
      to.px[j] = from.px[i]; to.py[j] = from.py[i]; to.pz[j] = from.pz[i];
      to.dx[j] = from.dx[i]; to.dy[j] = from.dy[i]; to.dz[j] = from.dz[i];
      to.E[j] = from.E[i]; to.E0[j] = from.E0[i]; to.life[j] = life;
      to.cell[j] = from.cell[i]; to.group[j] = from.group[i];
      to.desc[j] = CENSUS; to.stype[j] = from.stype[i];
      to.stream[j] = from.stream[i]; to.ctr[j] = from.ctr[i];
      to_fixed128(from.E[i], sa, lo, hi);
      const unsigned long long o = c_lo;
      c_lo += lo;
      c_hi += hi + (c_lo < o ? 1ULL : 0ULL);
    } else if (desc == EXIT) {
      to_fixed128(from.E[i], sa, lo, hi);
      const unsigned long long o = e_lo;
      e_lo += lo;
      e_hi += hi + (e_lo < o ? 1ULL : 0ULL);
    }
  }
  block_sum128(c_lo, c_hi, d->sum_census);
  block_sum128(e_lo, e_hi, d->sum_exit);
}

__global__ void k_census_finish(DeviceDiag *d, const unsigned long long *off) {
  const unsigned long long n_out = off[d->n_bank];
  d->n_census_out = n_out;
  d->census_E = from_fixed128(d->sum_census[0], d->sum_census[1], d->scale_abs);
  d->exit_E = from_fixed128(d->sum_exit[0], d->sum_exit[1], d->scale_abs);
  // the census becomes the head of the next step's bank
  d->n_census_in = n_out;
  d->census_E_in = d->census_E;
}

// 128-bit block sum via 43-bit limbs (exact for up to 2^21 terms per block)
__device__ __forceinline__ void block_sum128(unsigned long long lo, unsigned long long hi,
                                             unsigned long long *dst) {
  const unsigned long long M = (1ULL << 43) - 1ULL;
  unsigned long long a0 = lo & M, a1 = ((lo >> 43) | (hi << 21)) & M, a2 = hi >> 22;
  __shared__ unsigned long long s[3][32];
  for (int o = 16; o > 0; o >>= 1) {
    a0 += __shfl_down_sync(0xffffffffu, a0, o);
    a1 += __shfl_down_sync(0xffffffffu, a1, o);
    a2 += __shfl_down_sync(0xffffffffu, a2, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) { s[0][warp] = a0; s[1][warp] = a1; s[2][warp] = a2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b0 = 0, b1 = 0, b2 = 0;
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) { b0 += s[0][w]; b1 += s[1][w]; b2 += s[2][w]; }
    unsigned long long rlo = b0, rhi = 0;
    const unsigned long long t1 = b1 << 43, o = rlo;
    rlo += t1;
    rhi += (rlo < o) ? 1ULL : 0ULL;
    rhi += (b1 >> 21) + (b2 << 22);
    atomic_add128(&dst[0], &dst[1], rlo, rhi);
  }
}

// ---------------------------------------------------------------------------
TransportLaunch transport_launch_shape(int n_sm) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transport_history, kTransportThreads, 0);
  if (per_sm < 1) per_sm = 1;
  return {n_sm * per_sm, kTransportThreads};
}

void launch_transport_history(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d,
                              uint32_t seed, const TransportLaunch &shape, cudaStream_t s) {
  const unsigned long long seed_hi = (unsigned long long)seed << 32;
  k_transport_history<<<shape.blocks, shape.threads, 0, s>>>(m, c, b, d, seed_hi);
}

void launch_census(const Bank &from, const Bank &to, DeviceDiag *d, const unsigned long long *off,
                   double next_dt, int n_sm, cudaStream_t s) {
  cudaMemsetAsync(d->sum_census, 0, sizeof(d->sum_census), s);
  cudaMemsetAsync(d->sum_exit, 0, sizeof(d->sum_exit), s);
  k_census<<<n_sm * 4, 256, 0, s>>>(from, to, d, off, next_dt);
  k_census_finish<<<1, 1, 0, s>>>(d, off);
}

}  // namespace bgs
