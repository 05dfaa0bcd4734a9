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
#include "bgs_physics.cuh"

namespace bgs {

// Work items: bank indices 0..n-1, or (kResume) the indices of an event-mode
// active list, resumed with their carried per-cell tallies.  kThreads is the
// block size (64, 128 or 256, chosen by the tuner); every size keeps the
// register budget of BGS_MIN_BLOCKS blocks of 128 threads per SM.
template <int kThreads>
constexpr int min_blocks_for() {
  return (BGS_MIN_BLOCKS * 128 / kThreads) > 0 ? (BGS_MIN_BLOCKS * 128 / kThreads) : 1;
}

// Work items of one history launch: the whole bank (queue == nullptr: d's
// bank size and work counter), or bank entries [first, first + count) with
// their own counter (the pipelined drop-in transports a bank in chunks as
// its state arrives).
struct ItemRange {
  unsigned long long first, count;
  unsigned long long *queue;
};

// a lane's segment count, in 32 bits (one register): an ended history adds
// at most 1e8, and the count goes to the launch total before it reaches 2^31
__device__ __forceinline__ void add_segments(uint32_t &total, uint32_t segs, DeviceDiag *d) {
  total += segs;
  if (total >= (1u << 31)) {
    atomicAdd(&d->n_segments, (unsigned long long)total);
    total = 0;
  }
}

// Small meshes (kStagedCellsMax cells or fewer: 16 KB of per-cell data)
// run a build that keeps each block's cells in its shared memory: the whole
// per-cell transport table, copied in at launch and read by every segment,
// and the block's own 128-bit tallies, which its visit flushes add to with
// shared-memory atomics and which go to the global tallies once, when the
// block ends (few cells take every flush of the launch: global atomics on
// them queue in L2).  Integer sums do not depend on the order of the adds,
// so the tallies are the same bits.  Larger meshes keep both in global
// memory behind L1 (a block's lanes roam the whole mesh, so no smaller
// per-block set of cells exists to stage).
constexpr uint32_t kStagedCellsMax = 16384 / (sizeof(CellXS) + sizeof(TallyCell));
constexpr size_t staged_bytes(uint32_t n_cells) { return (size_t)n_cells * (sizeof(CellXS) + sizeof(TallyCell)); }

template <bool kResume, int kThreads, bool kGray = false, bool kStaged = false>
__global__ void __launch_bounds__(kThreads, min_blocks_for<kThreads>())
    k_transport_history(MeshDev m, CellsDev c, Bank b, DeviceDiag *d, unsigned long long seed_hi,
                        EventState es, ItemRange rg) {
  // kStaged: the mesh's n_cells CellXS entries, then the block's n_cells tallies
  extern __shared__ __align__(32) unsigned char staged[];
  CellXS *const staged_xs = reinterpret_cast<CellXS *>(staged);
  TallyCell *const staged_tally = reinterpret_cast<TallyCell *>(staged + (size_t)m.n_cells * sizeof(CellXS));
  TallyCell *const tally = kStaged ? staged_tally : c.tally;
  if constexpr (kStaged) {
    for (uint32_t g = threadIdx.x; g < m.n_cells; g += kThreads) {
      staged_xs[g] = c.xs[g];
      staged_tally[g] = TallyCell{0ULL, 0ULL, 0ULL, 0ULL};
    }
    __syncthreads();
  }
  const unsigned long long n = kResume ? (unsigned long long)*es.n_active : (rg.queue ? rg.count : d->n_bank);
  unsigned long long *const queue = rg.queue ? rg.queue : &d->work_counter;
  const int sa = d->scale_abs;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lanemask_lt = (1u << lane) - 1u;
  uint32_t flags = 0;
  uint32_t seg_total = 0;  // segments of this lane's ended histories (kept below 2^31)
  Lane L;
  bool active = false, done = false;
  __shared__ FlushRing rings[kThreads / 32];
  FlushRing &ring = rings[threadIdx.x >> 5];
  uint32_t head = 0, tail = 0;  // the warp's ring counters (the same in every lane)

  while (true) {
    // ---- refill lanes whose history ended
    const unsigned need = __ballot_sync(0xffffffffu, !active && !done);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) base = atomicAdd(queue, (unsigned long long)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!active && !done) {
        const unsigned long long w = base + __popc(need & lanemask_lt);
        if (w < n) {
          const unsigned long long i = kResume ? (unsigned long long)es.active[w] : rg.first + w;
          L.idx = i;
          L.px = b.px[i]; L.py = b.py[i]; L.pz = b.pz[i];
          L.dx = b.dx[i]; L.dy = b.dy[i]; L.dz = b.dz[i];
          L.E = b.E[i]; L.life = b.life[i];
          L.cell = b.cell[i]; L.group = b.group[i];
          L.rng.stream = b.stream[i]; L.rng.ctr = b.ctr[i]; L.rng.hi = seed_hi;
          L.segs = 0;
          if (kResume) {
            L.thr_abs = es.thr_abs[i];
          } else {
            L.thr_abs = 0.0;
          }
          set_birth(L, b.E0[i]);
          if (L.cell < m.n_cells) {
            locate(m, L);
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

    // ---- one segment of transport_photon (history_based_transport.h:55-139);
    // ended cell visits wait in the warp's ring, and every 32 of them go
    // through one warp-wide aggregated flush (FlushRing)
    bool flush = false;
    uint32_t fcell = 0;
    double fa = 0.0, ft = 0.0;
    if (active) {
      const CellXS xs = kStaged ? staged_xs[L.cell] : c.xs[L.cell];
      uint32_t surface_cross;
      const int ev = segment_advance(m, b.E0, xs, L, surface_cross, flags);
      if (ev == SEG_SCATTER) {
        scatter_update<false, kGray>(m, c, xs, L);
      } else {
        int bc = ELEMENT;
        if (ev == SEG_BOUNDARY) bc = face_bc(m, L, surface_cross);
        const bool moves_on = ev == SEG_BOUNDARY && bc == ELEMENT;
        const bool turns = ev == SEG_BOUNDARY && bc == REFLECT;
        if (!turns) {  // the visit to this cell ends
          flush = true;
          fcell = L.cell;
          fa = L.thr_abs;
          ft = visit_deposit(L, ev);
        }
        if (moves_on) {
          L.thr_abs = 0.0;
          enter_neighbour(m, L, surface_cross);
        } else if (turns) {
          reflect(m, L, surface_cross);
        } else {  // the history ends: cutoff kill, census, or out through a domain face
          const uint8_t desc = ev == SEG_KILLED ? KILLED : (ev == SEG_CENSUS ? CENSUS : (bc == PROCESSOR ? PASS : EXIT));
          store_end(b, L, desc);
          active = false;
          add_segments(seg_total, L.segs, d);
        }
      }
    }
    ring_push(ring, tail, tail, flush, fcell, fa, ft);
    if (tail - head >= 32u) {
      unsigned long long key;
      double a, t;
      ring_take(ring, head, 32u, key, a, t);
      flush_tally_warp(tally, true, (uint32_t)key, (uint32_t)key, a, t, flags, sa);
      head += 32u;
    }
  }
  while (tail != head) {  // the visits still waiting
    const uint32_t k = min(tail - head, 32u);
    unsigned long long key;
    double a, t;
    const bool take = ring_take(ring, head, k, key, a, t);
    flush_tally_warp(tally, take, (uint32_t)key, (uint32_t)key, a, t, flags, sa);
    head += k;
  }
  if constexpr (kStaged) {  // the block's tallies into the global ones
    __syncthreads();
    for (uint32_t g = threadIdx.x; g < m.n_cells; g += kThreads) {
      const TallyCell s = staged_tally[g];
      TallyCell *tc = &c.tally[g];
      if (s.abs_lo | s.abs_hi) atomic_add128(&tc->abs_lo, &tc->abs_hi, s.abs_lo, s.abs_hi);
      if (s.dep_lo | s.dep_hi) atomic_add128(&tc->dep_lo, &tc->dep_hi, s.dep_lo, s.dep_hi);
    }
  }

  // ---- per-warp totals
  unsigned long long segs = seg_total;
  for (int o = 16; o > 0; o >>= 1) {
    segs += __shfl_down_sync(0xffffffffu, segs, o);
    flags |= __shfl_down_sync(0xffffffffu, flags, o);
  }
  if (lane == 0) {
    atomicAdd(&d->n_segments, segs);
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

__device__ __forceinline__ void census_body(const Bank &from, const Bank &to, DeviceDiag *d,
                                            const unsigned long long *off, double next_dt, uint32_t bx,
                                            uint32_t nbx) {
  const unsigned long long n = d->n_bank;
  const int sa = d->scale_abs;
  const double life = kC * next_dt;
  unsigned long long c_lo = 0, c_hi = 0, e_lo = 0, e_hi = 0;
  for (unsigned long long i = bx * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)nbx * blockDim.x) {
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

__global__ void k_census(Bank from, Bank to, DeviceDiag *d, const unsigned long long *off, double next_dt) {
  census_body(from, to, d, off, next_dt, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void census_finish_body(DeviceDiag *d, const unsigned long long *off) {
  const unsigned long long n_out = off[d->n_bank];
  d->n_census_out = n_out;
  d->census_E = from_fixed128(d->sum_census[0], d->sum_census[1], d->scale_abs);
  d->exit_E = from_fixed128(d->sum_exit[0], d->sum_exit[1], d->scale_abs);
  // the census becomes the head of the next step's bank
  d->n_census_in = n_out;
  d->census_E_in = d->census_E;
}

__global__ void k_census_finish(DeviceDiag *d, const unsigned long long *off) { census_finish_body(d, off); }

__global__ void __launch_bounds__(256) k_b_census(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  census_body(P.from, P.to, P.d, P.off_bank, P.next_dt, blockIdx.x, gridDim.x);
}

__global__ void k_b_census_finish(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  if (threadIdx.x == 0) census_finish_body(P.d, P.off_bank);
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
template <int kThreads>
int history_blocks_per_sm() {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transport_history<false, kThreads>, kThreads, 0) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  return per_sm;
}

TransportLaunch transport_launch_shape(int n_sm, int threads) {
  switch (threads) {
    case 64: return {n_sm * history_blocks_per_sm<64>(), 64};
    case 256: return {n_sm * history_blocks_per_sm<256>(), 256};
    default: return {n_sm * history_blocks_per_sm<128>(), 128};
  }
}

// the whole-bank builds: gray or not, the cell table staged in shared
// memory or not (the same arithmetic, so the same results)
template <int kThreads, bool kGray>
void launch_history_whole(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d,
                          unsigned long long seed_hi, const EventState &es, const ItemRange &rg, int blocks,
                          cudaStream_t s) {
  if (m.n_cells <= kStagedCellsMax) {
    k_transport_history<false, kThreads, kGray, true>
        <<<blocks, kThreads, staged_bytes(m.n_cells), s>>>(m, c, b, d, seed_hi, es, rg);
  } else {
    k_transport_history<false, kThreads, kGray><<<blocks, kThreads, 0, s>>>(m, c, b, d, seed_hi, es, rg);
  }
}

template <bool kResume>
void launch_history_kernel(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d,
                           unsigned long long seed_hi, const EventState &es, const ItemRange &rg,
                           const TransportLaunch &shape, cudaStream_t s) {
  if (!kResume) {  // gray (one group, no physical scattering): the lean build, same results
    switch (shape.threads) {
      case 64:
        if (m.gray) launch_history_whole<64, true>(m, c, b, d, seed_hi, es, rg, shape.blocks, s);
        else launch_history_whole<64, false>(m, c, b, d, seed_hi, es, rg, shape.blocks, s);
        return;
      case 256:
        if (m.gray) launch_history_whole<256, true>(m, c, b, d, seed_hi, es, rg, shape.blocks, s);
        else launch_history_whole<256, false>(m, c, b, d, seed_hi, es, rg, shape.blocks, s);
        return;
      default:
        if (m.gray) launch_history_whole<128, true>(m, c, b, d, seed_hi, es, rg, shape.blocks, s);
        else launch_history_whole<128, false>(m, c, b, d, seed_hi, es, rg, shape.blocks, s);
        return;
    }
  }
  switch (shape.threads) {
    case 64:
      k_transport_history<kResume, 64><<<shape.blocks, 64, 0, s>>>(m, c, b, d, seed_hi, es, rg);
      break;
    case 256:
      k_transport_history<kResume, 256><<<shape.blocks, 256, 0, s>>>(m, c, b, d, seed_hi, es, rg);
      break;
    default:
      k_transport_history<kResume, 128><<<shape.blocks, 128, 0, s>>>(m, c, b, d, seed_hi, es, rg);
      break;
  }
}

void launch_transport_history(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d,
                              uint32_t seed, const TransportLaunch &shape, cudaStream_t s) {
  launch_history_kernel<false>(m, c, b, d, (unsigned long long)seed << 32, EventState{}, ItemRange{0, 0, nullptr},
                               shape, s);
}

void launch_transport_history_range(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d,
                                    uint32_t seed, unsigned long long first, unsigned long long count,
                                    unsigned long long *queue, const TransportLaunch &shape, cudaStream_t s) {
  launch_history_kernel<false>(m, c, b, d, (unsigned long long)seed << 32, EventState{},
                               ItemRange{first, count, queue}, shape, s);
}

void launch_transport_resume(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d,
                             uint32_t seed, const EventState &es, const TransportLaunch &shape,
                             cudaStream_t s) {
  launch_history_kernel<true>(m, c, b, d, (unsigned long long)seed << 32, es, ItemRange{0, 0, nullptr}, shape, s);
}

void launch_census(const Bank &from, const Bank &to, DeviceDiag *d, const unsigned long long *off,
                   double next_dt, int n_sm, cudaStream_t s) {
  cudaMemsetAsync(d->sum_census, 0, sizeof(d->sum_census), s);
  cudaMemsetAsync(d->sum_exit, 0, sizeof(d->sum_exit), s);
  k_census<<<n_sm * 4, 256, 0, s>>>(from, to, d, off, next_dt);
  k_census_finish<<<1, 1, 0, s>>>(d, off);
}

void launch_batch_census(const ProblemView *v, const BatchGrid &g, cudaStream_t s) {
  k_b_census<<<dim3(g.photons, g.n), 256, 0, s>>>(v);
  k_b_census_finish<<<dim3(1, g.n), 32, 0, s>>>(v);
}

}  // namespace bgs
