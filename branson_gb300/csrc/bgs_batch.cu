// One persistent transport launch over many independent problems.
//
// Each problem keeps its own context (mesh, cell table, tallies, banks,
// device scalars); a device table of ProblemView descriptors points at
// them (the other phases of a batched step run as launches over the same
// table, one problem per blockIdx.y: bgs_mesh.cu, bgs_source.cu,
// bgs_transport.cu).  Work items are the concatenation of every problem's bank
// (exclusive prefix sum of the problems' n_bank, formed on the device, so
// no count goes through the host); each warp pulls items from one global
// queue, a lane finds its problem at pickup (forward from its last one) and then runs
// the history exactly as k_transport_history does (same per-segment code
// from bgs_physics.cuh, the problem's seed, tallies and fixed-point scales),
// so every problem's end states and tallies are those of its own launch.
// Small problems no longer leave the GPU idle: the tail of one overlaps the
// bulk of the others.
#include "bgs_physics.cuh"

namespace bgs {

constexpr int kItemThreads = 1024;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// work_counter[0]: queue head; [1], [2]: first block start and last block
// end of the batched launch (global timer, ns), so the launch can be timed
// inside a CUDA graph
__global__ void __launch_bounds__(kItemThreads) k_batch_items(const ProblemView *probs, uint32_t n,
                                                              unsigned long long *item_off,
                                                              unsigned long long *work_counter) {
  __shared__ unsigned long long s_warp[kItemThreads / 32];
  __shared__ unsigned long long s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t base = 0; base < n; base += kItemThreads) {
    const uint32_t p = base + threadIdx.x;
    const unsigned long long v = p < n ? probs[p].d->n_bank : 0ULL;
    unsigned long long incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (unsigned)o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      unsigned long long w = s_warp[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= (unsigned)o) w += t;
      }
      s_warp[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const unsigned long long before = s_carry + (warp > 0 ? s_warp[warp - 1] : 0ULL) + incl - v;
    if (p < n) item_off[p] = before;
    __syncthreads();
    if (threadIdx.x == kItemThreads - 1) s_carry = before + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    item_off[n] = s_carry;
    work_counter[0] = 0;
    work_counter[1] = ~0ULL;
    work_counter[2] = 0;
  }
}

// the batched kernel keeps the face planes ahead in registers: its mesh
// planes sit behind the problem's view, one more dependent load per segment
constexpr bool kBatchFaces = true;

#ifndef BGS_BATCH_MIN_BLOCKS
#define BGS_BATCH_MIN_BLOCKS 7
#endif

// flush visits taken from the ring, each into its own problem's tallies
// with that problem's scale; range flags go to that problem
__device__ __forceinline__ void flush_ring_batched(const ProblemView *__restrict__ probs, bool take,
                                                   unsigned long long key, double a, double t) {
  const uint32_t q = (uint32_t)(key >> 32), cell = (uint32_t)key;
  TallyCell *tally = take ? probs[q].c.tally : nullptr;
  const int sa = take ? probs[q].d->scale_abs : 0;
  uint32_t f = 0;
  flush_tally_warp(tally, take, key, cell, a, t, f, sa);
  if (f) atomicOr(&probs[q].d->flags, f);
}

template <bool kGray>
__global__ void __launch_bounds__(kTransportThreads, BGS_BATCH_MIN_BLOCKS)
    k_transport_batched(const ProblemView *__restrict__ probs, uint32_t n_probs,
                        const unsigned long long *__restrict__ item_off, unsigned long long *work_counter) {
  const unsigned long long n = item_off[n_probs];
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lanemask_lt = (1u << lane) - 1u;
  if (threadIdx.x == 0) atomicMin(&work_counter[1], global_ns());
  uint32_t flags = 0;
  uint32_t seg_acc = 0, seg_p = 0;  // segments of ended histories not yet counted, and their problem
  Lane L;
  uint32_t p = 0;
  const CellXS *xs_p = nullptr;
  bool active = false, done = false;
  __shared__ FlushRing rings[kTransportThreads / 32];
  FlushRing &ring = rings[threadIdx.x >> 5];
  uint32_t head = 0, tail = 0;  // the warp's ring counters (the same in every lane)

  while (true) {
    const unsigned need = __ballot_sync(0xffffffffu, !active && !done);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) base = atomicAdd(work_counter, (unsigned long long)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!active && !done) {
        const unsigned long long w = base + __popc(need & lanemask_lt);
        if (w < n) {
          // a lane's items only increase (the queue head only moves up), so
          // its problem is at or after the last one: a few steps forward,
          // else a binary search over the rest
          uint32_t k = 0;
          while (k < 4 && p + 1 < n_probs && item_off[p + 1] <= w) { ++p; ++k; }
          if (k == 4) p = problem_of(item_off, n_probs, w, p);
          const ProblemView &P = probs[p];
          const unsigned long long i = w - item_off[p];
          const Bank &b = P.from;
          L.idx = i;
          L.px = b.px[i]; L.py = b.py[i]; L.pz = b.pz[i];
          L.dx = b.dx[i]; L.dy = b.dy[i]; L.dz = b.dz[i];
          L.E = b.E[i]; L.life = b.life[i];
          L.cell = b.cell[i]; L.group = b.group[i];
          L.rng.stream = b.stream[i]; L.rng.ctr = b.ctr[i]; L.rng.hi = P.seed_hi;
          L.segs = 0;
          L.thr_abs = 0.0;
          set_birth(L, b.E0[i]);
          xs_p = P.c.xs;
          if (L.cell < P.m.n_cells) {
            locate<kBatchFaces>(P.m, L);
            active = true;
          } else {
            atomicOr(&P.d->flags, (uint32_t)FLAG_BAD_CELL);
            b.desc[i] = KILLED;
          }
        } else {
          done = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, !active)) break;

    // ---- one segment of transport_photon (history_based_transport.h:55-139);
    // ended cell visits wait in the warp's ring and go, 32 at a time,
    // through one warp-wide aggregated flush keyed on (problem, cell), as in
    // k_transport_history
    bool flush = false, ended = false;
    uint32_t fcell = 0;
    double fa = 0.0, ft = 0.0;
    if (active) {
      const CellXS xs = xs_p[L.cell];
      uint32_t surface_cross;
      const int ev = segment_advance<kBatchFaces>(probs[p].m, probs[p].from.E0, xs, L, surface_cross, flags);
      if (ev == SEG_SCATTER) {
        scatter_update<kBatchFaces, kGray>(probs[p].m, probs[p].c, xs, L);
      } else {
        const MeshDev &m = probs[p].m;
        int bc = ELEMENT;
        if (ev == SEG_BOUNDARY) bc = face_bc(m, L, surface_cross);
        if (ev != SEG_BOUNDARY || bc != REFLECT) {  // the visit to this cell ends
          flush = true;
          fcell = L.cell;
          fa = L.thr_abs;
          ft = visit_deposit(L, ev);
        }
        if (ev == SEG_KILLED || ev == SEG_CENSUS || bc == VACUUM || bc == SOURCE || bc == PROCESSOR) {
          const uint8_t desc = ev == SEG_KILLED ? KILLED
                             : ev == SEG_CENSUS ? CENSUS : (bc == PROCESSOR ? PASS : EXIT);
          store_end(probs[p].from, L, desc);
          ended = true;
        } else if (bc == ELEMENT) {
          L.thr_abs = 0.0;
          enter_neighbour<kBatchFaces>(m, L, surface_cross);
        } else {
          reflect<kBatchFaces>(m, L, surface_cross);
        }
      }
    }
    ring_push(ring, tail, tail, flush, ((unsigned long long)p << 32) | fcell, fa, ft);
    if (ended) {
      // a lane's segments are summed while its histories stay in one problem
      // and added to that problem's count when they move on (consecutive work
      // items mostly share a problem): one global atomic per history on the
      // problem's counter serialised the launch on short histories
      if (seg_acc && seg_p != p) {
        atomicAdd(&probs[seg_p].d->n_segments, (unsigned long long)seg_acc);
        seg_acc = 0;
      }
      seg_p = p;
      seg_acc += L.segs;  // a history adds at most 1e8: flushed below 2^31
      if (seg_acc >= (1u << 31)) {
        atomicAdd(&probs[p].d->n_segments, (unsigned long long)seg_acc);
        seg_acc = 0;
      }
      if (flags) {
        atomicOr(&probs[p].d->flags, flags);
        flags = 0;
      }
      active = false;
    }
    if (tail - head >= 32u) {
      unsigned long long key;
      double a, t;
      ring_take(ring, head, 32u, key, a, t);
      flush_ring_batched(probs, true, key, a, t);
      head += 32u;
    }
  }
  while (tail != head) {  // the visits still waiting
    const uint32_t k = min(tail - head, 32u);
    unsigned long long key;
    double a, t;
    const bool take = ring_take(ring, head, k, key, a, t);
    flush_ring_batched(probs, take, key, a, t);
    head += k;
  }
  if (seg_acc) atomicAdd(&probs[seg_p].d->n_segments, (unsigned long long)seg_acc);
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(&work_counter[2], global_ns());
}

TransportLaunch batch_launch_shape(int n_sm) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transport_batched<false>, kTransportThreads, 0) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  return {n_sm * per_sm, kTransportThreads};
}

void launch_batch_items(const ProblemView *probs, uint32_t n, unsigned long long *item_off,
                        unsigned long long *work_counter, cudaStream_t s) {
  k_batch_items<<<1, kItemThreads, 0, s>>>(probs, n, item_off, work_counter);
}

// gray: every problem has one group and no physical scattering (MeshDev::gray),
// so the lean build, with the same results, runs
void launch_transport_batched(const ProblemView *probs, uint32_t n, const unsigned long long *item_off,
                              unsigned long long *work_counter, const TransportLaunch &shape, bool gray,
                              cudaStream_t s) {
  if (gray)
    k_transport_batched<true><<<shape.blocks, shape.threads, 0, s>>>(probs, n, item_off, work_counter);
  else
    k_transport_batched<false><<<shape.blocks, shape.threads, 0, s>>>(probs, n, item_off, work_counter);
}

}  // namespace bgs
