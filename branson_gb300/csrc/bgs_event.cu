// Event-based transport (the upstream event mode, event_based_transport.h:
// 32-381, restated as GPU stages).  Each round advances every active photon
// by one segment and sorts the outcomes into per-event queues; the scatter
// and boundary stages then run over their own queue, so every warp executes
// one branch of the segment with all lanes active.  Survivors form the next
// round's active list.  Stages share the per-segment arithmetic of the
// history kernel (bgs_physics.cuh), so each photon's end state is the same
// as in history mode.
//
// Per round the photon state makes one trip through HBM (about 200 bytes
// read and written per segment); the host runs rounds until the active set
// is small and hands the tail to the history kernel (launch_transport_resume),
// which continues each photon with its carried per-cell tallies.
#include "bgs_physics.cuh"

namespace bgs {

constexpr int kEventThreads = 256;

// warp-aggregated append of index p to a queue (one atomic per warp)
__device__ __forceinline__ void queue_push(bool want, uint32_t p, uint32_t *q, unsigned int *n) {
  const unsigned mask = __ballot_sync(0xffffffffu, want);
  if (!mask) return;
  const unsigned lane = threadIdx.x & 31u;
  const int leader = __ffs(mask) - 1;
  unsigned int base = 0;
  if ((int)lane == leader) base = atomicAdd(n, (unsigned int)__popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (want) q[base + __popc(mask & ((1u << lane) - 1u))] = p;
}

__device__ __forceinline__ void load_lane(const MeshDev &m, const Bank &b, const EventState &es,
                                          uint32_t p, unsigned long long seed_hi, bool first, Lane &L) {
  L.idx = p;
  L.px = b.px[p]; L.py = b.py[p]; L.pz = b.pz[p];
  L.dx = b.dx[p]; L.dy = b.dy[p]; L.dz = b.dz[p];
  L.E = b.E[p]; L.life = b.life[p];
  L.cell = b.cell[p]; L.group = b.group[p];
  L.rng.stream = b.stream[p]; L.rng.ctr = b.ctr[p]; L.rng.hi = seed_hi;
  L.thr_abs = first ? 0.0 : es.thr_abs[p];
  set_birth(L, b.E0[p]);
  L.segs = 0;
  locate(m, L);
}

__global__ void k_event_init(EventState es, const DeviceDiag *d) {
  const unsigned long long n = d->n_bank;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x)
    es.active[i] = (uint32_t)i;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *es.n_active = (unsigned int)n;
    *es.n_next = 0;
    *es.n_scatter = 0;
    *es.n_boundary = 0;
  }
}

// stage 1: one segment up to the event decision for every active photon
__global__ void __launch_bounds__(kEventThreads) k_event_advance(MeshDev m, CellsDev c, Bank b,
                                                                DeviceDiag *d, unsigned long long seed_hi,
                                                                EventState es, bool first) {
  const unsigned int n = *es.n_active;
  const int sa = d->scale_abs;
  uint32_t flags = 0;
  unsigned long long segs = 0;
  // uniform trip count per warp so the queue ballots see every lane
  const unsigned int stride = gridDim.x * blockDim.x;
  const unsigned int warp_base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
  for (unsigned int w0 = warp_base; w0 < n; w0 += stride) {
    const unsigned int w = w0 + (threadIdx.x & 31u);
    int ev = -1;
    uint32_t p = 0, sc = 0;
    bool flush = false;
    uint32_t fcell = 0;
    double fa = 0.0, ft = 0.0;
    if (w < n) {
      p = es.active[w];
      Lane L;
      load_lane(m, b, es, p, seed_hi, first, L);
      if (L.cell >= m.n_cells) {
        flags |= FLAG_BAD_CELL;
        b.desc[p] = KILLED;
      } else {
        ++segs;
        const CellXS xs = c.xs[L.cell];
        ev = segment_advance(m, b.E0, xs, L, sc, flags);
        if (ev == SEG_KILLED || ev == SEG_CENSUS) {
          flush = true;
          fcell = L.cell;
          fa = L.thr_abs;
          ft = visit_deposit(L, ev);
          store_end(b, L, ev == SEG_KILLED ? KILLED : CENSUS);
        } else {
          b.px[p] = L.px; b.py[p] = L.py; b.pz[p] = L.pz;
          b.E[p] = L.E; b.life[p] = L.life; b.ctr[p] = L.rng.ctr;
          es.thr_abs[p] = L.thr_abs;
          if (ev == SEG_BOUNDARY) es.surface[p] = (uint8_t)sc;
        }
      }
    }
    flush_tally_warp(c.tally, flush, fcell, fcell, fa, ft, flags, sa);
    queue_push(ev == SEG_SCATTER, p, es.q_scatter, es.n_scatter);
    queue_push(ev == SEG_BOUNDARY, p, es.q_boundary, es.n_boundary);
  }
  for (int o = 16; o > 0; o >>= 1) {
    segs += __shfl_down_sync(0xffffffffu, segs, o);
    flags |= __shfl_down_sync(0xffffffffu, flags, o);
  }
  if ((threadIdx.x & 31u) == 0) {
    if (segs) atomicAdd(&d->n_segments, segs);
    if (flags) atomicOr(&d->flags, flags);
  }
}

// stage 2: effective scatter for every photon in the scatter queue
__global__ void __launch_bounds__(kEventThreads) k_event_scatter(MeshDev m, CellsDev c, Bank b,
                                                                unsigned long long seed_hi, EventState es) {
  const unsigned int n = *es.n_scatter;
  const unsigned int stride = gridDim.x * blockDim.x;
  const unsigned int warp_base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
  for (unsigned int w0 = warp_base; w0 < n; w0 += stride) {
    const unsigned int w = w0 + (threadIdx.x & 31u);
    uint32_t p = 0;
    if (w < n) {
      p = es.q_scatter[w];
      Lane L;
      L.cell = b.cell[p];
      L.group = b.group[p];
      L.rng.stream = b.stream[p]; L.rng.ctr = b.ctr[p]; L.rng.hi = seed_hi;
      const CellXS xs = c.xs[L.cell];
      scatter_update(m, c, xs, L);
      b.dx[p] = L.dx; b.dy[p] = L.dy; b.dz[p] = L.dz;
      b.group[p] = L.group; b.ctr[p] = L.rng.ctr;
    }
    queue_push(w < n, p, es.next, es.n_next);
  }
}

// stage 3: boundary crossings (ELEMENT moves on, REFLECT turns, the domain
// boundary ends the history)
__global__ void __launch_bounds__(kEventThreads) k_event_boundary(MeshDev m, CellsDev c, Bank b,
                                                                 DeviceDiag *d, EventState es) {
  const unsigned int n = *es.n_boundary;
  const int sa = d->scale_abs;
  uint32_t flags = 0;
  const unsigned int stride = gridDim.x * blockDim.x;
  const unsigned int warp_base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
  for (unsigned int w0 = warp_base; w0 < n; w0 += stride) {
    const unsigned int w = w0 + (threadIdx.x & 31u);
    uint32_t p = 0;
    bool survive = false;
    bool flush = false;
    uint32_t fcell = 0;
    double fa = 0.0;
    if (w < n) {
      p = es.q_boundary[w];
      Lane L;
      L.cell = b.cell[p];
      cell_coords(m, L.cell, L.ci, L.cj, L.ck);
      const uint32_t sc = es.surface[p];
      const int bc = face_bc(m, L, sc);
      if (bc == ELEMENT || bc == VACUUM || bc == SOURCE || bc == PROCESSOR) {  // the visit ends
        flush = true;
        fcell = L.cell;
        fa = es.thr_abs[p];
      }
      if (bc == ELEMENT) {
        es.thr_abs[p] = 0.0;
        switch (sc) {
          case 0: L.cell -= 1; break;
          case 1: L.cell += 1; break;
          case 2: L.cell -= m.ngx; break;
          case 3: L.cell += m.ngx; break;
          case 4: L.cell -= m.ngx * m.ngy; break;
          default: L.cell += m.ngx * m.ngy; break;
        }
        b.cell[p] = L.cell;
        survive = true;
      } else if (bc == VACUUM || bc == SOURCE || bc == PROCESSOR) {
        b.desc[p] = bc == PROCESSOR ? PASS : EXIT;
      } else {  // REFLECT (photon.h:151-155)
        if (sc < 2) b.dx[p] = -b.dx[p];
        else if (sc < 4) b.dy[p] = -b.dy[p];
        else b.dz[p] = -b.dz[p];
        survive = true;
      }
    }
    flush_tally_warp(c.tally, flush, fcell, fcell, fa, 0.0, flags, sa);
    queue_push(survive, p, es.next, es.n_next);
  }
  for (int o = 16; o > 0; o >>= 1) flags |= __shfl_down_sync(0xffffffffu, flags, o);
  if ((threadIdx.x & 31u) == 0 && flags) atomicOr(&d->flags, flags);
}

// survivors become the next round's active list
__global__ void k_event_rotate(EventState es) {
  // swap by copying the counter; the host swaps the list pointers
  *es.n_active = *es.n_next;
  *es.n_next = 0;
  *es.n_scatter = 0;
  *es.n_boundary = 0;
}

void launch_event_init(const EventState &es, DeviceDiag *d, cudaStream_t s) {
  k_event_init<<<1024, 256, 0, s>>>(es, d);
}

void launch_event_round(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d, uint32_t seed,
                        const EventState &es, bool first, int n_sm, cudaStream_t s) {
  const unsigned long long seed_hi = (unsigned long long)seed << 32;
  const int grid = n_sm * 8;
  k_event_advance<<<grid, kEventThreads, 0, s>>>(m, c, b, d, seed_hi, es, first);
  k_event_scatter<<<grid, kEventThreads, 0, s>>>(m, c, b, seed_hi, es);
  k_event_boundary<<<grid, kEventThreads, 0, s>>>(m, c, b, d, es);
  k_event_rotate<<<1, 1, 0, s>>>(es);
}

}  // namespace bgs
