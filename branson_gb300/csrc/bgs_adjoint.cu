// Adjoint of one transport step: dL/dsigma_a per cell for L = sum_c w_c
// E_abs[c], the absorbed-energy tally weighted by the caller's w.
//
// Estimator.  A history is a sequence of segments k in cells c_k with
// lengths d_k; W_k is its weight before segment k, e_k = exp(-sigma_a f d_k)
// the implicit-capture decay, dE_k = W_k (1 - e_k) the deposit and G =
// sum_k w_{c_k} dE_k (+ w W at a cutoff kill) its contribution to L.  With
// kappa = sigma_a f and sigma_eff = (1 - f) sigma_a + sigma_s, where the
// Fleck factor is f = 1/(1 + K sigma_a), d kappa/d sigma_a = f^2 and
// d sigma_eff/d sigma_a = 1 - f^2.  Per segment k in cell j:
//   pathwise   -f^2 d_k (future_after_k - w_j W_{k+1})   (weight decay)
//   score      (1 - f^2) s_k future_from_k               (collision sampling)
// with s_k = 1/sigma_eff - d_k when the segment ended at the sampled
// collision distance and -d_k otherwise, the derivatives of the log density
// sigma_eff exp(-sigma_eff d) and exp(-sigma_eff d).  An emission photon born
// in cell b adds G f_b/sigma_b (its weight is proportional to f sigma_a with
// the photon counts held fixed).  Boundary-source and census weights do not
// depend on sigma_a, the group choice does not enter L, and the E/E0 < 0.01
// cutoff is a threshold that the estimator does not differentiate.
//
// A launch replays the saved histories of one or many problems (a batched
// backward): work items are all problems' histories, concatenated.
//
// future = G - running prefix: per cell visit the terms add up to
// G * A_v - B_v with A_v, B_v accumulated during the visit, so one replay
// logs (cell, A_v, B_v) per visit in a per-thread slot and flushes G A_v -
// B_v for every visit once the history ends and G is known.  Histories with
// more visits than a slot holds are listed and replayed twice (totals, then
// gradients).  Each history is recomputed from its saved start state and
// Random123 counter with the transport kernel's per-segment code
// (bgs_physics.cuh), so it retraces the forward history exactly.  Gradient
// sums are 128-bit two's-complement fixed point: exact and independent of
// thread order.
#include "bgs_physics.cuh"

namespace bgs {

constexpr int kAdjThreads = 128;
#ifndef BGS_ADJ_MIN_BLOCKS
#define BGS_ADJ_MIN_BLOCKS 6
#endif
constexpr uint8_t kEmission = 2;  // Photon source type of emission photons

__device__ __forceinline__ void flush_grad(const AdjProblem &P, uint32_t cell, double v, uint32_t &flags) {
  if ((__double_as_longlong(v) << 1) == 0) return;
  if (!(fabs(v) <= P.visit_bound)) {
    flags |= (v == v) ? FLAG_TALLY_RANGE : FLAG_NAN;
    return;
  }
  unsigned long long lo, hi;
  to_fixed128_signed(v, P.scale, lo, hi);
  atomic_add128(&P.grad[2 * (size_t)cell], &P.grad[2 * (size_t)cell + 1], lo, hi);
}

// Work items are the saved histories of all problems of the launch
// (item_off: exclusive prefix sum); a lane finds its problem at pickup.
// kPass 0: every history, logged; 1: totals of the listed long histories;
// 2: gradients of the listed long histories with their totals known.
template <int kPass>
__global__ void __launch_bounds__(kAdjThreads, BGS_ADJ_MIN_BLOCKS)
    k_adjoint_replay(const AdjProblem *__restrict__ probs, uint32_t n_probs,
                     const unsigned long long *__restrict__ item_off, AdjShared a) {
  const unsigned long long n = kPass == 0 ? item_off[n_probs] : (unsigned long long)*a.n_long;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lanemask_lt = (1u << lane) - 1u;
  const size_t log_base = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * a.log_len;
  uint32_t flags = 0;
  Lane L;
  bool active = false, done = false, overflow = false;
  unsigned long long item = 0, gitem = 0;
  uint32_t p = 0;
  const CellXS *xs_p = nullptr;
  const AdjCell *ac_p = nullptr;
  double prefix = 0.0, vis_a = 0.0, vis_b = 0.0, G = 0.0;
  uint32_t n_log = 0;

  while (true) {
    const unsigned need = __ballot_sync(0xffffffffu, !active && !done);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) base = atomicAdd(a.work, (unsigned long long)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!active && !done) {
        const unsigned long long w = base + __popc(need & lanemask_lt);
        if (w < n) {
          item = w;
          gitem = kPass == 0 ? w : a.long_list[w];
          if (kPass == 0) {  // items only increase per lane: search forward from the last problem
            uint32_t k = 0;
            while (k < 4 && p + 1 < n_probs && item_off[p + 1] <= gitem) { ++p; ++k; }
            if (k == 4) p = problem_of(item_off, n_probs, gitem, p);
          } else {
            p = problem_of(item_off, n_probs, gitem);
          }
          const AdjProblem &P = probs[p];
          const Bank &t = P.t;
          const unsigned long long i = gitem - item_off[p];
          L.idx = i;
          L.px = t.px[i]; L.py = t.py[i]; L.pz = t.pz[i];
          L.dx = t.dx[i]; L.dy = t.dy[i]; L.dz = t.dz[i];
          L.E = t.E[i]; L.life = t.life[i];
          L.cell = t.cell[i]; L.group = t.group[i];
          L.rng.stream = t.stream[i]; L.rng.ctr = t.ctr[i]; L.rng.hi = P.seed_hi;
          L.segs = 0;
          L.thr_abs = 0.0;
          set_birth(L, t.E0[i]);
          xs_p = P.xs;
          ac_p = P.cell;
          prefix = 0.0; vis_a = 0.0; vis_b = 0.0;
          n_log = 0;
          overflow = false;
          G = kPass == 2 ? a.long_G[w] : 0.0;
          if (L.cell < P.m.n_cells) {
            locate(P.m, L);
            active = true;
            if (t.stype[i] == kEmission) {  // source-weight term, a visit of its own
              const double s = P.src[L.cell];
              if (kPass == 0) {
                a.log_a[log_base] = s;
                a.log_b[log_base] = 0.0;
                a.log_cell[log_base] = L.cell;
                n_log = 1;
              } else if (kPass == 2) {
                flush_grad(P, L.cell, G * s - 0.0, flags);
              }
            }
          } else {
            flags |= FLAG_BAD_CELL;
          }
        } else {
          done = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, !active)) break;
    if (!active) continue;

    // ---- one segment, as in the forward transport
    const CellXS xs = xs_p[L.cell];
    const AdjCell ac = ac_p[L.cell];
    uint32_t surface_cross;
    SegInfo info;
    const int ev = segment_advance(probs[p].m, probs[p].t.E0, xs, L, surface_cross, flags, &info);
    {
      const double s = info.collided ? ac.inv_se - info.d : -info.d;
      const double gs = ac.g2 * s;
      const double pa = ac.f2 * info.d;
      const double prev = prefix;
      // fused where the estimator allows (the oracle's replay uses the same
      // fma): four FP64 operations fewer per segment
      prefix = __fma_rn(ac.w, info.absorbed, prefix);
      const double tail = __fma_rn(ac.w, L.E, prefix);  // prefix after the segment + w_j W_{k+1}
      vis_a = vis_a + (gs - pa);
      vis_b = __fma_rn(gs, prev, __fma_rn(-pa, tail, vis_b));
      if (ev == SEG_KILLED) prefix = tail;     // the cutoff deposits the remaining weight
    }
    bool leave = false, end = false;
    if (ev == SEG_KILLED || ev == SEG_CENSUS) {
      end = true;
    } else if (ev == SEG_SCATTER) {
      CellsDev c{};
      c.group_v = const_cast<double *>(probs[p].group_v);
      scatter_update(probs[p].m, c, xs, L);
    } else {
      const MeshDev &m = probs[p].m;
      const int bc = face_bc(m, L, surface_cross);
      if (bc == ELEMENT) leave = true;
      else if (bc == VACUUM || bc == SOURCE || bc == PROCESSOR) end = true;
      else reflect(m, L, surface_cross);
    }
    if (leave || end) {  // the visit to this cell is over
      if (kPass == 0) {
        if (n_log < a.log_len) {
          a.log_a[log_base + n_log] = vis_a;
          a.log_b[log_base + n_log] = vis_b;
          a.log_cell[log_base + n_log] = L.cell;
          ++n_log;
        } else {
          overflow = true;
        }
      } else if (kPass == 2) {
        flush_grad(probs[p], L.cell, G * vis_a - vis_b, flags);
      }
      vis_a = 0.0;
      vis_b = 0.0;
      if (leave) enter_neighbour(probs[p].m, L, surface_cross);
    }
    if (end) {
      active = false;
      if (kPass == 0) {
        if (overflow) {
          const unsigned int q = atomicAdd(a.n_long, 1u);
          a.long_list[q] = gitem;
        } else {
          G = prefix;
          const AdjProblem &P = probs[p];
          for (uint32_t k = 0; k < n_log; ++k)
            flush_grad(P, a.log_cell[log_base + k], G * a.log_a[log_base + k] - a.log_b[log_base + k], flags);
        }
      } else if (kPass == 1) {
        a.long_G[item] = prefix;
      }
    }
  }

  for (int o = 16; o > 0; o >>= 1) flags |= __shfl_down_sync(0xffffffffu, flags, o);
  if (lane == 0 && flags) atomicOr(a.flags, flags);
}

// per-cell coefficients from the step's opacities and Fleck factors, and the
// largest per-unit-weight coefficient (for the fixed-point range)
__global__ void k_adjoint_cells(CellsDev c, uint32_t n_cells, AdjCell *adj, double *src,
                                unsigned long long *coef_max_bits) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  double cmax = 0.0;
  if (g < n_cells) {
    const double op_a = c.op_a[g], op_s = c.op_s[g], f = c.f[g];
    const double sig_eff = (1.0 - f) * op_a + op_s;
    AdjCell x;
    x.w = 0.0;
    x.f2 = f * f;
    x.g2 = 1.0 - f * f;
    x.inv_se = sig_eff > 0.0 ? 1.0 / sig_eff : 0.0;
    adj[g] = x;
    const double s = op_a > 0.0 ? f / op_a : 0.0;
    src[g] = s;
    cmax = fmax(fabs(s), fabs(x.g2 * x.inv_se));
  }
  for (int o = 16; o > 0; o >>= 1) cmax = fmax(cmax, __shfl_down_sync(0xffffffffu, cmax, o));
  if ((threadIdx.x & 31u) == 0 && cmax > 0.0)
    atomicMax(coef_max_bits, (unsigned long long)__double_as_longlong(cmax));
}

__global__ void k_adjoint_set_w(uint32_t n_cells, AdjCell *adj, const double *w) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n_cells) adj[g].w = w[g];
}

__global__ void k_adjoint_grad_to_double(uint32_t n_cells, const unsigned long long *grad, int scale,
                                         double *out) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n_cells) out[g] = from_fixed128_signed(grad[2 * (size_t)g], grad[2 * (size_t)g + 1], scale);
}

TransportLaunch adjoint_launch_shape(int n_sm) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adjoint_replay<0>, kAdjThreads, 0) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  return {n_sm * per_sm, kAdjThreads};
}

void launch_adjoint_cells(const CellsDev &c, uint32_t n_cells, AdjCell *adj, double *src,
                          unsigned long long *coef_max_bits, cudaStream_t s) {
  cudaMemsetAsync(coef_max_bits, 0, sizeof(unsigned long long), s);
  k_adjoint_cells<<<(n_cells + 255) / 256, 256, 0, s>>>(c, n_cells, adj, src, coef_max_bits);
}

void launch_adjoint_set_w(uint32_t n_cells, AdjCell *adj, const double *w, cudaStream_t s) {
  k_adjoint_set_w<<<(n_cells + 255) / 256, 256, 0, s>>>(n_cells, adj, w);
}

// the three passes; passes 1 and 2 find an empty list in the common case
void launch_adjoint_replay(const AdjProblem *probs, uint32_t n, const unsigned long long *item_off,
                           const AdjShared &a, const TransportLaunch &shape, cudaStream_t s) {
  cudaMemsetAsync(a.work, 0, sizeof(unsigned long long), s);
  k_adjoint_replay<0><<<shape.blocks, shape.threads, 0, s>>>(probs, n, item_off, a);
  cudaMemsetAsync(a.work, 0, sizeof(unsigned long long), s);
  k_adjoint_replay<1><<<shape.blocks, shape.threads, 0, s>>>(probs, n, item_off, a);
  cudaMemsetAsync(a.work, 0, sizeof(unsigned long long), s);
  k_adjoint_replay<2><<<shape.blocks, shape.threads, 0, s>>>(probs, n, item_off, a);
}

void launch_adjoint_grad_to_double(uint32_t n_cells, const unsigned long long *grad, int scale, double *out,
                                   cudaStream_t s) {
  k_adjoint_grad_to_double<<<(n_cells + 255) / 256, 256, 0, s>>>(n_cells, grad, scale, out);
}

}  // namespace bgs
