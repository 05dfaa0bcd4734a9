// C ABI of the adjoint pair (include/branson_gb300.h): a forward that runs
// one step's sourcing and transport from the caller's per-cell sigma_a and
// saves what the backward needs (the photon bank before transport, the
// step's cell coefficients and photon counts), and a backward that replays
// the saved histories (bgs_adjoint.cu) for dL/dsigma_a given dL/dE_abs.
// Host orchestration only.
#include <cmath>
#include <cstring>
#include <new>

#include "bgs_context.cuh"

struct bgs_adjoint_tape {
  int device = 0;
  unsigned long long cap = 0;      // photons the bank arrays hold
  unsigned long long n = 0;        // photons saved by the last forward
  uint32_t n_cells = 0;
  unsigned long long mesh_generation = 0;
  uint32_t seed = 0;
  std::vector<void *> allocs;
  Bank bank{};
  CellXS *xs = nullptr;
  double *group_v = nullptr;
  AdjCell *adj = nullptr;
  double *src = nullptr;
  double *w = nullptr, *grad_out = nullptr;
  unsigned long long *grad = nullptr;
  unsigned long long *scalars = nullptr;  // [0] coefficient max bits
  std::vector<uint32_t> counts;           // emission | boundary source | initial census, per cell
  double max_E = 0.0, max_life = 0.0, coef_max = 0.0;
  unsigned long long n_segments = 0;
  bgs_adjoint_info info{};
  bool valid = false;
};

namespace {

void free_tape_memory(bgs_adjoint_tape *t) {
  free_list(t->allocs);
  t->cap = 0;
  t->n_cells = 0;
  t->valid = false;
}

int alloc_tape(bgs_context *ctx, bgs_adjoint_tape *t, unsigned long long cap, uint32_t n_cells) {
  if (t->cap >= cap && t->n_cells == n_cells && !t->allocs.empty()) return BGS_OK;
  free_tape_memory(t);
  auto &L = t->allocs;
  Bank &b = t->bank;
  int rc;
  if ((rc = dev_alloc(ctx, L, &b.px, cap)) || (rc = dev_alloc(ctx, L, &b.py, cap)) ||
      (rc = dev_alloc(ctx, L, &b.pz, cap)) || (rc = dev_alloc(ctx, L, &b.dx, cap)) ||
      (rc = dev_alloc(ctx, L, &b.dy, cap)) || (rc = dev_alloc(ctx, L, &b.dz, cap)) ||
      (rc = dev_alloc(ctx, L, &b.E, cap)) || (rc = dev_alloc(ctx, L, &b.E0, cap)) ||
      (rc = dev_alloc(ctx, L, &b.life, cap)) || (rc = dev_alloc(ctx, L, &b.cell, cap)) ||
      (rc = dev_alloc(ctx, L, &b.group, cap)) || (rc = dev_alloc(ctx, L, &b.stype, cap)) ||
      (rc = dev_alloc(ctx, L, &b.stream, cap)) || (rc = dev_alloc(ctx, L, &b.ctr, cap)) ||
      (rc = dev_alloc(ctx, L, &t->xs, n_cells)) || (rc = dev_alloc(ctx, L, &t->group_v, n_cells)) ||
      (rc = dev_alloc(ctx, L, &t->adj, n_cells)) || (rc = dev_alloc(ctx, L, &t->src, n_cells)) ||
      (rc = dev_alloc(ctx, L, &t->w, n_cells)) || (rc = dev_alloc(ctx, L, &t->grad_out, n_cells)) ||
      (rc = dev_alloc(ctx, L, &t->grad, 2 * (size_t)n_cells)) || (rc = dev_alloc(ctx, L, &t->scalars, 4))) {
    free_tape_memory(t);
    return rc;
  }
  b.desc = nullptr;  // the replay writes no end states
  t->cap = cap;
  t->n_cells = n_cells;
  return BGS_OK;
}

// one bank's first n photons into another (device to device)
int copy_bank(bgs_context *ctx, const Bank &from, const Bank &to, unsigned long long n, bool with_desc) {
  if (n == 0) return BGS_OK;
#define BGS_CPB(f, T) \
  BGS_CUDA(ctx, cudaMemcpyAsync(to.f, from.f, n * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
  BGS_CPB(px, double) BGS_CPB(py, double) BGS_CPB(pz, double)
  BGS_CPB(dx, double) BGS_CPB(dy, double) BGS_CPB(dz, double)
  BGS_CPB(E, double) BGS_CPB(E0, double) BGS_CPB(life, double)
  BGS_CPB(cell, uint32_t) BGS_CPB(group, uint32_t) BGS_CPB(stype, uint8_t)
  BGS_CPB(stream, unsigned long long) BGS_CPB(ctr, unsigned long long)
  if (with_desc) BGS_CPB(desc, uint8_t)
#undef BGS_CPB
  return BGS_OK;
}

// Replay scratch of a context, grown to `items` saved histories and `n`
// problems: per-thread visit logs, the long-history list, counters, and the
// problem table with its item offsets (device, and pinned host staging).
int ensure_replay_scratch(bgs_context *ctx, unsigned long long items, uint32_t n) {
  auto &L = ctx->adj_allocs;
  int rc;
  if (!ctx->adj_log_a) {
    ctx->adj_shape = adjoint_launch_shape(ctx->n_sm);
    const size_t slots = (size_t)ctx->adj_shape.blocks * ctx->adj_shape.threads * ctx->adj_log_len;
    if ((rc = dev_alloc(ctx, L, &ctx->adj_log_a, slots)) || (rc = dev_alloc(ctx, L, &ctx->adj_log_b, slots)) ||
        (rc = dev_alloc(ctx, L, &ctx->adj_log_cell, slots)) || (rc = dev_alloc(ctx, L, &ctx->adj_work, 4)))
      return rc;
  }
  if (items > ctx->adj_items_cap) {
    const unsigned long long cap = items > 1024 ? items : 1024;
    if ((rc = dev_alloc(ctx, L, &ctx->adj_long_list, cap)) || (rc = dev_alloc(ctx, L, &ctx->adj_long_G, cap)))
      return rc;
    ctx->adj_items_cap = cap;
  }
  if (n > ctx->adj_probs_cap) {
    if ((rc = dev_alloc(ctx, L, &ctx->adj_probs, n)) || (rc = dev_alloc(ctx, L, &ctx->adj_item_off, (size_t)n + 1)))
      return rc;
    ctx->h_adj_probs.resize(n);
    ctx->h_adj_item_off.resize((size_t)n + 1);
    ctx->adj_probs_cap = n;
  }
  return BGS_OK;
}

double bits_to_double(unsigned long long b) {
  double v;
  std::memcpy(&v, &b, sizeof(v));
  return v;
}

// Backward of n saved forwards in one replay launch: tapes[i] was made on
// ctxs[i]; owner supplies the stream, the events and the scratch.
int replay_backward(bgs_context *owner, bgs_context *const *ctxs, bgs_adjoint_tape *const *tapes, uint32_t n,
                    const double *const *w, double *const *out) {
  bgs_context *ctx = owner;
  unsigned long long items = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const bgs_adjoint_tape *t = tapes[i];
    const bgs_context *c = ctxs[i];
    if (!t || !c || !w[i] || !out[i]) return fail(ctx, BGS_ERR_INVALID, "problem %u: null tape, context or array", i);
    if (!t->valid) return fail(ctx, BGS_ERR_STATE, "problem %u: the tape holds no completed forward", i);
    if (t->device != ctx->device || c->device != ctx->device)
      return fail(ctx, BGS_ERR_INVALID, "problem %u: the tape belongs to device %d", i, t->device);
    if (!c->has_mesh || t->mesh_generation != c->mesh_generation || t->n_cells != c->mesh.n_cells)
      return fail(ctx, BGS_ERR_STATE, "problem %u: the mesh changed since the forward", i);
    items += t->n;
  }
  if (items >= 0xffffffffULL * 4096ULL) return fail(ctx, BGS_ERR_CAPACITY, "too many saved histories");
  int rc = set_device(ctx);
  if (rc) return rc;
  if ((rc = ensure_replay_scratch(ctx, items, n))) return rc;
  cudaStream_t s = ctx->stream;
  std::vector<int> scales(n);
  std::vector<double> bounds(n);
  unsigned long long off = 0;
  for (uint32_t i = 0; i < n; ++i) {
    bgs_adjoint_tape *t = tapes[i];
    const bgs_context *c = ctxs[i];
    const uint32_t nc = t->n_cells;
    double wmax = 0.0;
    for (uint32_t g = 0; g < nc; ++g) {
      if (!std::isfinite(w[i][g])) return fail(ctx, BGS_ERR_INVALID, "problem %u: grad_abs_E[%u] is not finite", i, g);
      wmax = std::fmax(wmax, std::fabs(w[i][g]));
    }
    // Range of one visit's contribution G*A - B: |G| <= wmax * E_start, and
    // per unit weight the coefficients sum to at most 3 * flight length plus
    // the per-collision and source coefficients; 2^12 of headroom, and every
    // visit is checked against the bound, so the sum over all visits (at most
    // segments + histories of them) stays inside 2^118.
    const double visit_bound = wmax * t->max_E * (3.0 * t->max_life + 8.0 * t->coef_max) * 4096.0;
    const double n_terms = (double)(t->n_segments + t->n + 1);
    int scale = 0;
    if (visit_bound > 0.0) {
      int e;
      std::frexp(visit_bound * n_terms, &e);
      scale = 118 - e;
    }
    scales[i] = scale;
    bounds[i] = visit_bound;
    BGS_CUDA(ctx, cudaMemcpyAsync(t->w, w[i], nc * sizeof(double), cudaMemcpyHostToDevice, s));
    launch_adjoint_set_w(nc, t->adj, t->w, s);
    BGS_LAUNCHED(ctx, 1);
    BGS_CUDA(ctx, cudaMemsetAsync(t->grad, 0, 2 * (size_t)nc * sizeof(unsigned long long), s));
    AdjProblem P{};
    P.m = c->mesh;
    P.xs = t->xs;
    P.group_v = t->group_v;
    P.t = t->bank;
    P.cell = t->adj;
    P.src = t->src;
    P.grad = t->grad;
    P.seed_hi = (unsigned long long)t->seed << 32;
    P.visit_bound = visit_bound;
    P.scale = scale;
    ctx->h_adj_probs[i] = P;
    ctx->h_adj_item_off[i] = off;
    off += t->n;
  }
  ctx->h_adj_item_off[n] = off;
  // (pageable staging: the copies complete before the calls return)
  BGS_CUDA(ctx, cudaMemcpyAsync(ctx->adj_probs, ctx->h_adj_probs.data(), n * sizeof(AdjProblem),
                                cudaMemcpyHostToDevice, s));
  BGS_CUDA(ctx, cudaMemcpyAsync(ctx->adj_item_off, ctx->h_adj_item_off.data(), ((size_t)n + 1) * sizeof(unsigned long long),
                                cudaMemcpyHostToDevice, s));
  BGS_CUDA(ctx, cudaMemsetAsync(ctx->adj_work + 1, 0, 2 * sizeof(unsigned long long), s));
  AdjShared a{};
  a.log_a = ctx->adj_log_a;
  a.log_b = ctx->adj_log_b;
  a.log_cell = ctx->adj_log_cell;
  a.log_len = ctx->adj_log_len;
  a.long_list = ctx->adj_long_list;
  a.long_G = ctx->adj_long_G;
  a.n_long = reinterpret_cast<unsigned int *>(ctx->adj_work + 1);
  a.work = ctx->adj_work;
  a.flags = reinterpret_cast<uint32_t *>(ctx->adj_work + 2);
  BGS_CUDA(ctx, cudaEventRecord(ctx->ev0, s));
  launch_adjoint_replay(ctx->adj_probs, n, ctx->adj_item_off, a, ctx->adj_shape, s);
  BGS_LAUNCHED(ctx, 3);
  BGS_CUDA(ctx, cudaEventRecord(ctx->ev1, s));
  for (uint32_t i = 0; i < n; ++i) {
    bgs_adjoint_tape *t = tapes[i];
    launch_adjoint_grad_to_double(t->n_cells, t->grad, scales[i], t->grad_out, s);
    BGS_LAUNCHED(ctx, 1);
    BGS_CUDA(ctx, cudaMemcpyAsync(out[i], t->grad_out, t->n_cells * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  unsigned long long sc[2];
  BGS_CUDA(ctx, cudaMemcpyAsync(sc, ctx->adj_work + 1, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  BGS_CUDA(ctx, cudaStreamSynchronize(s));
  float ms = 0.0f;
  BGS_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  for (uint32_t i = 0; i < n; ++i) {
    bgs_adjoint_tape *t = tapes[i];
    t->info.n_long = (uint32_t)sc[0];
    t->info.grad_scale = scales[i];
    t->info.device_flags = (uint32_t)sc[1];
    t->info.visit_bound = bounds[i];
    t->info.replay_ms = ms;
  }
  if (sc[1]) return check_flags(ctx, (uint32_t)sc[1]);
  return BGS_OK;
}

}  // namespace

extern "C" {

int bgs_adjoint_forward(bgs_context *ctx, const bgs_step_params *p, const double *sigma_a,
                        const uint32_t *counts, double *abs_E, bgs_adjoint_tape **tape) {
  if (!ctx || !p || !abs_E) return BGS_ERR_INVALID;
  if (!ctx->has_mesh) return fail(ctx, BGS_ERR_STATE, "no mesh");
  if (p->step < 1 || !(p->dt > 0.0)) return fail(ctx, BGS_ERR_INVALID, "step must be >= 1 and dt > 0");
  if (p->algorithm != BGS_HISTORY && p->algorithm != BGS_EVENT)
    return fail(ctx, BGS_ERR_INVALID, "unknown transport algorithm %u", p->algorithm);
  int rc = set_device(ctx);
  if (rc) return rc;
  const uint32_t nc = ctx->mesh.n_cells;
  cudaStream_t s = ctx->stream;
  // a forward is a function of its inputs: its device checks start clear
  BGS_CUDA(ctx, cudaMemsetAsync(&ctx->d_diag->flags, 0, sizeof(uint32_t), s));
  BGS_CUDA(ctx, cudaMemsetAsync(&ctx->d_diag->bad_counts_cell, 0, sizeof(uint32_t), s));

  // energies from the caller's opacities (or the region law)
  const double *sig_dev = nullptr;
  if (sigma_a) {
    for (uint32_t g = 0; g < nc; ++g)
      if (!(sigma_a[g] >= 0.0) || !std::isfinite(sigma_a[g]))
        return fail(ctx, BGS_ERR_INVALID, "sigma_a[%u] = %g is not a finite value >= 0", g, sigma_a[g]);
    if (ctx->sig_in_cells < nc) {
      if ((rc = dev_alloc(ctx, ctx->adj_allocs, &ctx->d_sig_in, nc))) return rc;
      ctx->sig_in_cells = nc;
    }
    BGS_CUDA(ctx, cudaMemcpyAsync(ctx->d_sig_in, sigma_a, nc * sizeof(double), cudaMemcpyHostToDevice, s));
    sig_dev = ctx->d_sig_in;
  }
  launch_cell_energy(ctx->mesh, ctx->cells, p->step, p->dt, ctx->d_mat_E, ctx->d_energy_part, ctx->d_diag,
                     ctx->n_user, s, sig_dev);
  BGS_LAUNCHED(ctx, 6);
  ctx->xs_dirty = false;
  if (counts) {  // photon counts held fixed (source.h:229-243 evaluated by the caller's earlier run)
    BGS_CUDA(ctx, cudaMemcpyAsync(ctx->cells.n_em, counts, nc * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    BGS_CUDA(ctx, cudaMemcpyAsync(ctx->cells.n_so, counts + nc, nc * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    BGS_CUDA(ctx, cudaMemcpyAsync(ctx->cells.n_ce, counts + 2 * (size_t)nc, nc * sizeof(uint32_t),
                                  cudaMemcpyHostToDevice, s));
    launch_check_counts(ctx->mesh, ctx->cells, ctx->d_diag, p->step, s);
    BGS_LAUNCHED(ctx, 1);
  }
  launch_scan_counts(ctx->cells.n_em, ctx->cells.n_so, nc, ctx->cells.off_new, ctx->d_tile_cells, s);
  BGS_LAUNCHED(ctx, 3);
  launch_scan_counts(ctx->cells.n_ce, nullptr, nc, ctx->cells.off_ce, ctx->d_tile_cells, s);
  BGS_LAUNCHED(ctx, 3);

  // photons into the current bank after its census, as bgs_source
  launch_plan_bank(ctx->mesh, ctx->cells, ctx->d_diag, p->step, ctx->capacity, s);
  BGS_LAUNCHED(ctx, 1);
  Bank &cur = ctx->bank[ctx->cur];
  launch_source(ctx->mesh, ctx->cells, cur, ctx->d_diag, ctx->seed, p->step, p->dt, ctx->n_sm, s);
  BGS_LAUNCHED(ctx, p->step == 1 ? 2 : 1);
  if ((rc = read_diag(ctx))) return rc;
  if ((rc = check_flags(ctx, ctx->h_diag->flags))) return rc;
  const unsigned long long n = ctx->h_diag->n_bank;
  if (tape && n >= 0xffffffffULL)
    return fail(ctx, BGS_ERR_CAPACITY, "a tape holds at most 2^32-1 photons (%llu made)", n);

  bgs_adjoint_tape *t = nullptr;
  if (tape) {
    t = *tape;
    if (!t) {
      t = new (std::nothrow) bgs_adjoint_tape();
      if (!t) return fail(ctx, BGS_ERR_INVALID, "out of host memory");
      t->device = ctx->device;
      *tape = t;
    } else if (t->device != ctx->device) {
      return fail(ctx, BGS_ERR_INVALID, "the tape belongs to device %d", t->device);
    }
    t->valid = false;
    if ((rc = alloc_tape(ctx, t, n > 0 ? n : 1, nc))) return rc;
    if ((rc = copy_bank(ctx, cur, t->bank, n, false))) return rc;
    BGS_CUDA(ctx, cudaMemcpyAsync(t->xs, ctx->cells.xs, nc * sizeof(CellXS), cudaMemcpyDeviceToDevice, s));
    BGS_CUDA(ctx, cudaMemcpyAsync(t->group_v, ctx->cells.group_v, nc * sizeof(double), cudaMemcpyDeviceToDevice, s));
    launch_adjoint_cells(ctx->cells, nc, t->adj, t->src, t->scalars, s);
    BGS_LAUNCHED(ctx, 1);
  }

  // transport a copy so that the context's bank keeps the start states
  Bank &work = ctx->bank[1 - ctx->cur];
  if ((rc = copy_bank(ctx, cur, work, n, true))) return rc;
  if ((rc = run_transport(ctx, work, p->algorithm))) return rc;
  launch_tally_to_double(ctx->mesh, ctx->cells, ctx->d_diag, ctx->d_abs, ctx->d_track, s);
  BGS_LAUNCHED(ctx, 2);
  BGS_CUDA(ctx, cudaMemcpyAsync(abs_E, ctx->d_abs, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  unsigned long long host_bits[3] = {0, 0, 0};
  BGS_CUDA(ctx, cudaMemcpyAsync(host_bits, ctx->d_maxbits, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  if (t) {
    BGS_CUDA(ctx, cudaMemcpyAsync(&host_bits[2], t->scalars, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    t->counts.resize(3 * (size_t)nc);
    BGS_CUDA(ctx, cudaMemcpyAsync(t->counts.data(), ctx->cells.n_em, nc * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    BGS_CUDA(ctx, cudaMemcpyAsync(t->counts.data() + nc, ctx->cells.n_so, nc * sizeof(uint32_t),
                                  cudaMemcpyDeviceToHost, s));
    BGS_CUDA(ctx, cudaMemcpyAsync(t->counts.data() + 2 * (size_t)nc, ctx->cells.n_ce, nc * sizeof(uint32_t),
                                  cudaMemcpyDeviceToHost, s));
  }
  if ((rc = read_diag(ctx))) return rc;  // synchronizes the stream
  if ((rc = check_flags(ctx, ctx->h_diag->flags))) return rc;
  if (t) {
    t->n = n;
    t->seed = ctx->seed;
    t->mesh_generation = ctx->mesh_generation;
    t->max_E = bits_to_double(host_bits[0]);
    t->max_life = bits_to_double(host_bits[1]);
    t->coef_max = bits_to_double(host_bits[2]);
    t->n_segments = ctx->h_diag->n_segments;
    t->info = bgs_adjoint_info{};
    t->info.n_histories = n;
    t->info.n_segments = t->n_segments;
    t->info.max_E = t->max_E;
    t->info.max_life = t->max_life;
    t->info.coef_max = t->coef_max;
    t->valid = true;
  }
  return BGS_OK;
}

int bgs_adjoint_backward(bgs_context *ctx, bgs_adjoint_tape *t, const double *grad_abs_E, double *grad_sigma_a) {
  if (!ctx || !t || !grad_abs_E || !grad_sigma_a) return BGS_ERR_INVALID;
  bgs_context *ctxs[1] = {ctx};
  bgs_adjoint_tape *tapes[1] = {t};
  const double *w[1] = {grad_abs_E};
  double *out[1] = {grad_sigma_a};
  return replay_backward(ctx, ctxs, tapes, 1, w, out);
}

int bgs_batch_adjoint_forward(bgs_batch *b, const bgs_step_params *params, const double *const *sigma_a,
                              const uint32_t *const *counts, double *const *abs_E, bgs_adjoint_tape **tapes) {
  if (!b || !params || !abs_E || !tapes) return BGS_ERR_INVALID;
  int rc = bgs_batch_synchronize(b);
  if (rc) return rc;
  const std::vector<bgs_context *> &ctx = batch_contexts(b);
  for (uint32_t i = 0; i < (uint32_t)ctx.size(); ++i) {
    rc = bgs_adjoint_forward(ctx[i], &params[i], sigma_a ? sigma_a[i] : nullptr, counts ? counts[i] : nullptr,
                             abs_E[i], &tapes[i]);
    if (rc) return batch_fail(b, rc, "problem " + std::to_string(i) + ": " + ctx[i]->err);
  }
  return BGS_OK;
}

int bgs_batch_adjoint_backward(bgs_batch *b, bgs_adjoint_tape *const *tapes, const double *const *grad_abs_E,
                               double *const *grad_sigma_a) {
  if (!b || !tapes || !grad_abs_E || !grad_sigma_a) return BGS_ERR_INVALID;
  int rc = bgs_batch_synchronize(b);
  if (rc) return rc;
  const std::vector<bgs_context *> &ctx = batch_contexts(b);
  rc = replay_backward(ctx[0], ctx.data(), tapes, (uint32_t)ctx.size(), grad_abs_E, grad_sigma_a);
  if (rc) return batch_fail(b, rc, ctx[0]->err);
  return BGS_OK;
}

int bgs_adjoint_counts(const bgs_adjoint_tape *t, uint32_t *counts) {
  if (!t || !counts) return BGS_ERR_INVALID;
  if (!t->valid) return BGS_ERR_STATE;
  std::memcpy(counts, t->counts.data(), t->counts.size() * sizeof(uint32_t));
  return BGS_OK;
}

int bgs_adjoint_get_info(const bgs_adjoint_tape *t, bgs_adjoint_info *info) {
  if (!t || !info) return BGS_ERR_INVALID;
  if (!t->valid) return BGS_ERR_STATE;
  *info = t->info;
  return BGS_OK;
}

int bgs_adjoint_release(bgs_adjoint_tape *t) {
  if (!t) return BGS_OK;
  cudaSetDevice(t->device);
  cudaDeviceSynchronize();
  free_tape_memory(t);
  delete t;
  return BGS_OK;
}

}  // extern "C"
