// C ABI of the GB300 replicated IMC step (include/branson_gb300.h): context
// lifetime, device memory, the staged step and the host-buffer drop-in for
// replicated_transport.  Host-side orchestration only; all arithmetic runs
// in the kernels of bgs_mesh.cu, bgs_source.cu and bgs_transport.cu.
#include <cstring>
#include <new>

#include "bgs_context.cuh"

namespace {

void fill_transport_diag(const DeviceDiag &d, bgs_transport_diag *out) {
  out->n_transported = d.n_bank;
  out->n_census = d.n_census_out;
  out->n_segments = d.n_segments;
  out->census_E = d.census_E;
  out->exit_E = d.exit_E;
  out->absorbed_E = d.absorbed_E;
  out->post_mat_E = d.post_mat_E;
  out->device_flags = d.flags;
  out->reserved = 0;
}

double *field_ptr(bgs_context *ctx, int field) {
  CellsDev &c = ctx->cells;
  switch (field) {
    case BGS_FIELD_T_E: return c.T_e;
    case BGS_FIELD_T_R: return c.T_r_diag;
    case BGS_FIELD_OP_A: return c.op_a;
    case BGS_FIELD_OP_S: return c.op_s;
    case BGS_FIELD_F: return c.f;
    case BGS_FIELD_EMISSION_E: return c.em_E;
    case BGS_FIELD_CENSUS_E: return c.ce_E;
    case BGS_FIELD_SOURCE_E: return c.so_E;
    case BGS_FIELD_ABS_E: return ctx->d_abs;
    case BGS_FIELD_TRACK_E: return ctx->d_track;
    default: return nullptr;
  }
}

int alloc_bank(bgs_context *ctx, Bank &b, unsigned long long cap) {
  int rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.px, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.py, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.pz, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.dx, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.dy, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.dz, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.E, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.E0, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.life, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.cell, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.group, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.desc, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.stype, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.stream, cap))) return rc;
  if ((rc = dev_alloc(ctx, ctx->bank_allocs, &b.ctr, cap))) return rc;
  return BGS_OK;
}

// copy count photons between a bank (at offset) and host SoA arrays
// photon fields of a host/device copy
enum : unsigned {
  F_POS = 1u, F_DIR = 2u, F_E = 4u, F_E0 = 8u, F_LIFE = 16u, F_CELL = 32u, F_GROUP = 64u, F_DESC = 128u,
  F_STYPE = 256u, F_STREAM = 512u, F_CTR = 1024u, F_ALL = 2047u
};

// photons [offset, offset + n) of the bank and of the host arrays (the same
// index in both), the fields in `fields` whose host pointer is set, on s
int copy_photons(bgs_context *ctx, const Bank &b, unsigned long long offset, unsigned long long n,
                 const bgs_photons_host *h, bool to_host, cudaStream_t s, unsigned fields) {
  if (n == 0) return BGS_OK;
  const cudaMemcpyKind kind = to_host ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice;
#define BGS_CP(dev, host, T, F)                                                                           \
  if (h->host && (fields & (F))) {                                                                        \
    if (to_host)                                                                                          \
      BGS_CUDA(ctx, cudaMemcpyAsync(h->host + offset, b.dev + offset, n * sizeof(T), kind, s));           \
    else                                                                                                  \
      BGS_CUDA(ctx, cudaMemcpyAsync(b.dev + offset, h->host + offset, n * sizeof(T), kind, s));           \
  }
  BGS_CP(px, pos_x, double, F_POS)
  BGS_CP(py, pos_y, double, F_POS)
  BGS_CP(pz, pos_z, double, F_POS)
  BGS_CP(dx, dir_x, double, F_DIR)
  BGS_CP(dy, dir_y, double, F_DIR)
  BGS_CP(dz, dir_z, double, F_DIR)
  BGS_CP(E, E, double, F_E)
  BGS_CP(E0, E0, double, F_E0)
  BGS_CP(life, life_dx, double, F_LIFE)
  BGS_CP(cell, cell, uint32_t, F_CELL)
  BGS_CP(group, group, uint32_t, F_GROUP)
  BGS_CP(desc, descriptor, uint8_t, F_DESC)
  BGS_CP(stype, source_type, uint8_t, F_STYPE)
  BGS_CP(stream, rng_stream, uint64_t, F_STREAM)
  BGS_CP(ctr, rng_counter, uint64_t, F_CTR)
#undef BGS_CP
  return BGS_OK;
}

// the whole photon state on the context's stream: host arrays [0, n) at bank [offset, offset + n)
int copy_photons(bgs_context *ctx, const Bank &b, unsigned long long offset, unsigned long long n,
                 const bgs_photons_host *h, bool to_host) {
  if (offset == 0) return copy_photons(ctx, b, 0, n, h, to_host, ctx->stream, F_ALL);
  Bank shifted = b;  // host index 0 is bank index offset
  shifted.px += offset; shifted.py += offset; shifted.pz += offset;
  shifted.dx += offset; shifted.dy += offset; shifted.dz += offset;
  shifted.E += offset; shifted.E0 += offset; shifted.life += offset;
  shifted.cell += offset; shifted.group += offset; shifted.desc += offset; shifted.stype += offset;
  shifted.stream += offset; shifted.ctr += offset;
  return copy_photons(ctx, shifted, 0, n, h, to_host, ctx->stream, F_ALL);
}

__global__ void k_set_bank_size(DeviceDiag *d, unsigned long long n) {
  d->n_bank = n;
  d->n_census_in = n;
  d->census_E_in = 0.0;
  d->n_new = 0;
  d->n_init_census = 0;
}

__global__ void k_reset_queue(DeviceDiag *d) {
  d->work_counter = 0;
  d->n_segments = 0;
}

// the history tail after event rounds restarts the work queue only; the
// segments the event stages counted stay in the step's total
__global__ void k_reset_work(DeviceDiag *d) { d->work_counter = 0; }

}  // namespace

namespace {

// The device address of a host array the GPU can read and write in place:
// page-locked host memory mapped into the device's address space
// (cudaMallocHost, cudaHostAlloc, or cudaHostRegister with mapping), or
// nullptr for any other memory (pageable host memory, device memory).
template <typename T>
T *mapped_alias(T *host) {
  if (!host) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    (void)cudaGetLastError();  // not memory the runtime knows: no alias
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr) return nullptr;
  return static_cast<T *>(a.devicePointer);
}

// every array of the caller's photons as a device-visible bank, or false
bool mapped_bank(const bgs_photons_host *in, Bank &b) {
  b.px = mapped_alias(in->pos_x); b.py = mapped_alias(in->pos_y); b.pz = mapped_alias(in->pos_z);
  b.dx = mapped_alias(in->dir_x); b.dy = mapped_alias(in->dir_y); b.dz = mapped_alias(in->dir_z);
  b.E = mapped_alias(in->E); b.E0 = mapped_alias(in->E0); b.life = mapped_alias(in->life_dx);
  b.cell = mapped_alias(in->cell); b.group = mapped_alias(in->group);
  b.desc = mapped_alias(in->descriptor); b.stype = mapped_alias(in->source_type);
  b.stream = reinterpret_cast<unsigned long long *>(mapped_alias(in->rng_stream));
  b.ctr = reinterpret_cast<unsigned long long *>(mapped_alias(in->rng_counter));
  return b.px && b.py && b.pz && b.dx && b.dy && b.dz && b.E && b.E0 && b.life && b.cell && b.group &&
         b.desc && b.stype && b.stream && b.ctr;
}

// Drop-in transport of photons in mapped host memory, in place: the history
// kernel reads each photon's state at pickup and writes its end state at
// the end straight to the caller's arrays (over the host link: NVLink-C2C
// on GB300), the census pass reads them there and compacts the census into
// the device bank, and no bulk copy runs before or after the kernel.  The
// arithmetic and the work items are those of the device-bank path, so the
// results are the same bits.
int transport_mapped(bgs_context *ctx, uint64_t n, const Bank &hb, double next_dt) {
  const uint64_t before = ctx->launches;
  k_set_bank_size<<<1, 1, 0, ctx->stream>>>(ctx->d_diag, n);
  BGS_LAUNCHED(ctx, 1);
  int rc;
  if ((rc = run_transport(ctx, hb, BGS_HISTORY))) return rc;
  if ((rc = finish_transport_from(ctx, hb, next_dt))) return rc;
  ctx->last_launches = (uint32_t)(ctx->launches - before);
  return BGS_OK;
}

// Drop-in transport of a large host bank as a pipeline: the weights and
// flights go first (the fixed-point scales need the whole bank's maxima),
// the rest of the state follows in chunks on a copy stream, and each chunk
// is transported as soon as it is on the device, alternating two compute
// streams so one chunk's tail overlaps the next chunk; each chunk's end
// states (all but life_dx, which the census pass resets) go back while the
// later chunks run.  Results are those of one launch over the whole bank:
// every photon owns its RNG stream and the tallies are exact fixed-point
// sums.
int pipe_setup(bgs_context *ctx) {
  if (ctx->copy_stream) return BGS_OK;
  BGS_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  BGS_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking));
  for (cudaEvent_t *e : {&ctx->pipe_start, &ctx->pipe_prep, &ctx->pipe_aux, &ctx->pipe_back})
    BGS_CUDA(ctx, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  for (int k = 0; k < bgs_context::kPipeChunks; ++k) {
    BGS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->pipe_in[k], cudaEventDisableTiming));
    BGS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->pipe_done[k], cudaEventDisableTiming));
  }
  return dev_alloc(ctx, ctx->pipe_allocs, &ctx->pipe_queue, (size_t)bgs_context::kPipeChunks);
}

int transport_pipelined(bgs_context *ctx, uint64_t n, const bgs_photons_host *in, double next_dt) {
  int rc;
  if ((rc = pipe_setup(ctx))) return rc;
  Bank &b = ctx->bank[ctx->cur];
  cudaStream_t s = ctx->stream, cs = ctx->copy_stream, as = ctx->aux_stream;
  constexpr int K = bgs_context::kPipeChunks;
  const uint64_t chunk = (n + K - 1) / K;
  const uint64_t before = ctx->launches;
  // nothing may touch the bank before the context's earlier work is done
  BGS_CUDA(ctx, cudaEventRecord(ctx->pipe_start, s));
  BGS_CUDA(ctx, cudaStreamWaitEvent(cs, ctx->pipe_start, 0));
  BGS_CUDA(ctx, cudaStreamWaitEvent(as, ctx->pipe_start, 0));
  // weights and flights, then the scales from their maxima
  if ((rc = copy_photons(ctx, b, 0, n, in, false, s, F_E | F_LIFE))) return rc;
  if (!in->descriptor) BGS_CUDA(ctx, cudaMemsetAsync(b.desc, PASS, n, s));
  if (!in->source_type) BGS_CUDA(ctx, cudaMemsetAsync(b.stype, 0, n, s));
  k_set_bank_size<<<1, 1, 0, s>>>(ctx->d_diag, n);
  BGS_LAUNCHED(ctx, 1);
  if ((rc = prepare_transport(ctx, b))) return rc;
  BGS_CUDA(ctx, cudaMemsetAsync(ctx->pipe_queue, 0, K * sizeof(unsigned long long), s));
  BGS_CUDA(ctx, cudaEventRecord(ctx->pipe_prep, s));
  // the rest of the state, chunk by chunk
  const unsigned rest = F_ALL & ~(F_E | F_LIFE);
  for (int k = 0; k < K; ++k) {
    const uint64_t first = k * chunk, cnt = first < n ? (n - first < chunk ? n - first : chunk) : 0;
    if ((rc = copy_photons(ctx, b, first, cnt, in, false, cs, rest))) return rc;
    BGS_CUDA(ctx, cudaEventRecord(ctx->pipe_in[k], cs));
  }
  // each chunk's transport once its state has arrived
  BGS_CUDA(ctx, cudaStreamWaitEvent(as, ctx->pipe_prep, 0));
  BGS_CUDA(ctx, cudaEventRecord(ctx->ev0, s));
  for (int k = 0; k < K; ++k) {
    const uint64_t first = k * chunk, cnt = first < n ? (n - first < chunk ? n - first : chunk) : 0;
    cudaStream_t st = (k & 1) ? as : s;
    BGS_CUDA(ctx, cudaStreamWaitEvent(st, ctx->pipe_in[k], 0));
    if (cnt) {
      launch_transport_history_range(ctx->mesh, ctx->cells, b, ctx->d_diag, ctx->seed, first, cnt,
                                     ctx->pipe_queue + k, ctx->tshape, st);
      BGS_LAUNCHED(ctx, 1);
    }
    BGS_CUDA(ctx, cudaEventRecord(ctx->pipe_done[k], st));
  }
  BGS_CUDA(ctx, cudaEventRecord(ctx->pipe_aux, as));
  BGS_CUDA(ctx, cudaStreamWaitEvent(s, ctx->pipe_aux, 0));
  BGS_CUDA(ctx, cudaEventRecord(ctx->ev1, s));
  // end states back as chunks finish (life_dx after the census pass)
  bgs_photons_host back = *in;
  back.E0 = nullptr;  // unchanged by transport
  back.rng_stream = nullptr;
  back.source_type = nullptr;
  for (int k = 0; k < K; ++k) {
    const uint64_t first = k * chunk, cnt = first < n ? (n - first < chunk ? n - first : chunk) : 0;
    BGS_CUDA(ctx, cudaStreamWaitEvent(cs, ctx->pipe_done[k], 0));
    if ((rc = copy_photons(ctx, b, first, cnt, &back, true, cs, F_ALL & ~F_LIFE))) return rc;
  }
  BGS_CUDA(ctx, cudaEventRecord(ctx->pipe_back, cs));
  if ((rc = finish_transport(ctx, next_dt))) return rc;
  if ((rc = copy_photons(ctx, b, 0, n, &back, true, s, F_LIFE))) return rc;
  BGS_CUDA(ctx, cudaStreamWaitEvent(s, ctx->pipe_back, 0));
  ctx->bank_is_census = true;
  ctx->last_launches = (uint32_t)(ctx->launches - before);
  return BGS_OK;
}

}  // namespace

// ===================================================================== C ABI
extern "C" {

const char *bgs_version(void) { return "branson_gb300 0.1 (sm_103a)"; }

const char *bgs_status_string(int status) {
  switch (status) {
    case BGS_OK: return "ok";
    case BGS_ERR_INVALID: return "invalid argument";
    case BGS_ERR_CUDA: return "CUDA runtime error";
    case BGS_ERR_CAPACITY: return "capacity exceeded";
    case BGS_ERR_STATE: return "call out of order";
    case BGS_ERR_DEVICE: return "device-side check fired";
    case BGS_ERR_NO_DEVICE: return "no usable sm_103 device";
    default: return "unknown status";
  }
}

const char *bgs_last_error(const bgs_context *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int bgs_create(bgs_context **out, int device, uint64_t photon_capacity, void *stream, uint32_t seed,
               uint64_t n_user_photons) {
  if (!out) return BGS_ERR_INVALID;
  *out = nullptr;
  if (photon_capacity >= (1ULL << 32)) return BGS_ERR_INVALID;  // bank indices are 32-bit on the device
  int n_dev = 0;
  if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev <= device || device < 0)
    return BGS_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return BGS_ERR_NO_DEVICE;
  if (prop.major != 10 || prop.minor != 3) return BGS_ERR_NO_DEVICE;  // built for sm_103a only
  bgs_context *ctx = new (std::nothrow) bgs_context();
  if (!ctx) return BGS_ERR_INVALID;
  ctx->device = device;
  ctx->n_sm = prop.multiProcessorCount;
  ctx->seed = seed;
  ctx->n_user = n_user_photons;
  ctx->capacity = photon_capacity > 0 ? photon_capacity : 1;
  int rc = set_device(ctx);
  if (!rc && stream) {
    ctx->stream = static_cast<cudaStream_t>(stream);
  } else if (!rc) {
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) rc = BGS_ERR_CUDA;
    ctx->own_stream = true;
  }
  if (!rc && (cudaMalloc(&ctx->d_diag, sizeof(DeviceDiag)) != cudaSuccess ||
              cudaMallocHost(&ctx->h_diag, sizeof(DeviceDiag)) != cudaSuccess ||
              cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess))
    rc = BGS_ERR_CUDA;
  if (!rc) rc = alloc_bank(ctx, ctx->bank[0], ctx->capacity);
  if (!rc) rc = alloc_bank(ctx, ctx->bank[1], ctx->capacity);
  if (!rc) {
    const uint32_t tiles = scan_tiles_needed(ctx->capacity) + 1;
    rc = dev_alloc(ctx, ctx->bank_allocs, &ctx->d_off_bank, ctx->capacity + 1);
    if (!rc) rc = dev_alloc(ctx, ctx->bank_allocs, &ctx->d_tile_bank, (size_t)tiles + 1);
    if (!rc) rc = dev_alloc(ctx, ctx->bank_allocs, &ctx->d_maxbits, 2);
  }
  if (!rc && cudaMemsetAsync(ctx->d_diag, 0, sizeof(DeviceDiag), ctx->stream) != cudaSuccess) rc = BGS_ERR_CUDA;
  if (!rc) ctx->tshape = transport_launch_shape(ctx->n_sm);
  if (rc) {
    bgs_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return BGS_OK;
}

int bgs_destroy(bgs_context *ctx) {
  if (!ctx) return BGS_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_list(ctx->mesh_allocs);
  free_list(ctx->bank_allocs);
  free_list(ctx->event_allocs);
  free_list(ctx->adj_allocs);
  free_list(ctx->comb_allocs);
  free_list(ctx->pipe_allocs);
  for (cudaEvent_t e : {ctx->pipe_start, ctx->pipe_prep, ctx->pipe_aux, ctx->pipe_back})
    if (e) cudaEventDestroy(e);
  for (int k = 0; k < bgs_context::kPipeChunks; ++k) {
    if (ctx->pipe_in[k]) cudaEventDestroy(ctx->pipe_in[k]);
    if (ctx->pipe_done[k]) cudaEventDestroy(ctx->pipe_done[k]);
  }
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
  if (ctx->h_counter) cudaFreeHost(ctx->h_counter);
  if (ctx->d_diag) cudaFree(ctx->d_diag);
  if (ctx->h_diag) cudaFreeHost(ctx->h_diag);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return BGS_OK;
}

uint32_t bgs_n_cells(const bgs_context *ctx) { return ctx && ctx->has_mesh ? ctx->mesh.n_cells : 0u; }

uint64_t bgs_kernel_launch_count(const bgs_context *ctx) { return ctx ? ctx->launches : 0ULL; }

int bgs_set_mesh(bgs_context *ctx, const bgs_mesh_desc *md) {
  if (!ctx || !md) return BGS_ERR_INVALID;
  if (!md->x_planes || !md->y_planes || !md->z_planes || !md->cell_region || !md->regions)
    return fail(ctx, BGS_ERR_INVALID, "mesh description has a null array");
  const uint64_t n64 = (uint64_t)md->ngx * md->ngy * md->ngz;
  if (md->ngx == 0 || md->ngy == 0 || md->ngz == 0 || n64 > 0x7fffffffULL)
    return fail(ctx, BGS_ERR_INVALID, "mesh dimensions %u x %u x %u out of range", md->ngx, md->ngy,
                md->ngz);
  if (md->n_regions == 0 || md->n_groups == 0)
    return fail(ctx, BGS_ERR_INVALID, "need at least one region and one group");
  const uint32_t n = (uint32_t)n64;
  for (uint32_t g = 0; g < n; ++g)
    if (md->cell_region[g] >= md->n_regions)
      return fail(ctx, BGS_ERR_INVALID, "cell %u names region %u of %u", g, md->cell_region[g],
                  md->n_regions);
  for (int f = 0; f < 6; ++f)
    if (md->bc[f] != BGS_REFLECT && md->bc[f] != BGS_VACUUM && md->bc[f] != BGS_SOURCE)
      return fail(ctx, BGS_ERR_INVALID, "boundary %d has code %d (REFLECT, VACUUM or SOURCE)", f,
                  md->bc[f]);
  int rc = set_device(ctx);
  if (rc) return rc;
  BGS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  free_list(ctx->mesh_allocs);
  ctx->has_mesh = false;
  double *x, *y, *z, *regions;
  uint32_t *region;
  auto &L = ctx->mesh_allocs;
  if ((rc = dev_alloc(ctx, L, &x, md->ngx + 1)) || (rc = dev_alloc(ctx, L, &y, md->ngy + 1)) ||
      (rc = dev_alloc(ctx, L, &z, md->ngz + 1)) || (rc = dev_alloc(ctx, L, &region, n)) ||
      (rc = dev_alloc(ctx, L, &regions, (size_t)md->n_regions * 8)))
    return rc;
  CellsDev &c = ctx->cells;
  double **dbl[] = {&c.T_e, &c.T_r, &c.T_s, &c.op_a, &c.op_s, &c.f, &c.em_E, &c.ce_E, &c.so_E,
                    &c.T_r_diag, &c.group_v, &c.inv_saf, &ctx->d_mat_E, &ctx->d_abs, &ctx->d_track};
  for (double **p : dbl)
    if ((rc = dev_alloc(ctx, L, p, n))) return rc;
  if ((rc = dev_alloc(ctx, L, &c.xs, n)) || (rc = dev_alloc(ctx, L, &c.tally, n)) ||
      (rc = dev_alloc(ctx, L, &c.source_face, n)) || (rc = dev_alloc(ctx, L, &c.n_em, n)) ||
      (rc = dev_alloc(ctx, L, &c.n_so, n)) || (rc = dev_alloc(ctx, L, &c.n_ce, n)) ||
      (rc = dev_alloc(ctx, L, &c.off_new, (size_t)n + 1)) ||
      (rc = dev_alloc(ctx, L, &c.off_ce, (size_t)n + 1)) ||
      (rc = dev_alloc(ctx, L, &ctx->d_mat_part, update_temperature_parts(n) + 1)) ||
      (rc = dev_alloc(ctx, L, &ctx->d_energy_part, 5 * (size_t)energy_parts(n) + 5)) ||
      (rc = dev_alloc(ctx, L, &ctx->d_tile_cells, (size_t)scan_tiles_needed(n) + 2)))
    return rc;
  BGS_CUDA(ctx, cudaMemcpyAsync(x, md->x_planes, (md->ngx + 1) * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  BGS_CUDA(ctx, cudaMemcpyAsync(y, md->y_planes, (md->ngy + 1) * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  BGS_CUDA(ctx, cudaMemcpyAsync(z, md->z_planes, (md->ngz + 1) * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  BGS_CUDA(ctx, cudaMemcpyAsync(region, md->cell_region, n * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
  BGS_CUDA(ctx, cudaMemcpyAsync(regions, md->regions, (size_t)md->n_regions * 8 * sizeof(double),
                                cudaMemcpyHostToDevice, ctx->stream));
  BGS_CUDA(ctx, cudaMemsetAsync(c.tally, 0, n * sizeof(TallyCell), ctx->stream));
  BGS_CUDA(ctx, cudaMemsetAsync(c.op_a, 0, n * sizeof(double), ctx->stream));
  BGS_CUDA(ctx, cudaMemsetAsync(c.op_s, 0, n * sizeof(double), ctx->stream));
  BGS_CUDA(ctx, cudaMemsetAsync(c.f, 0, n * sizeof(double), ctx->stream));
  MeshDev &m = ctx->mesh;
  m.ngx = md->ngx; m.ngy = md->ngy; m.ngz = md->ngz; m.n_groups = md->n_groups;
  m.n_cells = n; m.n_regions = md->n_regions;
  m.x = x; m.y = y; m.z = z; m.region = region; m.regions = regions;
  for (int f = 0; f < 6; ++f) m.bc[f] = md->bc[f];
  m.T_source = md->T_source;
  m.inv_ngx = div_multiplier(m.ngx);
  m.inv_ngxy = div_multiplier((uint64_t)m.ngx * m.ngy);
  bool no_scatter = true;  // op_s of every cell is its region's opacS (index 5 of the row)
  for (uint32_t r = 0; r < md->n_regions; ++r)
    if (md->regions[8 * (size_t)r + 5] != 0.0) no_scatter = false;
  m.gray = (md->n_groups == 1 && no_scatter) ? 1u : 0u;
  launch_init_cells(m, c, ctx->stream);
  BGS_LAUNCHED(ctx, 1);
  BGS_CUDA(ctx, cudaMemsetAsync(ctx->d_diag, 0, sizeof(DeviceDiag), ctx->stream));
  BGS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->has_mesh = true;
  ++ctx->mesh_generation;
  ctx->xs_dirty = true;
  ctx->bank_is_census = true;
  return BGS_OK;
}

int bgs_get_cell_field(bgs_context *ctx, int field, double *host_out) {
  if (!ctx || !host_out) return BGS_ERR_INVALID;
  if (!ctx->has_mesh) return fail(ctx, BGS_ERR_STATE, "no mesh");
  double *p = field_ptr(ctx, field);
  if (!p) return fail(ctx, BGS_ERR_INVALID, "unknown cell field %d", field);
  int rc = set_device(ctx);
  if (rc) return rc;
  BGS_CUDA(ctx, cudaMemcpyAsync(host_out, p, ctx->mesh.n_cells * sizeof(double), cudaMemcpyDeviceToHost,
                                ctx->stream));
  BGS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BGS_OK;
}

int bgs_set_cell_field(bgs_context *ctx, int field, const double *host_in) {
  if (!ctx || !host_in) return BGS_ERR_INVALID;
  if (!ctx->has_mesh) return fail(ctx, BGS_ERR_STATE, "no mesh");
  if (field != BGS_FIELD_T_E && field != BGS_FIELD_OP_A && field != BGS_FIELD_OP_S && field != BGS_FIELD_F)
    return fail(ctx, BGS_ERR_INVALID, "cell field %d is not writable", field);
  double *p = field_ptr(ctx, field);
  int rc = set_device(ctx);
  if (rc) return rc;
  BGS_CUDA(ctx, cudaMemcpyAsync(p, host_in, ctx->mesh.n_cells * sizeof(double), cudaMemcpyHostToDevice,
                                ctx->stream));
  BGS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (field != BGS_FIELD_T_E) ctx->xs_dirty = true;
  if (field == BGS_FIELD_OP_S)  // physical scattering anywhere: the general transport build until the next mesh
    for (uint32_t g = 0; g < ctx->mesh.n_cells && ctx->mesh.gray; ++g)
      if (host_in[g] != 0.0) ctx->mesh.gray = 0;
  return BGS_OK;
}

int bgs_calculate_photon_energy(bgs_context *ctx, uint32_t step, double dt, bgs_energy_diag *out) {
  if (!ctx) return BGS_ERR_INVALID;
  if (!ctx->has_mesh) return fail(ctx, BGS_ERR_STATE, "no mesh");
  if (step < 1 || !(dt > 0.0)) return fail(ctx, BGS_ERR_INVALID, "step must be >= 1 and dt > 0");
  int rc = set_device(ctx);
  if (rc) return rc;
  const uint32_t n = ctx->mesh.n_cells;
  launch_cell_energy(ctx->mesh, ctx->cells, step, dt, ctx->d_mat_E, ctx->d_energy_part, ctx->d_diag,
                     ctx->n_user, ctx->stream);
  BGS_LAUNCHED(ctx, 6);
  launch_scan_counts(ctx->cells.n_em, ctx->cells.n_so, n, ctx->cells.off_new, ctx->d_tile_cells, ctx->stream);
  BGS_LAUNCHED(ctx, 3);
  launch_scan_counts(ctx->cells.n_ce, nullptr, n, ctx->cells.off_ce, ctx->d_tile_cells, ctx->stream);
  BGS_LAUNCHED(ctx, 3);
  ctx->xs_dirty = false;
  if (out) {
    if ((rc = read_diag(ctx))) return rc;
    unsigned long long offs[2];
    BGS_CUDA(ctx, cudaMemcpy(&offs[0], ctx->cells.off_new + n, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    BGS_CUDA(ctx, cudaMemcpy(&offs[1], ctx->cells.off_ce + n, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    const DeviceDiag &d = *ctx->h_diag;
    out->total_photon_E = d.total_photon_E;
    out->emission_E = d.emission_E;
    out->census_E = d.census_cell_E;
    out->source_E = d.source_E;
    out->pre_mat_E = d.pre_mat_E;
    out->n_new_photons = offs[0];
    out->n_initial_census = step == 1 ? offs[1] : 0;
  }
  return BGS_OK;
}

int bgs_source(bgs_context *ctx, uint32_t step, double dt) {
  if (!ctx) return BGS_ERR_INVALID;
  if (!ctx->has_mesh) return fail(ctx, BGS_ERR_STATE, "no mesh");
  int rc = set_device(ctx);
  if (rc) return rc;
  launch_plan_bank(ctx->mesh, ctx->cells, ctx->d_diag, step, ctx->capacity, ctx->stream);
  BGS_LAUNCHED(ctx, 1);
  launch_source(ctx->mesh, ctx->cells, ctx->bank[ctx->cur], ctx->d_diag, ctx->seed, step, dt, ctx->n_sm,
                ctx->stream);
  BGS_LAUNCHED(ctx, step == 1 ? 2 : 1);
  ctx->bank_is_census = false;
  return BGS_OK;
}

}  // extern "C"

namespace {

int ensure_event_state(bgs_context *ctx) {
  if (ctx->ev_a.active) return BGS_OK;
  const unsigned long long cap = ctx->capacity;
  EventState e{};
  int rc;
  auto &L = ctx->event_allocs;
  if ((rc = dev_alloc(ctx, L, &e.thr_abs, cap)) ||
      (rc = dev_alloc(ctx, L, &e.surface, cap)) || (rc = dev_alloc(ctx, L, &e.active, cap)) ||
      (rc = dev_alloc(ctx, L, &e.next, cap)) || (rc = dev_alloc(ctx, L, &e.q_scatter, cap)) ||
      (rc = dev_alloc(ctx, L, &e.q_boundary, cap)))
    return rc;
  unsigned int *cnt;
  if ((rc = dev_alloc(ctx, L, &cnt, 4))) return rc;
  e.n_active = cnt; e.n_next = cnt + 1; e.n_scatter = cnt + 2; e.n_boundary = cnt + 3;
  if (!ctx->h_counter && cudaMallocHost(&ctx->h_counter, sizeof(unsigned int)) != cudaSuccess)
    return fail(ctx, BGS_ERR_CUDA, "cudaMallocHost failed");
  ctx->ev_a = e;
  ctx->ev_b = e;
  ctx->ev_b.active = e.next;
  ctx->ev_b.next = e.active;
  return BGS_OK;
}

// Event mode: stage rounds while the active set is large, then the history
// kernel finishes the tail from the carried state.
int transport_event(bgs_context *ctx, const Bank &from) {
  int rc;
  if ((rc = ensure_event_state(ctx))) return rc;
  launch_event_init(ctx->ev_a, ctx->d_diag, ctx->stream);
  BGS_LAUNCHED(ctx, 1);
  BGS_CUDA(ctx, cudaMemcpyAsync(ctx->h_counter, ctx->ev_a.n_active, sizeof(unsigned int),
                                cudaMemcpyDeviceToHost, ctx->stream));
  BGS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const double n0 = (double)*ctx->h_counter;
  const double tail = n0 * ctx->event_tail_fraction;
  uint32_t round = 0;
  unsigned int active = *ctx->h_counter;
  while (active > 0 && round < ctx->event_round_cap && (double)active >= tail) {
    const EventState &es = (round & 1) ? ctx->ev_b : ctx->ev_a;
    launch_event_round(ctx->mesh, ctx->cells, from, ctx->d_diag, ctx->seed, es, round == 0, ctx->n_sm,
                       ctx->stream);
    BGS_LAUNCHED(ctx, 4);
    ++round;
    if (round % ctx->event_check_every == 0) {
      BGS_CUDA(ctx, cudaMemcpyAsync(ctx->h_counter, ctx->ev_a.n_active, sizeof(unsigned int),
                                    cudaMemcpyDeviceToHost, ctx->stream));
      BGS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      active = *ctx->h_counter;
    }
  }
  ctx->last_event_rounds = round;
  // the survivors are in the list the last round wrote (its `next`)
  const EventState &tail_es = (round & 1) ? ctx->ev_b : ctx->ev_a;
  if (round == 0) {
    launch_transport_history(ctx->mesh, ctx->cells, from, ctx->d_diag, ctx->seed, ctx->tshape, ctx->stream);
  } else {
    k_reset_work<<<1, 1, 0, ctx->stream>>>(ctx->d_diag);
    BGS_LAUNCHED(ctx, 1);
    launch_transport_resume(ctx->mesh, ctx->cells, from, ctx->d_diag, ctx->seed, tail_es, ctx->tshape,
                            ctx->stream);
  }
  BGS_LAUNCHED(ctx, 1);
  return BGS_OK;
}

}  // namespace

int prepare_transport(bgs_context *ctx, const Bank &from) {
  if (ctx->xs_dirty) {
    launch_cell_xs(ctx->mesh, ctx->cells, ctx->stream);
    BGS_LAUNCHED(ctx, 1);
    ctx->xs_dirty = false;
  }
  launch_bank_bounds(from, ctx->d_maxbits, ctx->d_diag, ctx->n_sm, ctx->stream);
  BGS_LAUNCHED(ctx, 2);
  BGS_CUDA(ctx, cudaMemsetAsync(ctx->cells.tally, 0, ctx->mesh.n_cells * sizeof(TallyCell), ctx->stream));
  k_reset_queue<<<1, 1, 0, ctx->stream>>>(ctx->d_diag);
  BGS_LAUNCHED(ctx, 1);
  return BGS_OK;
}

int run_transport(bgs_context *ctx, const Bank &from, uint32_t algorithm) {
  if (algorithm != BGS_HISTORY && algorithm != BGS_EVENT)
    return fail(ctx, BGS_ERR_INVALID, "unknown transport algorithm %u", algorithm);
  int rc;
  if ((rc = prepare_transport(ctx, from))) return rc;
  BGS_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  if (algorithm == BGS_EVENT) {
    if ((rc = transport_event(ctx, from))) return rc;
  } else {
    launch_transport_history(ctx->mesh, ctx->cells, from, ctx->d_diag, ctx->seed, ctx->tshape, ctx->stream);
    BGS_LAUNCHED(ctx, 1);
  }
  BGS_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  return BGS_OK;
}

// census compaction of the transported bank `from` into the other device
// bank (which becomes current), tallies to doubles
int finish_transport_from(bgs_context *ctx, const Bank &from, double next_dt) {
  Bank &to = ctx->bank[1 - ctx->cur];
  launch_scan_flags(from.desc, CENSUS, (uint32_t)ctx->capacity, &ctx->d_diag->n_bank, ctx->d_off_bank,
                    ctx->d_tile_bank, ctx->stream);
  BGS_LAUNCHED(ctx, 3);
  launch_census(from, to, ctx->d_diag, ctx->d_off_bank, next_dt, ctx->n_sm, ctx->stream);
  BGS_LAUNCHED(ctx, 2);
  launch_tally_to_double(ctx->mesh, ctx->cells, ctx->d_diag, ctx->d_abs, ctx->d_track, ctx->stream);
  BGS_LAUNCHED(ctx, 2);
  ctx->cur = 1 - ctx->cur;
  ctx->bank_is_census = true;
  return BGS_OK;
}

int finish_transport(bgs_context *ctx, double next_dt) {
  return finish_transport_from(ctx, ctx->bank[ctx->cur], next_dt);
}

namespace {

int transport_impl(bgs_context *ctx, double next_dt, uint32_t algorithm) {
  const uint64_t before = ctx->launches;
  int rc;
  if ((rc = run_transport(ctx, ctx->bank[ctx->cur], algorithm))) return rc;
  if ((rc = finish_transport(ctx, next_dt))) return rc;
  ctx->last_launches = (uint32_t)(ctx->launches - before);
  return BGS_OK;
}

}  // namespace

extern "C" {

int bgs_transport(bgs_context *ctx, double next_dt, uint32_t algorithm, bgs_transport_diag *out) {
  if (!ctx) return BGS_ERR_INVALID;
  if (!ctx->has_mesh) return fail(ctx, BGS_ERR_STATE, "no mesh");
  int rc = set_device(ctx);
  if (rc) return rc;
  if ((rc = transport_impl(ctx, next_dt, algorithm))) return rc;
  if (out) {
    if ((rc = read_diag(ctx))) return rc;
    fill_transport_diag(*ctx->h_diag, out);
    return check_flags(ctx, ctx->h_diag->flags);
  }
  return BGS_OK;
}

int bgs_update_temperature(bgs_context *ctx, double dt, bgs_transport_diag *out) {
  if (!ctx) return BGS_ERR_INVALID;
  if (!ctx->has_mesh) return fail(ctx, BGS_ERR_STATE, "no mesh");
  int rc = set_device(ctx);
  if (rc) return rc;
  launch_update_temperature(ctx->mesh, ctx->cells, ctx->d_diag, dt, ctx->d_abs, ctx->d_track,
                            ctx->d_mat_part, ctx->stream);
  BGS_LAUNCHED(ctx, 2);
  if (out) {
    if ((rc = read_diag(ctx))) return rc;
    fill_transport_diag(*ctx->h_diag, out);
    return check_flags(ctx, ctx->h_diag->flags);
  }
  return BGS_OK;
}

int bgs_step(bgs_context *ctx, const bgs_step_params *p, bgs_transport_diag *out) {
  if (!ctx || !p) return BGS_ERR_INVALID;
  int rc;
  if ((rc = bgs_calculate_photon_energy(ctx, p->step, p->dt, nullptr))) return rc;
  if ((rc = bgs_source(ctx, p->step, p->dt))) return rc;
  if ((rc = transport_impl(ctx, p->next_dt, p->algorithm))) return rc;
  if ((rc = bgs_update_temperature(ctx, p->dt, out))) return rc;
  return BGS_OK;
}

int bgs_synchronize(bgs_context *ctx) {
  if (!ctx) return BGS_ERR_INVALID;
  int rc = set_device(ctx);
  if (rc) return rc;
  if ((rc = read_diag(ctx))) return rc;
  return check_flags(ctx, ctx->h_diag->flags);
}

int bgs_bank_size(bgs_context *ctx, uint64_t *n) {
  if (!ctx || !n) return BGS_ERR_INVALID;
  int rc = set_device(ctx);
  if (rc) return rc;
  if ((rc = read_diag(ctx))) return rc;
  *n = ctx->bank_is_census ? ctx->h_diag->n_census_in : ctx->h_diag->n_bank;
  return BGS_OK;
}

int bgs_get_photons(bgs_context *ctx, uint64_t offset, uint64_t count, const bgs_photons_host *out) {
  if (!ctx || !out) return BGS_ERR_INVALID;
  uint64_t n = 0;
  int rc = bgs_bank_size(ctx, &n);
  if (rc) return rc;
  if (offset > n || count > n - offset)
    return fail(ctx, BGS_ERR_INVALID, "photon range [%llu, %llu) outside a bank of %llu",
                (unsigned long long)offset, (unsigned long long)(offset + count), (unsigned long long)n);
  if ((rc = copy_photons(ctx, ctx->bank[ctx->cur], offset, count, out, true))) return rc;
  BGS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BGS_OK;
}

int bgs_set_photons(bgs_context *ctx, uint64_t count, const bgs_photons_host *in) {
  if (!ctx || !in) return BGS_ERR_INVALID;
  if (count > ctx->capacity)
    return fail(ctx, BGS_ERR_CAPACITY, "%llu photons exceed the bank capacity %llu",
                (unsigned long long)count, ctx->capacity);
  if (count > 0 && (!in->pos_x || !in->pos_y || !in->pos_z || !in->dir_x || !in->dir_y || !in->dir_z ||
                    !in->E || !in->E0 || !in->life_dx || !in->cell || !in->group || !in->rng_stream ||
                    !in->rng_counter))
    return fail(ctx, BGS_ERR_INVALID, "input photons need every state array");
  int rc = set_device(ctx);
  if (rc) return rc;
  Bank &b = ctx->bank[ctx->cur];
  if ((rc = copy_photons(ctx, b, 0, count, in, false))) return rc;
  if (!in->descriptor) BGS_CUDA(ctx, cudaMemsetAsync(b.desc, PASS, count, ctx->stream));
  if (!in->source_type) BGS_CUDA(ctx, cudaMemsetAsync(b.stype, 0, count, ctx->stream));
  k_set_bank_size<<<1, 1, 0, ctx->stream>>>(ctx->d_diag, count);
  BGS_LAUNCHED(ctx, 1);
  BGS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->bank_is_census = false;
  return BGS_OK;
}

int bgs_replicated_transport(bgs_context *ctx, uint64_t n, const bgs_photons_host *photons,
                             double next_dt, uint32_t algorithm, double *rank_abs_E,
                             double *rank_track_E, const bgs_photons_host *census,
                             uint64_t census_capacity, uint64_t *n_census, double *census_E,
                             double *exit_E) {
  if (!ctx || !photons) return BGS_ERR_INVALID;
  if (!ctx->has_mesh) return fail(ctx, BGS_ERR_STATE, "no mesh");
  int rc;
  Bank mapped;
  if (algorithm == BGS_HISTORY && ctx->zero_copy && n > 0 && !(rc = set_device(ctx)) &&
      mapped_bank(photons, mapped)) {
    if (n > ctx->capacity)
      return fail(ctx, BGS_ERR_CAPACITY, "%llu photons exceed the bank capacity %llu", (unsigned long long)n,
                  ctx->capacity);
    if ((rc = transport_mapped(ctx, n, mapped, next_dt))) return rc;
  } else if (algorithm == BGS_HISTORY && ctx->pipe_min_photons > 0 && n >= ctx->pipe_min_photons && n > 0) {
    if (n > ctx->capacity)
      return fail(ctx, BGS_ERR_CAPACITY, "%llu photons exceed the bank capacity %llu", (unsigned long long)n,
                  ctx->capacity);
    if (!photons->pos_x || !photons->pos_y || !photons->pos_z || !photons->dir_x || !photons->dir_y ||
        !photons->dir_z || !photons->E || !photons->E0 || !photons->life_dx || !photons->cell ||
        !photons->group || !photons->rng_stream || !photons->rng_counter)
      return fail(ctx, BGS_ERR_INVALID, "input photons need every state array");
    if ((rc = set_device(ctx))) return rc;
    if ((rc = transport_pipelined(ctx, n, photons, next_dt))) return rc;
  } else {
    if ((rc = bgs_set_photons(ctx, n, photons))) return rc;
    if ((rc = transport_impl(ctx, next_dt, algorithm))) return rc;
    // end states come back from the bank that was transported
    const Bank &done = ctx->bank[1 - ctx->cur];
    bgs_photons_host back = *photons;
    back.E0 = nullptr;           // unchanged by transport
    back.rng_stream = nullptr;
    back.source_type = nullptr;
    if ((rc = copy_photons(ctx, done, 0, n, &back, true))) return rc;
  }
  if (rank_abs_E)
    BGS_CUDA(ctx, cudaMemcpyAsync(rank_abs_E, ctx->d_abs, ctx->mesh.n_cells * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
  if (rank_track_E)
    BGS_CUDA(ctx, cudaMemcpyAsync(rank_track_E, ctx->d_track, ctx->mesh.n_cells * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
  if ((rc = read_diag(ctx))) return rc;
  const DeviceDiag &d = *ctx->h_diag;
  if (census_E) *census_E = d.census_E;
  if (exit_E) *exit_E = d.exit_E;
  if (n_census) *n_census = d.n_census_out;
  if ((rc = check_flags(ctx, d.flags))) return rc;
  if (census) {
    if (d.n_census_out > census_capacity)
      return fail(ctx, BGS_ERR_CAPACITY, "census of %llu photons exceeds the buffer of %llu",
                  d.n_census_out, (unsigned long long)census_capacity);
    if ((rc = copy_photons(ctx, ctx->bank[ctx->cur], 0, d.n_census_out, census, true))) return rc;
    BGS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return BGS_OK;
}

int bgs_set_option(bgs_context *ctx, int option, double value) {
  if (!ctx) return BGS_ERR_INVALID;
  switch (option) {
    case BGS_OPT_EVENT_ROUND_CAP:
      if (!(value >= 0 && value <= 1e6)) break;
      ctx->event_round_cap = (uint32_t)value;
      return BGS_OK;
    case BGS_OPT_EVENT_CHECK_EVERY:
      if (!(value >= 1 && value <= 1e6)) break;
      ctx->event_check_every = (uint32_t)value;
      return BGS_OK;
    case BGS_OPT_EVENT_TAIL_FRACTION:
      if (!(value >= 0 && value <= 1)) break;
      ctx->event_tail_fraction = value;
      return BGS_OK;
    case BGS_OPT_TRANSPORT_BLOCKS:
      if (!(value >= 0 && value <= 1e6)) break;
      ctx->transport_blocks = (int)value;
      ctx->tshape = transport_launch_shape(ctx->n_sm, ctx->tshape.threads);
      if (value > 0) ctx->tshape.blocks = (int)value;
      return BGS_OK;
    case BGS_OPT_PIPELINE_MIN_PHOTONS:
      if (!(value >= 0 && value <= 1e15)) break;
      ctx->pipe_min_photons = (unsigned long long)value;
      return BGS_OK;
    case BGS_OPT_ZERO_COPY:
      if (value != 0 && value != 1) break;
      ctx->zero_copy = value != 0;
      return BGS_OK;
    case BGS_OPT_TRANSPORT_THREADS:
      if (value != 64 && value != 128 && value != 256) break;
      ctx->tshape = transport_launch_shape(ctx->n_sm, (int)value);
      if (ctx->transport_blocks > 0) ctx->tshape.blocks = ctx->transport_blocks;
      return BGS_OK;
    default:
      return fail(ctx, BGS_ERR_INVALID, "unknown option %d", option);
  }
  return fail(ctx, BGS_ERR_INVALID, "option %d: value %g out of range", option, value);
}

int bgs_last_transport_ms(bgs_context *ctx, float *ms, uint32_t *kernel_launches) {
  if (!ctx || !ms) return BGS_ERR_INVALID;
  BGS_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
  BGS_CUDA(ctx, cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
  if (kernel_launches) *kernel_launches = ctx->last_launches;
  return BGS_OK;
}

}  // extern "C"
