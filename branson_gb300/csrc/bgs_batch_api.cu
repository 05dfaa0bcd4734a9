// C ABI of batched stepping (include/branson_gb300.h): n existing contexts
// step together.  Every phase of the step is one launch over all problems
// (problem = blockIdx.y of a device table of ProblemView): energies and
// photon counts, sourcing, fixed-point scales, one persistent transport
// launch over every problem's bank, census compaction, tally reduce and
// temperature update -- about thirty launches per step whatever the number
// of problems.  The step's parameters (step number, dt, the current banks)
// are in the table, which a copy at the head of the step refreshes from
// pinned host memory, so the launch sequence is recorded once as a CUDA
// graph and relaunched unchanged every step.
#include <cstring>
#include <new>

#include "bgs_context.cuh"

struct bgs_batch {
  int device = 0;
  int n_sm = 0;
  cudaStream_t stream = nullptr;   // the batch's own stream (joins and the batched launch)
  std::vector<bgs_context *> ctx;
  std::vector<void *> allocs;
  ProblemView *d_views = nullptr;
  ProblemView *h_views = nullptr;   // pinned staging of the view table
  DeviceDiag *d_diags = nullptr;    // every problem's diagnostics after a step, gathered
  DeviceDiag *h_diags = nullptr;    // pinned copy of d_diags, written by the step itself
  BatchGrid grid{};
  unsigned long long *d_item_off = nullptr;
  unsigned long long *d_work = nullptr;  // queue head, launch start and end stamps (ns)
  TransportLaunch shape{};
  cudaEvent_t done = nullptr;
  cudaEvent_t order = nullptr;      // orders the batch after work queued on the contexts' streams
  bool use_graph = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool step_in_flight = false;
  bool gray = false;                // every problem gray (MeshDev::gray): the batched launch's lean build
  float last_transport_ms = 0.0f;
  unsigned long long launches = 0;
  std::string err;
};

namespace {

// launches of one batched step: begin 1, energies and counts 12, sourcing 3,
// scales 2, items + transport 2, census offsets 3, census 2, tallies and
// temperatures 4, diagnostics gather 1
constexpr unsigned long long kLaunchesPerStep = 30;

uint32_t blocks_for(unsigned long long items, uint32_t per_block, uint32_t cap) {
  const unsigned long long b = (items + per_block - 1) / per_block;
  return (uint32_t)(b < 1 ? 1 : (b > cap ? cap : b));
}

int bfail(bgs_batch *b, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define BGS_BCUDA(b, call)                                                                  \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return bfail((b), BGS_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));      \
  } while (0)

void fill_view(const bgs_context *c, const bgs_step_params &p, ProblemView &V) {
  V.m = c->mesh;
  V.c = c->cells;
  V.d = c->d_diag;
  V.from = c->bank[c->cur];
  V.to = c->bank[1 - c->cur];
  V.mat_E = c->d_mat_E;
  V.energy_part = c->d_energy_part;
  V.abs = c->d_abs;
  V.track = c->d_track;
  V.mat_part = c->d_mat_part;
  V.tile_cells = c->d_tile_cells;
  V.off_bank = c->d_off_bank;
  V.tile_bank = c->d_tile_bank;
  V.maxbits = c->d_maxbits;
  V.n_user = c->n_user;
  V.seed_hi = (unsigned long long)c->seed << 32;
  V.capacity = (uint32_t)c->capacity;
  V.step = p.step;
  V.dt = p.dt;
  V.next_dt = p.next_dt;
}

// One whole step for every problem from the view table (capturable: no host waits).
int issue_step(bgs_batch *b) {
  const uint32_t n = (uint32_t)b->ctx.size();
  cudaStream_t s = b->stream;
  BGS_BCUDA(b, cudaMemcpyAsync(b->d_views, b->h_views, n * sizeof(ProblemView), cudaMemcpyHostToDevice, s));
  launch_batch_begin(b->d_views, b->grid, s);
  launch_batch_energy(b->d_views, b->grid, s);
  launch_batch_source(b->d_views, b->grid, s);
  launch_batch_bounds(b->d_views, b->grid, s);
  launch_batch_items(b->d_views, n, b->d_item_off, b->d_work, s);
  launch_transport_batched(b->d_views, n, b->d_item_off, b->d_work, b->shape, b->gray, s);
  launch_batch_census_scan(b->d_views, b->grid, s);
  launch_batch_census(b->d_views, b->grid, s);
  launch_batch_finish(b->d_views, b->grid, s);
  // the diagnostics of all problems reach the host in one copy (n small
  // synchronous copies after the step cost more than the whole census phase)
  launch_batch_diag_gather(b->d_views, n, b->d_diags, s);
  BGS_BCUDA(b, cudaMemcpyAsync(b->h_diags, b->d_diags, n * sizeof(DeviceDiag), cudaMemcpyDeviceToHost, s));
  BGS_BCUDA(b, cudaGetLastError());
  b->launches += kLaunchesPerStep;
  return BGS_OK;
}

// duration of the last batched launch from its in-kernel global-timer stamps
int read_transport_time(bgs_batch *b) {
  unsigned long long t[2];
  BGS_BCUDA(b, cudaMemcpy(t, b->d_work + 1, sizeof(t), cudaMemcpyDeviceToHost));
  b->last_transport_ms = t[1] > t[0] ? (float)((double)(t[1] - t[0]) * 1e-6) : 0.0f;
  return BGS_OK;
}

}  // namespace

const std::vector<bgs_context *> &batch_contexts(const bgs_batch *b) { return b->ctx; }

int batch_fail(bgs_batch *b, int code, const std::string &msg) { return bfail(b, code, "%s", msg.c_str()); }

extern "C" {

int bgs_batch_create(bgs_batch **out, uint32_t n, bgs_context *const *contexts) {
  if (!out || !contexts || n == 0) return BGS_ERR_INVALID;
  *out = nullptr;
  bgs_batch *b = new (std::nothrow) bgs_batch();
  if (!b) return BGS_ERR_INVALID;
  b->ctx.assign(contexts, contexts + n);
  for (uint32_t i = 0; i < n; ++i) {
    bgs_context *c = b->ctx[i];
    if (!c || !c->has_mesh) {
      delete b;
      return BGS_ERR_STATE;
    }
    if (c->device != b->ctx[0]->device) {
      delete b;
      return BGS_ERR_INVALID;
    }
    for (uint32_t j = 0; j < i; ++j)
      if (b->ctx[j] == c) {
        delete b;
        return BGS_ERR_INVALID;
      }
  }
  b->device = b->ctx[0]->device;
  b->n_sm = b->ctx[0]->n_sm;
  int rc = BGS_OK;
  if (cudaSetDevice(b->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->order, cudaEventDisableTiming) != cudaSuccess ||
      cudaMallocHost(&b->h_views, n * sizeof(ProblemView)) != cudaSuccess ||
      cudaMallocHost(&b->h_diags, n * sizeof(DeviceDiag)) != cudaSuccess)
    rc = BGS_ERR_CUDA;
  void *q = nullptr;
  if (!rc && cudaMalloc(&q, n * sizeof(ProblemView)) == cudaSuccess) {
    b->allocs.push_back(q);
    b->d_views = static_cast<ProblemView *>(q);
  } else {
    rc = BGS_ERR_CUDA;
  }
  if (!rc && cudaMalloc(&q, n * sizeof(DeviceDiag)) == cudaSuccess) {
    b->allocs.push_back(q);
    b->d_diags = static_cast<DeviceDiag *>(q);
  } else {
    rc = BGS_ERR_CUDA;
  }
  if (!rc && cudaMalloc(&q, (n + 4) * sizeof(unsigned long long)) == cudaSuccess) {
    b->allocs.push_back(q);
    b->d_item_off = static_cast<unsigned long long *>(q);
    b->d_work = b->d_item_off + n + 1;
  } else {
    rc = BGS_ERR_CUDA;
  }
  if (rc) {
    bgs_batch_destroy(b);
    return rc;
  }
  b->shape = batch_launch_shape(b->n_sm);
  // blocks per problem: enough for the largest problem, but about 32 blocks
  // per SM in total over all problems
  unsigned long long max_cells = 0, max_cap = 0;
  for (bgs_context *c : b->ctx) {
    max_cells = c->mesh.n_cells > max_cells ? c->mesh.n_cells : max_cells;
    max_cap = c->capacity > max_cap ? c->capacity : max_cap;
  }
  const uint32_t per_problem = (uint32_t)(32u * b->n_sm / n) > 8u ? (uint32_t)(32u * b->n_sm / n) : 8u;
  b->grid.n = n;
  b->grid.cells = blocks_for(max_cells, 256, per_problem);
  b->grid.photons = blocks_for(max_cap, 256, 4 * per_problem);
  b->grid.cell_tiles = blocks_for(max_cells, 4096, per_problem);
  b->grid.bank_tiles = blocks_for(max_cap, 4096, per_problem);
  *out = b;
  return BGS_OK;
}

int bgs_batch_destroy(bgs_batch *b) {
  if (!b) return BGS_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (void *p : b->allocs) cudaFree(p);
  if (b->h_views) cudaFreeHost(b->h_views);
  if (b->h_diags) cudaFreeHost(b->h_diags);
  if (b->done) cudaEventDestroy(b->done);
  if (b->order) cudaEventDestroy(b->order);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return BGS_OK;
}

const char *bgs_batch_last_error(const bgs_batch *b) { return b ? b->err.c_str() : "null batch"; }

int bgs_batch_step(bgs_batch *b, const bgs_step_params *params, bgs_transport_diag *out) {
  if (!b || !params) return BGS_ERR_INVALID;
  const uint32_t n = (uint32_t)b->ctx.size();
  for (uint32_t i = 0; i < n; ++i)
    if (params[i].algorithm != BGS_HISTORY || params[i].step < 1 || !(params[i].dt > 0.0))
      return bfail(b, BGS_ERR_INVALID, "problem %u: batched steps are history mode with step >= 1 and dt > 0", i);
  BGS_BCUDA(b, cudaSetDevice(b->device));
  // the pinned view table is rewritten below: the previous step must have read it
  if (b->step_in_flight) BGS_BCUDA(b, cudaEventSynchronize(b->done));
  for (uint32_t i = 0; i < n; ++i) {
    const bgs_context *c = b->ctx[i];
    if (params[i].step == 1 || !c->bank_is_census) {
      // step 1 makes its own census; later steps need the census a step left
      if (params[i].step != 1 && !c->bank_is_census)
        return bfail(b, BGS_ERR_STATE, "problem %u: the bank does not hold a census", i);
    }
    fill_view(c, params[i], b->h_views[i]);
    // after anything already queued on the problem's own stream
    BGS_BCUDA(b, cudaEventRecord(b->order, c->stream));
    BGS_BCUDA(b, cudaStreamWaitEvent(b->stream, b->order, 0));
  }
  bool gray = true;
  for (const bgs_context *c : b->ctx) gray = gray && c->mesh.gray;
  if (gray != b->gray && b->exec) {  // the recorded launch is the other build: record the step again
    cudaGraphExecDestroy(b->exec);
    cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
  }
  b->gray = gray;
  int rc;
  if (b->use_graph) {
    if (!b->exec) {  // record once: every step relaunches the same graph
      BGS_BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      rc = issue_step(b);
      cudaGraph_t g = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (ce != cudaSuccess) return bfail(b, BGS_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(ce));
      b->graph = g;
      BGS_BCUDA(b, cudaGraphInstantiate(&b->exec, g, 0));
    } else {
      b->launches += kLaunchesPerStep;
    }
    BGS_BCUDA(b, cudaGraphLaunch(b->exec, b->stream));
  } else {
    if ((rc = issue_step(b))) return rc;
  }
  for (bgs_context *c : b->ctx) {  // the census is now the current bank
    c->cur = 1 - c->cur;
    c->bank_is_census = true;
    c->xs_dirty = false;
  }
  BGS_BCUDA(b, cudaEventRecord(b->done, b->stream));
  for (bgs_context *c : b->ctx)  // later work on a problem's stream sees the step
    BGS_BCUDA(b, cudaStreamWaitEvent(c->stream, b->done, 0));
  b->step_in_flight = true;
  if (out) {
    BGS_BCUDA(b, cudaEventSynchronize(b->done));
    b->step_in_flight = false;
    for (uint32_t i = 0; i < n; ++i) {
      bgs_context *c = b->ctx[i];
      *c->h_diag = b->h_diags[i];  // copied by the step (issue_step)
      const DeviceDiag &d = *c->h_diag;
      bgs_transport_diag &o = out[i];
      o.n_transported = d.n_bank;
      o.n_census = d.n_census_out;
      o.n_segments = d.n_segments;
      o.census_E = d.census_E;
      o.exit_E = d.exit_E;
      o.absorbed_E = d.absorbed_E;
      o.post_mat_E = d.post_mat_E;
      o.device_flags = d.flags;
      o.reserved = 0;
      if (d.flags) {
        rc = check_flags(c, d.flags);
        return bfail(b, rc, "problem %u: %s", i, c->err.c_str());
      }
    }
    if ((rc = read_transport_time(b))) return rc;
  }
  return BGS_OK;
}

int bgs_batch_synchronize(bgs_batch *b) {
  if (!b) return BGS_ERR_INVALID;
  BGS_BCUDA(b, cudaSetDevice(b->device));
  BGS_BCUDA(b, cudaStreamSynchronize(b->stream));
  b->step_in_flight = false;
  return read_transport_time(b);
}

int bgs_batch_set_option(bgs_batch *b, int option, double value) {
  if (!b) return BGS_ERR_INVALID;
  switch (option) {
    case BGS_BATCH_OPT_GRAPH:
      b->use_graph = value != 0.0;
      return BGS_OK;
    case BGS_BATCH_OPT_TRANSPORT_BLOCKS:
      if (value < 0.0) return bfail(b, BGS_ERR_INVALID, "transport blocks must be >= 0");
      b->shape = value >= 1.0 ? TransportLaunch{(int)value, b->shape.threads} : batch_launch_shape(b->n_sm);
      return BGS_OK;
    default:
      return bfail(b, BGS_ERR_INVALID, "unknown batch option %d", option);
  }
}

int bgs_batch_last_transport_ms(bgs_batch *b, float *ms, uint64_t *kernel_launches) {
  if (!b) return BGS_ERR_INVALID;
  if (ms) *ms = b->last_transport_ms;
  if (kernel_launches) *kernel_launches = b->launches;
  return BGS_OK;
}

}  // extern "C"
