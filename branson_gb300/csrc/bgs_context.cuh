// Host-side state of one device context and the helpers the C-ABI
// translation units share (bgs_api.cu, bgs_adjoint_api.cu).  Private to the
// library: nothing here is part of the public header.
#pragma once

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/branson_gb300.h"
#include "bgs_kernels.cuh"

using namespace bgs;

struct bgs_context {
  int device = 0;
  int n_sm = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  uint32_t seed = 0;
  unsigned long long n_user = 0;
  unsigned long long capacity = 0;
  bool has_mesh = false;
  bool xs_dirty = true;

  MeshDev mesh{};
  CellsDev cells{};
  std::vector<void *> mesh_allocs;  // freed on set_mesh / destroy
  double *d_mat_E = nullptr, *d_abs = nullptr, *d_track = nullptr, *d_mat_part = nullptr;
  double *d_energy_part = nullptr;
  unsigned long long *d_tile_cells = nullptr;

  Bank bank[2]{};
  int cur = 0;
  std::vector<void *> bank_allocs;
  unsigned long long *d_off_bank = nullptr, *d_tile_bank = nullptr, *d_maxbits = nullptr;

  // event mode (allocated on first use): carried tallies, surfaces, lists, counters
  std::vector<void *> event_allocs;
  EventState ev_a{}, ev_b{};     // ev_b has active/next swapped
  unsigned int *h_counter = nullptr;  // pinned
  uint32_t event_round_cap = 64;      // rounds before the tail goes to the history kernel
  uint32_t event_check_every = 4;     // rounds between host reads of the active count
  double event_tail_fraction = 0.02;  // active share below which the tail goes to history mode
  unsigned long long last_event_rounds = 0;

  // adjoint (allocated on first use): the caller's opacities, replay logs
  std::vector<void *> adj_allocs;
  double *d_sig_in = nullptr;
  uint32_t sig_in_cells = 0;
  TransportLaunch adj_shape{};
  uint32_t adj_log_len = 256;          // cell visits one replay thread logs
  double *adj_log_a = nullptr, *adj_log_b = nullptr;
  uint32_t *adj_log_cell = nullptr;
  unsigned long long *adj_work = nullptr;          // [0] queue head, [1] long-history count, [2] flags
  unsigned long long *adj_long_list = nullptr;     // long histories (work items)
  double *adj_long_G = nullptr;
  unsigned long long adj_items_cap = 0;
  AdjProblem *adj_probs = nullptr;                 // replay problem table and item offsets
  unsigned long long *adj_item_off = nullptr;
  uint32_t adj_probs_cap = 0;
  std::vector<AdjProblem> h_adj_probs;
  std::vector<unsigned long long> h_adj_item_off;
  unsigned long long mesh_generation = 0;  // bumped by every bgs_set_mesh

  // pipelined drop-in transport (created on first use): a copy stream, a
  // second compute stream, per-chunk events and work counters
  static constexpr int kPipeChunks = 8;
  unsigned long long pipe_min_photons = 1ULL << 20;  // 0: never pipelined
  bool zero_copy = true;  // history-mode drop-in on mapped host arrays: transported in place
  cudaStream_t copy_stream = nullptr, aux_stream = nullptr;
  cudaEvent_t pipe_start = nullptr, pipe_prep = nullptr, pipe_aux = nullptr, pipe_back = nullptr;
  cudaEvent_t pipe_in[kPipeChunks] = {}, pipe_done[kPipeChunks] = {};
  unsigned long long *pipe_queue = nullptr;
  std::vector<void *> pipe_allocs;

  // census comb (allocated on first use): radix-sort buffers, cell ranges
  std::vector<void *> comb_allocs;
  uint32_t *comb_keys = nullptr, *comb_pos = nullptr;  // 2n each: sort input, output
  uint32_t *comb_first = nullptr;                      // 2 n_cells: first, last sorted slot
  double *comb_scalars = nullptr;                      // list energy, comb energy
  uint8_t *comb_temp = nullptr;
  uint32_t comb_cap = 0, comb_cells_cap = 0;
  size_t comb_temp_bytes = 0;

  DeviceDiag *d_diag = nullptr;
  DeviceDiag *h_diag = nullptr;  // pinned
  TransportLaunch tshape{};
  int transport_blocks = 0;           // grid override of the history kernel (0: occupancy)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  uint32_t last_launches = 0;
  unsigned long long launches = 0;
  bool bank_is_census = true;  // current bank holds a census (after transport)
  std::string err;
};



inline int fail(bgs_context *ctx, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  return code;
}

#define BGS_CUDA(ctx, call)                                                                   \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fail((ctx), BGS_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));       \
  } while (0)

#define BGS_LAUNCHED(ctx, n)                                                                  \
  do {                                                                                        \
    cudaError_t e_ = cudaGetLastError();                                                      \
    if (e_ != cudaSuccess)                                                                    \
      return fail((ctx), BGS_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e_));   \
    (ctx)->launches += (n);                                                                   \
  } while (0)

template <typename T>
inline int dev_alloc(bgs_context *ctx, std::vector<void *> &list, T **p, size_t count) {
  void *q = nullptr;
  const size_t bytes = count * sizeof(T) > 0 ? count * sizeof(T) : 16;
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess)
    return fail(ctx, BGS_ERR_CUDA, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
  list.push_back(q);
  *p = static_cast<T *>(q);
  return BGS_OK;
}

inline void free_list(std::vector<void *> &list) {
  for (void *p : list) cudaFree(p);
  list.clear();
}

inline int set_device(bgs_context *ctx) {
  BGS_CUDA(ctx, cudaSetDevice(ctx->device));
  return BGS_OK;
}

inline int check_flags(bgs_context *ctx, uint32_t flags) {
  if (!flags) return BGS_OK;
  std::string what;
  if (flags & FLAG_CAPACITY) what += " photon-bank capacity exceeded (no photons made);";
  if (flags & FLAG_TALLY_RANGE) what += " tally contribution outside the fixed-point range;";
  if (flags & FLAG_SEGMENT_LIMIT) what += " a history hit the segment limit;";
  if (flags & FLAG_BAD_CELL) what += " a photon referenced a cell outside the mesh;";
  if (flags & FLAG_NAN) what += " a non-finite tally contribution was dropped;";
  if (flags & FLAG_BAD_COUNTS) {
    what += " supplied photon counts disagree with the cell energies";
    if (ctx->h_diag && ctx->h_diag->bad_counts_cell)
      what += " (cell " + std::to_string(ctx->h_diag->bad_counts_cell - 1) + ")";
    what += ";";
  }
  return fail(ctx, (flags & FLAG_CAPACITY) ? BGS_ERR_CAPACITY : BGS_ERR_DEVICE,
              "device check fired (flags 0x%x):%s", flags, what.c_str());
}

inline int read_diag(bgs_context *ctx) {
  BGS_CUDA(ctx, cudaMemcpyAsync(ctx->h_diag, ctx->d_diag, sizeof(DeviceDiag), cudaMemcpyDeviceToHost,
                                ctx->stream));
  BGS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BGS_OK;
}

// Transport phases (bgs_api.cu).  prepare_transport: per-cell table if
// stale, fixed-point scales from the bank, zeroed tallies and work queue.
// run_transport: prepare + every photon in `from` transported (history or
// event mode) into the context's tallies.  finish_transport: census
// compaction into the other bank (which becomes current) and the tallies
// converted to doubles; finish_transport_from does the same for another
// transported bank (the caller's mapped host arrays).
int prepare_transport(bgs_context *ctx, const Bank &from);

// a batch's contexts in problem order, and its error message (bgs_batch_api.cu)
struct bgs_batch;
const std::vector<bgs_context *> &batch_contexts(const bgs_batch *b);
int batch_fail(bgs_batch *b, int code, const std::string &msg);
int run_transport(bgs_context *ctx, const Bank &from, uint32_t algorithm);
int finish_transport(bgs_context *ctx, double next_dt);
int finish_transport_from(bgs_context *ctx, const Bank &from, double next_dt);
