/*
 * branson_gb300 — C ABI of the GB300 (sm_103a) replicated-mode IMC step.
 *
 * One context owns one GPU stream, the replicated structured mesh, the
 * per-cell material state, two photon banks (structure of arrays) and the
 * per-cell tallies.  Every call returns BGS_OK (0) or an error code; the
 * message for the last failure is bgs_last_error(ctx).  Calls on one context
 * must come from one host thread at a time (one context per host thread, no
 * global state).  No call falls back to the CPU: without a usable GPU
 * bgs_create fails.
 *
 * Upstream interfaces each entry point replaces (file:line in Branson's src/):
 *   bgs_set_mesh                 Mesh(...) + Mesh::initialize_physical_properties
 *                                (mesh.h:54-127, :426-439) and GPU_Setup's
 *                                cell upload (gpu_setup.h:23-40)
 *   bgs_calculate_photon_energy  Mesh::calculate_photon_energy (mesh.h:237-323)
 *   bgs_source                   make_initial_census_photons / make_photons +
 *                                join_photon_arrays (source.h:134-366,
 *                                census_functions.h:20-29)
 *   bgs_transport                replicated_transport's history/event branches
 *                                and post_process_photons
 *                                (replicated_transport.h:33-158,
 *                                post_process_functions.h:29-109)
 *   bgs_update_temperature       the tally allreduce + Mesh::update_temperature
 *                                (replicated_driver.h:90-96, mesh.h:327-423)
 *   bgs_step                     one pass of imc_replicated_driver's loop body
 *                                (replicated_driver.h:47-121)
 *   bgs_replicated_transport     replicated_transport<Census_T>(...) itself
 *                                (replicated_transport.h:33-38) with host
 *                                photon buffers: the drop-in the C++ shim in
 *                                branson_gb300_transport.hpp calls
 *   bgs_comb_census              comb_photons (census_functions.h:48-93)
 */
#ifndef BRANSON_GB300_H
#define BRANSON_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define BGS_API __attribute__((visibility("default")))
#else
#define BGS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  BGS_OK = 0,
  BGS_ERR_INVALID = 1,   /* bad argument or size */
  BGS_ERR_CUDA = 2,      /* a CUDA runtime call failed */
  BGS_ERR_CAPACITY = 3,  /* photon bank or census buffer too small */
  BGS_ERR_STATE = 4,     /* call made before what it needs (e.g. no mesh) */
  BGS_ERR_DEVICE = 5,    /* a device-side check fired (see bgs_last_error) */
  BGS_ERR_NO_DEVICE = 6  /* no CUDA device, or not an sm_103 part */
};

/* Constants::bc_type (constants.h:26) */
enum { BGS_REFLECT = 0, BGS_VACUUM = 1, BGS_ELEMENT = 2, BGS_SOURCE = 3, BGS_PROCESSOR = 4 };
/* Constants::event_type (constants.h:28), the photon descriptor */
enum { BGS_EXIT = 0, BGS_PASS = 1, BGS_CENSUS = 2, BGS_SCATTER = 3, BGS_KILLED = 4, BGS_BOUND = 5 };
/* transport algorithms (constants.h:34) */
enum { BGS_HISTORY = 0, BGS_EVENT = 1 };

typedef struct bgs_context bgs_context;

/* Replicated structured mesh as the deck defines it.  Cell
 * g = i + ngx*j + ngx*ngy*k (proto_mesh.h:106-218); its nodes are
 * x_planes[i..i+1], y_planes[j..j+1], z_planes[k..k+1].  Regions are rows of
 * 8 doubles: cV, rho, opacA, opacB, opacC, opacS, initial T_e, initial T_r
 * (region.h:74-83).  bc[] is indexed X-, X+, Y-, Y+, Z-, Z+ (constants.h:27). */
typedef struct {
  uint32_t ngx, ngy, ngz;
  uint32_t n_groups;                 /* BRANSON_N_GROUPS */
  const double *x_planes, *y_planes, *z_planes;
  const uint32_t *cell_region;       /* n_cells region indices (0-based rows) */
  uint32_t n_regions;
  const double *regions;             /* n_regions x 8 */
  int32_t bc[6];
  double T_source;
} bgs_mesh_desc;

/* Photons in host memory as structure of arrays (the Photon fields,
 * photon.h:172-181).  The RNG of a photon is its stream number and the low
 * counter word; the high word is the deck seed << 32 (RNG.h:318-330). */
typedef struct {
  double *pos_x, *pos_y, *pos_z;
  double *dir_x, *dir_y, *dir_z;
  double *E, *E0, *life_dx;
  uint32_t *cell, *group;
  uint8_t *descriptor, *source_type;
  uint64_t *rng_stream, *rng_counter;
} bgs_photons_host;

/* Energies of one bgs_calculate_photon_energy call (mesh.h:282-322). */
typedef struct {
  double total_photon_E, emission_E, census_E, source_E, pre_mat_E;
  uint64_t n_new_photons, n_initial_census;
} bgs_energy_diag;

/* What one step or transport call reports (imc_state.h:254-258 quantities). */
typedef struct {
  uint64_t n_transported;    /* histories in the bank this step */
  uint64_t n_census;         /* census photons left at the end */
  uint64_t n_segments;       /* history-loop trips (transport_photon :55) */
  double census_E, exit_E;   /* post-process sums (post_process_functions.h:46-53) */
  double absorbed_E, post_mat_E;
  uint32_t device_flags;     /* nonzero: a device-side check fired */
  uint32_t reserved;
} bgs_transport_diag;

typedef struct {
  uint32_t step;             /* cycle number, 1-based (imc_state.h:91) */
  uint32_t algorithm;        /* BGS_HISTORY or BGS_EVENT */
  double dt, next_dt;        /* this step's dt and imc_state.get_next_dt() */
} bgs_step_params;

/* per-cell fields readable with bgs_get_cell_field / writable with set */
enum {
  BGS_FIELD_T_E = 0,         /* material temperature (cell.h:334) */
  BGS_FIELD_T_R = 1,         /* radiation temperature from track_E (mesh.h:358) */
  BGS_FIELD_OP_A = 2,        /* absorption opacity (cell.h:330) */
  BGS_FIELD_OP_S = 3,        /* scattering opacity (cell.h:331) */
  BGS_FIELD_F = 4,           /* Fleck factor (cell.h:332) */
  BGS_FIELD_EMISSION_E = 5,  /* mesh.h:272 */
  BGS_FIELD_CENSUS_E = 6,    /* mesh.h:274-277 */
  BGS_FIELD_SOURCE_E = 7,    /* mesh.h:280 */
  BGS_FIELD_ABS_E = 8,       /* last transport's absorbed-energy tally */
  BGS_FIELD_TRACK_E = 9,     /* last transport's track-length tally */
  BGS_FIELD_COUNT = 10
};

/* ------------------------------------------------------------ lifecycle */
/* Create a context on `device` with room for `photon_capacity` photons per
 * bank (below 2^32: BGS_ERR_INVALID otherwise; two banks of 2^32 photons
 * would not fit in the device memory anyway).  `stream` is a cudaStream_t to
 * launch on (NULL: the context creates its own non-blocking stream).  seed
 * and n_user_photons are the deck's <seed> and <photons>
 * (imc_parameters.h:30-40). */
BGS_API int bgs_create(bgs_context **ctx, int device, uint64_t photon_capacity, void *stream,
               uint32_t seed, uint64_t n_user_photons);
BGS_API int bgs_destroy(bgs_context *ctx);
BGS_API const char *bgs_last_error(const bgs_context *ctx);
BGS_API const char *bgs_status_string(int status);
/* Library version string and the device architecture it was built for. */
BGS_API const char *bgs_version(void);

/* ---------------------------------------------------------------- mesh */
/* The replicated Mesh (mesh.h:50-150, built from the deck by its
 * constructor at mesh.h:54) uploaded once; its per-cell state (Cell,
 * cell.h:29-340: T_e, T_r, opacities, Fleck factor, energies) is read and
 * written per field with bgs_get_cell_field / bgs_set_cell_field. */
BGS_API int bgs_set_mesh(bgs_context *ctx, const bgs_mesh_desc *mesh);
BGS_API uint32_t bgs_n_cells(const bgs_context *ctx);
BGS_API int bgs_get_cell_field(bgs_context *ctx, int field, double *host_out);
BGS_API int bgs_set_cell_field(bgs_context *ctx, int field, const double *host_in);

/* ------------------------------------------------------- staged step */
/* Each stage is one phase of imc_replicated_driver's step loop
 * (replicated_driver.h:47-121), on the device. */
/* Mesh::calculate_photon_energy (mesh.h:237-323): per-cell emission,
 * boundary-source and (step 1) initial-census energies, their total, and the
 * per-cell photon counts make_photons draws from them (source.h:207-366). */
BGS_API int bgs_calculate_photon_energy(bgs_context *ctx, uint32_t step, double dt, bgs_energy_diag *out);
/* make_photons (source.h:207-366, called at replicated_driver.h:73): this
 * step's photons on the device after the census already in the bank (step 1
 * also makes the initial census first). */
BGS_API int bgs_source(bgs_context *ctx, uint32_t step, double dt);
/* The transport of replicated_transport (replicated_transport.h:88-92:
 * history_based_transport.h:279-343 in history mode, event_based_transport.h
 * in event mode) and post_process_photons (post_process_functions.h:33-109):
 * every photon in the bank; census photons are compacted (in bank order,
 * life_dx = c*next_dt) into the other bank, which becomes current. */
BGS_API int bgs_transport(bgs_context *ctx, double next_dt, uint32_t algorithm, bgs_transport_diag *out);
/* The tally reduce (replicated_driver.h:90-94) and Mesh::update_temperature
 * (mesh.h:327-423, called at replicated_driver.h:96). */
BGS_API int bgs_update_temperature(bgs_context *ctx, double dt, bgs_transport_diag *out);
/* All four stages, one pass of the step loop (replicated_driver.h:47-121);
 * `out` may be NULL (then nothing is copied back and the call does not wait
 * for the GPU). */
BGS_API int bgs_step(bgs_context *ctx, const bgs_step_params *p, bgs_transport_diag *out);
/* Wait for the context's stream; returns BGS_ERR_DEVICE if a device check
 * fired.  No counterpart in the reference, whose calls return when done. */
BGS_API int bgs_synchronize(bgs_context *ctx);

/* --------------------------------------------------------- photon I/O */
/* The driver's photon list (std::vector<Photon>, photon.h:33-183, or
 * PhotonArray, photon_array.h:25-135), held on the device as the bank. */
/* Number of photons in the current bank (the census after bgs_transport). */
BGS_API int bgs_bank_size(bgs_context *ctx, uint64_t *n);
/* Copy photons [offset, offset+count) of the current bank out / in. */
BGS_API int bgs_get_photons(bgs_context *ctx, uint64_t offset, uint64_t count, const bgs_photons_host *out);
BGS_API int bgs_set_photons(bgs_context *ctx, uint64_t count, const bgs_photons_host *in);

/* Census population control: comb_photons (census_functions.h:48-93) on
 * the census the last transport left in the bank, in bank order, with the
 * caller's RNG(seed, stream) at *rng_counter (RNG.h:318-340): the comb
 * energy is the census's left-to-right energy sum over max_census_photons;
 * census photon k draws number k and survives if the draw exceeds
 * 1 - E/comb_E or it is the last photon left in its cell; survivors take
 * the comb energy plus an equal share of their cell's energy defect.  The
 * survivors (in bank order) become the census the next step starts from.
 * *rng_counter advances by one per census photon; *n_census (may be NULL)
 * receives the survivors.  BGS_ERR_STATE unless the bank holds a census. */
BGS_API int bgs_comb_census(bgs_context *ctx, int64_t max_census_photons, uint32_t seed, uint64_t stream,
                            uint64_t *rng_counter, uint64_t *n_census);

/* ------------------------------------------------ drop-in transport */
/* replicated_transport<Census_T> (replicated_transport.h:33-158) on host
 * buffers: `photons` (n entries) is copied to the device, transported with
 * the context's current cell opacities and Fleck factors, and written back
 * in place (end states); the CENSUS photons are returned in `census` in
 * their input order with life_dx = c*next_dt; rank_abs_E / rank_track_E
 * (n_cells each) are overwritten with this call's tallies.  In history mode,
 * when every photon array is page-locked host memory mapped into the device
 * (cudaMallocHost, cudaHostAlloc, cudaHostRegister with mapping), the kernels
 * transport the photons in place there, reading each state at pickup and
 * writing its end state back over the host link, with no bulk copies
 * (BGS_OPT_ZERO_COPY turns this off); the results are the same bits. */
BGS_API int bgs_replicated_transport(bgs_context *ctx, uint64_t n, const bgs_photons_host *photons,
                             double next_dt, uint32_t algorithm, double *rank_abs_E,
                             double *rank_track_E, const bgs_photons_host *census,
                             uint64_t census_capacity, uint64_t *n_census, double *census_E,
                             double *exit_E);

/* ------------------------------------------- transport without allocation */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory -- host codes that own every device byte through their own pool
 * allocator, or code that must not trigger a cudaMalloc/cudaFree between
 * its launches: the history transport of bgs_replicated_transport on device
 * buffers the caller owns, with all scratch (fixed-point tallies, the
 * per-cell table, counters) in one static device array of the library, so
 * the call allocates nothing.
 *   x/y/z_planes   device, ngx+1 / ngy+1 / ngz+1 node planes
 *   bc             host, 6 domain boundary codes (REFLECT, VACUUM, SOURCE)
 *   op_a, op_s, f  device, one value per cell (cell g = i + ngx*(j + ngy*k))
 *   photons        device structure of arrays, n photons, updated in place
 *                  with their end states; CENSUS photons get life_dx =
 *                  c*next_dt (no compaction: the census stays in place)
 *   abs_E, track_E device outputs, one value per cell (overwritten)
 *   stream         cudaStream_t (NULL: the legacy default stream)
 * Limit: at most 131072 cells (BGS_ERR_CAPACITY beyond); the array (about
 * 11 MB) is held by every GPU that loads the library until exit.  The first
 * call on a device looks up the array's address, so it must come before
 * any stream capture.  All calls share the array: calls that overlap on the
 * GPU race.  Each call is synchronous: it enqueues its work on `stream`,
 * copies the device checks' flags to host memory and waits for the stream,
 * returning BGS_ERR_DEVICE if a check fired. */
BGS_API int bgs_transport_device_noalloc(uint32_t ngx, uint32_t ngy, uint32_t ngz, uint32_t n_groups,
                                         const double *x_planes, const double *y_planes,
                                         const double *z_planes, const int32_t bc[6], const double *op_a,
                                         const double *op_s, const double *f, uint32_t seed, uint64_t n,
                                         const bgs_photons_host *photons, double next_dt, double *abs_E,
                                         double *track_E, void *stream);

/* ------------------------------------------------------------- adjoint */
/* No counterpart in the reference, which computes no derivatives.  An
 * autograd-style pair for L = sum_c w_c E_abs[c], any weighted sum of one
 * step's absorbed-energy tally, differentiated with respect to each cell's
 * absorption opacity sigma_a (the Fleck factor f = 1/(1 + K sigma_a) of
 * mesh.h:267 and the emission energy dt V f sigma_a a c T^4 of mesh.h:272
 * follow sigma_a; photon counts are held at the forward's values).
 *
 * bgs_adjoint_forward: one step's energies (calculate_photon_energy with the
 *   caller's sigma_a per cell in place of the region law when sigma_a is not
 *   NULL), photon counts (the caller's when counts is not NULL: 3*n_cells
 *   values, emission | boundary source | initial census, e.g. from
 *   bgs_adjoint_counts of an earlier forward, so that perturbed runs use
 *   the same photons and random streams), sourcing and history/event
 *   transport; abs_E (host, n_cells) receives the tally.  The context's
 *   bank keeps the step's start states (the transport runs on a copy), its
 *   cell fields hold this step's opacities, Fleck factors and energies, and
 *   its step counter does not move, so repeated forwards at the same step
 *   see the same census.  With tape != NULL the start states and the step's
 *   cell coefficients are saved: *tape == NULL makes a new tape, an existing
 *   tape is reused (its memory grows if needed).
 * bgs_adjoint_backward: grad_abs_E = dL/dE_abs (host, n_cells) in,
 *   grad_sigma_a = dL/dsigma_a (host, n_cells) out.  Replays every saved
 *   history from its start state and random-number counter (nothing per
 *   segment is stored by the forward): pathwise derivatives of the weight
 *   decay exp(-sigma_a f d) and of f, a score-function term for the
 *   sampling of effective-scatter collision distances, and the emission
 *   weight term; sums are exact 128-bit fixed point.  A tape can be
 *   backpropagated any number of times, with any weights, while the
 *   context's mesh is unchanged.
 * bgs_adjoint_counts: the forward's photon counts (3*n_cells values). */
typedef struct bgs_adjoint_tape bgs_adjoint_tape;

typedef struct {
  uint64_t n_histories;      /* photons the forward transported and saved */
  uint64_t n_segments;       /* their history-loop trips */
  uint64_t n_long;           /* last backward: histories replayed twice (long visit lists) */
  double max_E, max_life;    /* largest starting weight and flight length on the tape */
  double coef_max;           /* largest per-cell f/sigma_a or (1-f^2)/sigma_eff */
  double visit_bound;        /* last backward: range of one cell visit's contribution */
  int32_t grad_scale;        /* last backward: fixed-point exponent of the sums */
  uint32_t device_flags;     /* last backward: device checks that fired */
  float replay_ms;           /* last backward: device time of the replay kernels */
  float reserved;
} bgs_adjoint_info;

BGS_API int bgs_adjoint_forward(bgs_context *ctx, const bgs_step_params *p, const double *sigma_a,
                                const uint32_t *counts, double *abs_E, bgs_adjoint_tape **tape);
BGS_API int bgs_adjoint_backward(bgs_context *ctx, bgs_adjoint_tape *tape, const double *grad_abs_E,
                                 double *grad_sigma_a);
BGS_API int bgs_adjoint_counts(const bgs_adjoint_tape *tape, uint32_t *counts);
BGS_API int bgs_adjoint_get_info(const bgs_adjoint_tape *tape, bgs_adjoint_info *info);
BGS_API int bgs_adjoint_release(bgs_adjoint_tape *tape);

/* ------------------------------------------------------------ batching */
/* No counterpart in the reference, which steps one problem per process.
 * n independent problems, each an existing context (own mesh, deck, seed,
 * photon count and bank), step together: per problem the energy,
 * sourcing and transport-preparation phases run on the context's stream,
 * one persistent launch then transports every problem's bank from a global
 * work queue, and census compaction, tally reduce and temperature update
 * follow per problem.  Each problem's results are those of bgs_step on its
 * context alone.  By default the whole step is recorded as one CUDA graph
 * (stream capture over the batch's and the contexts' streams) and launched
 * with one call.  History mode only.  While a batch exists, its contexts
 * must not be stepped or used on their own streams by other threads; the
 * per-problem results are read with the usual per-context calls
 * (bgs_get_cell_field, bgs_get_photons, ...).
 *   params  n entries (step, BGS_HISTORY, dt, next_dt) per problem
 *   out     n entries or NULL (NULL: the call returns without waiting) */
typedef struct bgs_batch bgs_batch;
enum {
  BGS_BATCH_OPT_GRAPH = 0,            /* 1 (default): record each step as a CUDA graph; 0: plain launches */
  BGS_BATCH_OPT_TRANSPORT_BLOCKS = 1  /* persistent-grid blocks of the batched launch (0: occupancy) */
};
BGS_API int bgs_batch_create(bgs_batch **batch, uint32_t n, bgs_context *const *contexts);
BGS_API int bgs_batch_destroy(bgs_batch *batch);
BGS_API const char *bgs_batch_last_error(const bgs_batch *batch);
BGS_API int bgs_batch_step(bgs_batch *batch, const bgs_step_params *params, bgs_transport_diag *out);
BGS_API int bgs_batch_synchronize(bgs_batch *batch);
BGS_API int bgs_batch_set_option(bgs_batch *batch, int option, double value);
/* Adjoint of a batch's current step (see bgs_adjoint_forward / _backward):
 * the forward runs per problem (arrays of n entries: sigma_a[i] and
 * counts[i] may be NULL, or the arrays themselves NULL; tapes[i] as in
 * bgs_adjoint_forward); the backward replays every problem's tape in one
 * persistent launch (work items: all problems' saved histories) and writes
 * grad_sigma_a[i] for each.  The results equal the per-problem calls. */
BGS_API int bgs_batch_adjoint_forward(bgs_batch *batch, const bgs_step_params *params, const double *const *sigma_a,
                                      const uint32_t *const *counts, double *const *abs_E, bgs_adjoint_tape **tapes);
BGS_API int bgs_batch_adjoint_backward(bgs_batch *batch, bgs_adjoint_tape *const *tapes,
                                       const double *const *grad_abs_E, double *const *grad_sigma_a);
/* Device time (ms) of the last batched transport launch, and the kernels
 * the batch has launched (its own and the contexts' phases). */
BGS_API int bgs_batch_last_transport_ms(bgs_batch *batch, float *ms, uint64_t *kernel_launches);

/* ---------------------------------------------------------------- tuning */
/* Execution options (the autotuner in branson_gb300/tune.py sets these; none
 * changes results, only how the work is scheduled).  No upstream counterpart:
 * the reference's knobs are batch_size and n_omp_threads (input.h:249-268). */
enum {
  BGS_OPT_EVENT_ROUND_CAP = 0,      /* event rounds before the tail goes to the history kernel */
  BGS_OPT_EVENT_CHECK_EVERY = 1,    /* rounds between host reads of the active count */
  BGS_OPT_EVENT_TAIL_FRACTION = 2,  /* active share below which event rounds stop */
  BGS_OPT_TRANSPORT_BLOCKS = 3,     /* persistent-grid blocks for the history kernel (0: occupancy);
                                       histories per thread = histories / (blocks * threads) */
  BGS_OPT_TRANSPORT_THREADS = 4,    /* block size of the history kernel: 64, 128 (default) or 256 */
  BGS_OPT_PIPELINE_MIN_PHOTONS = 5, /* bgs_replicated_transport in history mode overlaps its copies
                                       with chunked transport from this many photons (default 2^20;
                                       0 never) */
  BGS_OPT_ZERO_COPY = 6             /* 1 (default): when every photon array given to
                                       bgs_replicated_transport in history mode is page-locked host
                                       memory mapped into the device (cudaMallocHost, cudaHostAlloc,
                                       cudaHostRegister with mapping), the kernels transport the
                                       photons in place there with no bulk copies; 0: always copy */
};
BGS_API int bgs_set_option(bgs_context *ctx, int option, double value);

/* ------------------------------------------------------- instrumentation */
/* Device time (ms) of the last transport kernel span, measured with CUDA
 * events on the context's stream, and its launch count (the reference's
 * transport timer, replicated_transport.h:63-143, times the same span). */
BGS_API int bgs_last_transport_ms(bgs_context *ctx, float *ms, uint32_t *kernel_launches);
/* Kernels launched by this context since creation (its own kernels only).
 * No counterpart in the reference. */
BGS_API uint64_t bgs_kernel_launch_count(const bgs_context *ctx);

#ifdef __cplusplus
}
#endif
#endif
