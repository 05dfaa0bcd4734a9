/*
 * branson_oracle — CPU restatement of Branson's replicated-mode IMC step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the GPU path is
 * compared against (tests/, __graft_entry__.smoke(), and the CPU-baseline
 * leg of bench.py).  The product library never links, loads or calls it.
 *
 * Every function restates the upstream algorithm in plain C, in the same
 * floating-point operation order, and cites the upstream file:line it
 * follows.  It is pinned against outputs of the upstream headers compiled
 * unmodified (oracle/ref_harness.cc) through the committed golden vectors in
 * tests/golden/.
 */
#ifndef BRANSON_ORACLE_H
#define BRANSON_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* boundary condition codes, Constants::bc_type (constants.h:26) */
enum { BO_REFLECT = 0, BO_VACUUM = 1, BO_ELEMENT = 2, BO_SOURCE = 3, BO_PROCESSOR = 4 };
/* photon descriptors, Constants::event_type (constants.h:28) */
enum { BO_EXIT = 0, BO_PASS = 1, BO_CENSUS = 2, BO_SCATTER = 3, BO_KILLED = 4, BO_BOUND = 5 };

/* Photon record: the layout oracle/ref_harness.cc dumps (104 bytes).
 * stream/counter are RNG words data[2]/data[0] (RNG.h:318-330). */
typedef struct {
  uint64_t stream, counter;
  uint32_t cell, group, source_type, descriptor;
  double pos[3], dir[3], E, E0, life_dx;
} bo_photon;

/* Region physical data (region.h:74-83 plus the deck's region block). */
typedef struct {
  double cv, rho, opacA, opacB, opacC, opacS, T_e, T_r;
} bo_region;

/* Structured replicated mesh.  Cell g = i + ngx*j + ngx*ngy*k
 * (proto_mesh.h:106-218); nodes come from the plane arrays x[ngx+1] etc. */
typedef struct {
  uint32_t ngx, ngy, ngz, n_groups;
  const double *x, *y, *z;        /* planes */
  const uint32_t *region;         /* region index per cell */
  const bo_region *regions;
  int bc[6];                      /* X-, X+, Y-, Y+, Z-, Z+ domain faces */
  double T_source;
} bo_mesh;

/* Per-cell mutable state and per-step derived data. */
typedef struct {
  double *T_e, *T_r, *T_s;        /* temperatures (T_s nonzero on source cells) */
  double *op_a, *op_s, *f;        /* set by bo_calculate_photon_energy */
  double *emission_E, *census_E, *source_E;
  double *T_r_diag;               /* radiation temperature from track_E (mesh.h:358) */
} bo_cells;

typedef struct {
  double total_photon_E, emission_E, census_E, source_E, pre_mat_E;
} bo_energy;

/* Threefry2x64-20 block function (Salmon et al., SC'11; threefry.h:190-293). */
void bo_threefry2x64_20(const uint64_t ctr[2], const uint64_t key[2], uint64_t out[2]);
/* One draw of RNG::generate_random_number (RNG.h:262-285,333-334): advances
 * *counter and returns u01fixedpt of the first output word. */
double bo_rng_draw(uint32_t seed, uint64_t stream, uint64_t *counter);

/* Node array (x_lo, x_hi, y_lo, y_hi, z_lo, z_hi) of cell g (cell.h:325). */
void bo_cell_nodes(const bo_mesh *m, uint32_t g, double nodes[6]);
/* Cell::get_distance_to_boundary (cell.h:117-132). */
double bo_distance_to_boundary(const double nodes[6], const double pos[3], const double dir[3],
                               uint32_t *surface_cross);

/* Mesh::initialize_physical_properties (mesh.h:426-439). */
void bo_initialize_cells(const bo_mesh *m, bo_cells *c);
/* Mesh::calculate_photon_energy for one rank (mesh.h:237-323). */
void bo_calculate_photon_energy(const bo_mesh *m, bo_cells *c, uint32_t step, double dt,
                                bo_energy *out);
/* Photon counts; returns the number make_photons / make_initial_census_photons
 * create (source.h:139-156, 225-245). */
uint64_t bo_count_photons(const bo_mesh *m, const bo_cells *c, uint64_t n_user, double total_E);
uint64_t bo_count_initial_census(const bo_mesh *m, const bo_cells *c, uint64_t n_user,
                                 double total_E);
/* make_photons (source.h:294-366) / make_initial_census_photons (source.h:183-204). */
void bo_make_photons(const bo_mesh *m, const bo_cells *c, double dt, uint32_t cycle, uint32_t seed,
                     uint64_t n_user, double total_E, bo_photon *out);
void bo_make_initial_census(const bo_mesh *m, const bo_cells *c, double dt, uint32_t seed,
                            uint64_t n_user, double total_E, bo_photon *out);

/* history_cpu_transport_photons (history_based_transport.h:279-308) over
 * transport_photon (:33-141).  Tallies are overwritten.  n_threads<=0 uses
 * the OpenMP default.  Returns the number of segments (loop trips). */
uint64_t bo_transport(const bo_mesh *m, const bo_cells *c, uint32_t seed, bo_photon *photons,
                      size_t n, double *abs_E, double *track_E, int n_threads);

/* One segment of a traced history: the three event distances the loop
 * compares (history_based_transport.h:56-67), the three face quotients
 * get_distance_to_boundary takes the smallest of (cell.h:117-132), the
 * weight after the segment (for the cutoff test E/E0 < 0.01,
 * photon.h:47-49), the cell the segment ran in, the descriptor it ended
 * with, the face picked, and the low word of the RNG counter after it. */
typedef struct {
  double d_scatter, d_boundary, d_census, face_q[3], E, E0;
  uint32_t cell, descriptor, surface, counter;
} bo_trace_rec;

/* transport_photon on one photon with a per-segment trace: up to
 * max_segments records go to out; returns the number of segments; the end
 * state goes to *end (may be NULL). */
size_t bo_trace_photon(const bo_mesh *m, const bo_cells *c, uint32_t seed, const bo_photon *start,
                       bo_trace_rec *out, size_t max_segments, bo_photon *end);

/* post_process_photons (post_process_functions.h:33-59): census photons are
 * copied in order into census_out (may be NULL to count only).  Returns the
 * census size. */
size_t bo_post_process(double next_dt, bo_photon *photons, size_t n, bo_photon *census_out,
                       double *census_E, double *exit_E);

/* comb_photons (census_functions.h:48-93), census population control: the
 * comb energy is the list's left-to-right energy sum over max_census; photon
 * k of the list takes draw k of RNG(seed, stream) from *counter (one draw per
 * photon) and survives when the draw exceeds 1 - E/comb_E or it is the only
 * photon left in its cell; survivors take the comb energy, and then every
 * survivor of a cell gets an equal share of the cell's energy defect.  The
 * per-cell maps are arrays over n_cells with sums in list order, as upstream.
 * Survivors are written in list order to out (which may alias photons);
 * returns their number and advances *counter past the draws. */
size_t bo_comb_census(const bo_photon *photons, size_t n, uint32_t n_cells, int64_t max_census, uint32_t seed,
                      uint64_t stream, uint64_t *counter, bo_photon *out);

/* Mesh::update_temperature (mesh.h:327-362); abs/track are zeroed. */
void bo_update_temperature(const bo_mesh *m, bo_cells *c, double dt, double *abs_E,
                           double *track_E, double *total_abs_E, double *post_mat_E);

/* Adjoint replay (no upstream counterpart): dL/dsigma_a per cell for
 * L = sum_c w_c abs_E[c], from the start states of one step's photons and
 * the step's op_a/op_s/f, with the estimator and the 128-bit fixed-point
 * sums (exponent `scale`) of the GPU backward.  Visits whose contribution
 * exceeds visit_bound are dropped and counted (the return value). */
uint64_t bo_adjoint_replay(const bo_mesh *m, const bo_cells *c, uint32_t seed, const bo_photon *start,
                           size_t n, const double *w, int scale, double visit_bound, double *grad,
                           int n_threads);
/* L at perturbed opacities/Fleck factors (op_a_p, f_p) estimated on the
 * unperturbed paths with causal likelihood ratios; its finite difference
 * reproduces bo_adjoint_replay's per-history terms. */
double bo_adjoint_reweighted(const bo_mesh *m, const bo_cells *c, const double *op_a_p, const double *f_p,
                             uint32_t seed, const bo_photon *start, size_t n, const double *w);

#ifdef __cplusplus
}
#endif
#endif
