/*
 * branson_oracle.c — CPU restatement of Branson's replicated-mode IMC step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; see branson_oracle.h).  Written in
 * plain C from the upstream algorithm; each function keeps the upstream
 * floating-point operation order so that, built with -ffp-contract=off and
 * the same libm, it reproduces the upstream CPU path bit for bit.  Citations
 * are file:line within the upstream src/ directory.
 */
#include "branson_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Constants namespace (constants.h:16-24) */
static const double BO_PI = 3.1415926535897932384626433832795;
static const double BO_C = 299.792458;  /* cm/shake */
static const double BO_A = 0.01372;     /* GJ/cm^3/keV^4 */
static const double BO_CUTOFF = 0.01;

/* The transcendental functions of the photon arithmetic.  The default build
 * calls the host libm, as the upstream code does: that build is the oracle.
 * The BO_GPU_MATH build (make -C oracle gpumath) is a diagnostic twin: the
 * same C with -log(u), exp(x) and sin/cos(phi) taken from the GPU path's
 * integer fixed-point routines compiled for the host (oracle/gpu_math.cc),
 * and the boundary-source polar angle from cos(acos(sqrt u)) = sqrt(u),
 * sin(acos(sqrt u)) = sqrt(1 - u), as the GPU sources it.  Everything else
 * is IEEE arithmetic in the upstream order in both builds, so a history on
 * which the GPU and the oracle disagree, while the GPU and the twin agree,
 * differs only through the last-bit rounding of those functions; the
 * per-segment trace (bo_trace_photon) of both builds then locates the
 * comparison at which the two paths parted. */
#ifdef BO_GPU_MATH
double bo_gm_neg_log_u53(uint64_t m);
double bo_gm_exp_neg(double t);
void bo_gm_sincos_phi(double phi, double *s, double *c);
/* u is an RNG draw m * 2^-53 (odd m < 2^53), so m is recovered exactly */
static inline double neg_log_u(double u) { return bo_gm_neg_log_u53((uint64_t)(u * 9007199254740992.0)); }
static inline double exp_of(double x) { return bo_gm_exp_neg(-x); }
static inline void sincos_of(double phi, double *s, double *c) { bo_gm_sincos_phi(phi, s, c); }
#else
static inline double neg_log_u(double u) { return -log(u); }
static inline double exp_of(double x) { return exp(x); }
static inline void sincos_of(double phi, double *s, double *c) {
  *s = sin(phi);
  *c = cos(phi);
}
#endif

/* ------------------------------------------------------------------------ */
/* Threefry2x64 with 20 rounds, restated from the published Random123
 * specification (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11): rotation schedule for the 2x64 variant and the
 * Threefish key-schedule parity word; key injected every four rounds with
 * the injection index added to the last word.  Matches threefry.h:190-293
 * (Nrounds = 20, threefry.h:178-179). */
static inline uint64_t rotl64(uint64_t x, unsigned r) { return (x << r) | (x >> (64u - r)); }

#define BO_MIX(R)          \
  do {                     \
    x0 += x1;              \
    x1 = rotl64(x1, (R));  \
    x1 ^= x0;              \
  } while (0)

/* the 20 rounds with their rotation schedule written out, key injections
 * 1..5 after every fourth round */
static inline void threefry_rounds(uint64_t *p0, uint64_t *p1, const uint64_t ks[3]) {
  uint64_t x0 = *p0 + ks[0], x1 = *p1 + ks[1];
  BO_MIX(16); BO_MIX(42); BO_MIX(12); BO_MIX(31);
  x0 += ks[1]; x1 += ks[2] + 1u;
  BO_MIX(16); BO_MIX(32); BO_MIX(24); BO_MIX(21);
  x0 += ks[2]; x1 += ks[0] + 2u;
  BO_MIX(16); BO_MIX(42); BO_MIX(12); BO_MIX(31);
  x0 += ks[0]; x1 += ks[1] + 3u;
  BO_MIX(16); BO_MIX(32); BO_MIX(24); BO_MIX(21);
  x0 += ks[1]; x1 += ks[2] + 4u;
  BO_MIX(16); BO_MIX(42); BO_MIX(12); BO_MIX(31);
  x0 += ks[2]; x1 += ks[0] + 5u;
  *p0 = x0;
  *p1 = x1;
}
#undef BO_MIX

void bo_threefry2x64_20(const uint64_t ctr[2], const uint64_t key[2], uint64_t out[2]) {
  const uint64_t ks[3] = {key[0], key[1], 0x1BD11BDAA9FC1A22ULL ^ key[0] ^ key[1]};
  uint64_t x0 = ctr[0], x1 = ctr[1];
  threefry_rounds(&x0, &x1, ks);
  out[0] = x0;
  out[1] = x1;
}

typedef struct {
  uint64_t ks[3];   /* key schedule of {stream, 0} */
  uint64_t hi;      /* counter high word: seed << 32 */
  uint64_t counter; /* counter low word */
} bo_rng;

static inline void rng_init(bo_rng *r, uint32_t seed, uint64_t stream, uint64_t counter) {
  r->ks[0] = stream;
  r->ks[1] = 0;
  r->ks[2] = 0x1BD11BDAA9FC1A22ULL ^ stream;
  r->hi = (uint64_t)seed << 32;
  r->counter = counter;
}

/* _ran (RNG.h:262-285): counter {data[0], data[1] = seed<<32}, key
 * {stream, 0}; the counter advances by one per draw; the first output word
 * becomes u01fixedpt<double>: ((w >> 11) | 1) * 2^-53 (RNG.h:202-238). */
static inline double rng_next(bo_rng *r) {
  uint64_t x0 = r->counter, x1 = r->hi;
  threefry_rounds(&x0, &x1, r->ks);
  r->counter += 1; /* array.h:133-141; the high word never carries in practice */
  return (double)((x0 >> 11) | 1u) * (1.0 / 9007199254740992.0);
}

double bo_rng_draw(uint32_t seed, uint64_t stream, uint64_t *counter) {
  bo_rng r;
  rng_init(&r, seed, stream, *counter);
  const double u = rng_next(&r);
  *counter = r.counter;
  return u;
}

/* ------------------------------------------------------------------------ */
/* geometry */

void bo_cell_nodes(const bo_mesh *m, uint32_t g, double nodes[6]) {
  const uint32_t i = g % m->ngx;
  const uint32_t j = (g / m->ngx) % m->ngy;
  const uint32_t k = g / (m->ngx * m->ngy);
  nodes[0] = m->x[i];
  nodes[1] = m->x[i + 1];
  nodes[2] = m->y[j];
  nodes[3] = m->y[j + 1];
  nodes[4] = m->z[k];
  nodes[5] = m->z[k + 1];
}

/* Cell::get_volume (cell.h:188-191) */
static inline double cell_volume(const double n[6]) {
  return (n[1] - n[0]) * (n[3] - n[2]) * (n[5] - n[4]);
}

/* Boundary code and neighbour of face `face` of cell g: interior faces are
 * ELEMENT, domain faces carry the deck's boundary (proto_mesh.h:156-202). */
static inline int cell_bc(const bo_mesh *m, uint32_t g, uint32_t face, uint32_t *next) {
  const uint32_t i = g % m->ngx;
  const uint32_t j = (g / m->ngx) % m->ngy;
  const uint32_t k = g / (m->ngx * m->ngy);
  const uint32_t sxy = m->ngx * m->ngy;
  switch (face) {
  case 0: if (i > 0) { *next = g - 1; return BO_ELEMENT; } break;
  case 1: if (i + 1 < m->ngx) { *next = g + 1; return BO_ELEMENT; } break;
  case 2: if (j > 0) { *next = g - m->ngx; return BO_ELEMENT; } break;
  case 3: if (j + 1 < m->ngy) { *next = g + m->ngx; return BO_ELEMENT; } break;
  case 4: if (k > 0) { *next = g - sxy; return BO_ELEMENT; } break;
  default: if (k + 1 < m->ngz) { *next = g + sxy; return BO_ELEMENT; } break;
  }
  *next = g;
  return m->bc[face];
}

/* Cell::get_source_face (cell.h:69-76): first face whose bc is SOURCE. */
static int cell_source_face(const bo_mesh *m, uint32_t g) {
  for (uint32_t f = 0; f < 6; ++f) {
    uint32_t nxt;
    if (cell_bc(m, g, f, &nxt) == BO_SOURCE)
      return (int)f;
  }
  return -1;
}

/* Cell::get_face_area (cell.h:83-100) */
static double face_area(const double n[6], int face) {
  if (face == 0 || face == 1)
    return (n[3] - n[2]) * (n[5] - n[4]);
  if (face == 2 || face == 3)
    return (n[1] - n[0]) * (n[5] - n[4]);
  if (face == 4 || face == 5)
    return (n[1] - n[0]) * (n[3] - n[2]);
  return -1.0;
}

/* Cell::get_distance_to_boundary (cell.h:117-132), sgn (cell.h:23-25) */
static inline double distance_to_boundary(const double nodes[6], const double pos[3],
                                          const double dir[3], uint32_t *surface_cross) {
  double min_dist = 1.0e16;
  for (uint32_t i = 0; i < 3; i++) {
    const uint32_t index = 2 * i + (uint32_t)(0.0 < dir[i]);
    const double dist = (nodes[index] - pos[i]) / dir[i];
    if (dist < min_dist) {
      min_dist = dist;
      *surface_cross = index;
    }
  }
  return min_dist;
}

double bo_distance_to_boundary(const double nodes[6], const double pos[3], const double dir[3],
                               uint32_t *surface_cross) {
  return distance_to_boundary(nodes, pos, dir, surface_cross);
}

/* ------------------------------------------------------------------------ */
/* mesh physics */

void bo_initialize_cells(const bo_mesh *m, bo_cells *c) {
  const uint32_t n = m->ngx * m->ngy * m->ngz;
  for (uint32_t g = 0; g < n; ++g) {
    const bo_region *r = &m->regions[m->region[g]];
    c->T_e[g] = r->T_e;
    c->T_r[g] = r->T_r;
    c->T_s[g] = cell_source_face(m, g) != -1 ? m->T_source : 0.0; /* mesh.h:436-437 */
  }
}

/* Mesh::calculate_photon_energy (mesh.h:237-323) with one rank: the
 * replicated factor is 1 and the replicated redistribution (:291-315) leaves
 * every energy unchanged, so total_photon_E is the first pass's sum. */
void bo_calculate_photon_energy(const bo_mesh *m, bo_cells *c, uint32_t step, double dt,
                                bo_energy *out) {
  const uint32_t n = m->ngx * m->ngy * m->ngz;
  const double rf = 1.0;
  double total = 0.0, tot_em = 0.0, tot_ce = 0.0, tot_so = 0.0, pre_mat = 0.0;
  for (uint32_t g = 0; g < n; ++g) {
    const bo_region *r = &m->regions[m->region[g]];
    double nodes[6];
    bo_cell_nodes(m, g, nodes);
    const double vol = cell_volume(nodes);
    const double cV = r->cv, rho = r->rho;
    const double T = c->T_e[g], Tr = c->T_r[g], Ts = c->T_s[g];
    const double op_a = r->opacA + r->opacB * pow(T, r->opacC); /* region.h:44-46 */
    const double op_s = r->opacS;
    const double f = 1.0 / (1.0 + dt * op_a * BO_C * (4.0 * BO_A * pow(T, 3) / (cV * rho)));
    c->op_a[g] = op_a;
    c->op_s[g] = op_s;
    c->f[g] = f;
    c->emission_E[g] = rf * dt * vol * f * op_a * BO_A * BO_C * pow(T, 4);
    if (step > 1)
      c->census_E[g] = 0.0;
    else
      c->census_E[g] = rf * vol * BO_A * pow(Tr, 4);
    c->source_E[g] = rf * 0.25 * BO_A * BO_C * face_area(nodes, cell_source_face(m, g)) *
                     pow(Ts, 4) * dt;
    pre_mat += T * cV * vol * rho;
    tot_em += c->emission_E[g];
    tot_ce += c->census_E[g];
    tot_so += c->source_E[g];
    total += c->source_E[g] + c->census_E[g] + c->emission_E[g];
  }
  out->total_photon_E = total;
  out->emission_E = tot_em;
  out->census_E = tot_ce;
  out->source_E = tot_so;
  out->pre_mat_E = pre_mat;
}

/* photon count for one cell's energy (source.h:229-243): at least one. */
static inline uint32_t photons_for(uint64_t n_user, double E, double total_E) {
  if (!(E > 0.0))
    return 0;
  uint32_t t = (uint32_t)(int)((double)n_user * E / total_E);
  return t == 0 ? 1u : t;
}

uint64_t bo_count_photons(const bo_mesh *m, const bo_cells *c, uint64_t n_user, double total_E) {
  const uint32_t n = m->ngx * m->ngy * m->ngz;
  uint64_t total = 0;
  for (uint32_t g = 0; g < n; ++g)
    total += photons_for(n_user, c->emission_E[g], total_E) +
             photons_for(n_user, c->source_E[g], total_E);
  return total;
}

uint64_t bo_count_initial_census(const bo_mesh *m, const bo_cells *c, uint64_t n_user,
                                 double total_E) {
  const uint32_t n = m->ngx * m->ngy * m->ngz;
  uint64_t total = 0;
  for (uint32_t g = 0; g < n; ++g)
    total += photons_for(n_user, c->census_E[g], total_E);
  return total;
}

/* get_uniform_position_in_cell (sampling_functions.h:22-29) */
static void uniform_position_in_cell(const double n[6], bo_rng *r, double pos[3]) {
  pos[0] = n[0] + rng_next(r) * (n[1] - n[0]);
  pos[1] = n[2] + rng_next(r) * (n[3] - n[2]);
  pos[2] = n[4] + rng_next(r) * (n[5] - n[4]);
}

/* get_uniform_position_on_face (sampling_functions.h:32-52) */
static void uniform_position_on_face(const double n[6], bo_rng *r, int face, double pos[3]) {
  if (face == 0 || face == 1) {
    pos[0] = (face == 0) ? n[0] : n[1];
    pos[1] = n[2] + rng_next(r) * (n[3] - n[2]);
    pos[2] = n[4] + rng_next(r) * (n[5] - n[4]);
  } else if (face == 2 || face == 3) {
    pos[0] = n[0] + rng_next(r) * (n[1] - n[0]);
    pos[1] = (face == 2) ? n[2] : n[3];
    pos[2] = n[4] + rng_next(r) * (n[5] - n[4]);
  } else {
    pos[0] = n[0] + rng_next(r) * (n[1] - n[0]);
    pos[1] = n[2] + rng_next(r) * (n[3] - n[2]);
    pos[2] = (face == 4) ? n[4] : n[5];
  }
}

/* get_uniform_angle (sampling_functions.h:57-70) */
static void uniform_angle(bo_rng *r, double dir[3]) {
  const double mu = rng_next(r) * 2.0 - 1.0;
  const double phi = rng_next(r) * 2.0 * BO_PI;
  const double sin_theta = sqrt(1.0 - mu * mu);
  double sp, cp;
  sincos_of(phi, &sp, &cp);
  dir[0] = sin_theta * cp;
  dir[1] = sin_theta * sp;
  dir[2] = mu;
}

/* get_source_angle_on_face (sampling_functions.h:94-121); only the x faces
 * carry the inward sign, as upstream. */
static void source_angle_on_face(bo_rng *r, int face, double dir[3]) {
#ifdef BO_GPU_MATH
  const double u = rng_next(r);
  const double ct = sqrt(u), st = sqrt(1.0 - u);
#else
  const double theta = acos(sqrt(rng_next(r)));
  const double ct = cos(theta), st = sin(theta);
#endif
  const double phi = rng_next(r) * 2.0 * BO_PI;
  const double sign = (face % 2) ? -1.0 : 1.0;
  double sp, cp;
  sincos_of(phi, &sp, &cp);
  if (face == 0 || face == 1) {
    dir[0] = ct * sign;
    dir[1] = st * sp;
    dir[2] = st * cp;
  } else if (face == 2 || face == 3) {
    dir[0] = st * sp;
    dir[1] = ct;
    dir[2] = st * cp;
  } else {
    dir[0] = st * cp;
    dir[1] = st * sp;
    dir[2] = ct;
  }
}

/* get_emission_photon (source.h:84-97): 7 draws */
static void emission_photon(const bo_mesh *m, uint32_t g, double E, double dt, uint32_t seed,
                            uint64_t stream, bo_photon *p) {
  double n[6];
  bo_cell_nodes(m, g, n);
  bo_rng r;
  rng_init(&r, seed, stream, 0);
  memset(p, 0, sizeof(*p));
  p->source_type = 2;
  uniform_position_in_cell(n, &r, p->pos);
  uniform_angle(&r, p->dir);
  p->E = E; /* Photon::set_E0 sets both (photon.h:128-131) */
  p->E0 = E;
  p->cell = g;
  p->life_dx = rng_next(&r) * BO_C * dt;
  p->group = (uint32_t)floor(rng_next(&r) * (double)m->n_groups);
  p->stream = stream;
  p->counter = r.counter;
  p->descriptor = BO_PASS;
}

/* get_boundary_source_photon (source.h:100-114): 6 draws */
static void boundary_source_photon(const bo_mesh *m, uint32_t g, double E, double dt,
                                   uint32_t seed, uint64_t stream, int face, bo_photon *p) {
  double n[6];
  bo_cell_nodes(m, g, n);
  bo_rng r;
  rng_init(&r, seed, stream, 0);
  memset(p, 0, sizeof(*p));
  p->source_type = 1;
  uniform_position_on_face(n, &r, face, p->pos);
  source_angle_on_face(&r, face, p->dir);
  p->E = E; /* Photon::set_E0 sets both (photon.h:128-131) */
  p->E0 = E;
  p->cell = g;
  p->life_dx = rng_next(&r) * BO_C * dt;
  p->group = (uint32_t)floor(rng_next(&r) * (double)m->n_groups);
  p->stream = stream;
  p->counter = r.counter;
  p->descriptor = BO_PASS;
}

/* get_initial_census_photon (source.h:117-131): 6 draws */
static void initial_census_photon(const bo_mesh *m, uint32_t g, double E, double dt,
                                  uint32_t seed, uint64_t stream, bo_photon *p) {
  double n[6];
  bo_cell_nodes(m, g, n);
  bo_rng r;
  rng_init(&r, seed, stream, 0);
  memset(p, 0, sizeof(*p));
  p->source_type = 0;
  uniform_position_in_cell(n, &r, p->pos);
  uniform_angle(&r, p->dir);
  p->E = E; /* Photon::set_E0 sets both (photon.h:128-131) */
  p->E0 = E;
  p->cell = g;
  p->life_dx = BO_C * dt;
  p->group = (uint32_t)floor(rng_next(&r) * (double)m->n_groups);
  p->stream = stream;
  p->counter = r.counter;
  p->descriptor = BO_PASS;
}

/* make_photons (source.h:294-366), rank 0: stream = 1e13*cycle + ith.  The
 * upstream loop walks the cells in order with a running photon index ith;
 * every photon depends only on its cell, its energy and its stream, so the
 * cells are made in parallel from the prefix sums of their counts (the same
 * photons at the same list positions, only faster to build). */
void bo_make_photons(const bo_mesh *m, const bo_cells *c, double dt, uint32_t cycle, uint32_t seed,
                     uint64_t n_user, double total_E, bo_photon *out) {
  const uint32_t n = m->ngx * m->ngy * m->ngz;
  const uint64_t cycle_offset = 10000000000000ULL * (uint64_t)cycle;
  uint64_t *first = (uint64_t *)malloc(((size_t)n + 1) * sizeof(uint64_t));
  uint64_t ith = 0;
  for (uint32_t g = 0; g < n; ++g) {
    first[g] = ith;
    ith += photons_for(n_user, c->emission_E[g], total_E) + photons_for(n_user, c->source_E[g], total_E);
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (long gl = 0; gl < (long)n; ++gl) {
    const uint32_t g = (uint32_t)gl;
    uint64_t k = first[g];
    const uint32_t n_em = photons_for(n_user, c->emission_E[g], total_E);
    if (n_em) {
      const double E = c->emission_E[g] / n_em;
      for (uint32_t p = 0; p < n_em; ++p, ++k)
        emission_photon(m, g, E, dt, seed, cycle_offset + k, &out[k]);
    }
    const uint32_t n_so = photons_for(n_user, c->source_E[g], total_E);
    if (n_so) {
      const double E = c->source_E[g] / n_so;
      const int face = cell_source_face(m, g);
      for (uint32_t p = 0; p < n_so; ++p, ++k)
        boundary_source_photon(m, g, E, dt, seed, cycle_offset + k, face, &out[k]);
    }
  }
  free(first);
}

/* make_initial_census_photons (source.h:183-204), rank 0: stream = ith;
 * cells in parallel from the prefix sums of their counts, as above. */
void bo_make_initial_census(const bo_mesh *m, const bo_cells *c, double dt, uint32_t seed,
                            uint64_t n_user, double total_E, bo_photon *out) {
  const uint32_t n = m->ngx * m->ngy * m->ngz;
  uint64_t *first = (uint64_t *)malloc(((size_t)n + 1) * sizeof(uint64_t));
  uint64_t ith = 0;
  for (uint32_t g = 0; g < n; ++g) {
    first[g] = ith;
    ith += photons_for(n_user, c->census_E[g], total_E);
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (long gl = 0; gl < (long)n; ++gl) {
    const uint32_t g = (uint32_t)gl;
    uint64_t k = first[g];
    const uint32_t n_ce = photons_for(n_user, c->census_E[g], total_E);
    if (n_ce) {
      const double E = c->census_E[g] / n_ce;
      for (uint32_t p = 0; p < n_ce; ++p, ++k)
        initial_census_photon(m, g, E, dt, seed, k, &out[k]);
    }
  }
  free(first);
}

/* ------------------------------------------------------------------------ */
/* transport */

/* sample_emission_group, Cell version (sampling_functions.h:126-138), with
 * every group's opacity equal to op_a (Cell::set_op_a, cell.h:260-266).  A
 * walk that runs past the last group (possible only when u rounds above the
 * accumulated CDF) reads past the group array upstream; here it stays in
 * the last group. */
static uint32_t sample_emission_group(bo_rng *r, double op_a, uint32_t n_groups) {
  double cdf_value = rng_next(r);
  int new_group = -1;
  const double norm_factor = 1.0 / (op_a * (double)n_groups);
  while (cdf_value > 0) {
    new_group++;
    cdf_value -= op_a * norm_factor;
    if ((uint32_t)new_group == n_groups - 1)
      break;
  }
  if (new_group < 0)
    new_group = 0;
  return (uint32_t)new_group;
}

/* transport_photon, AoS form (history_based_transport.h:33-141).  The cell
 * is tracked by its (i, j, k) position so that nodes, neighbours and
 * boundary codes come from the plane arrays without any division, the way
 * the upstream loop reads them from its precomputed Cell. */
static inline __attribute__((always_inline)) uint64_t
transport_photon_traced(const bo_mesh *m, const bo_cells *c, uint32_t seed, bo_photon *p, double *abs_t,
                        double *track_t, bo_trace_rec *trace, size_t trace_cap) {
  bo_rng r;
  rng_init(&r, seed, p->stream, p->counter);
  uint32_t surface_cross = 0;
  uint32_t cell = p->cell;
  const uint32_t sxy = m->ngx * m->ngy;
  uint32_t ci = cell % m->ngx, cj = (cell / m->ngx) % m->ngy, ck = cell / sxy;
  double nodes[6] = {m->x[ci], m->x[ci + 1], m->y[cj], m->y[cj + 1], m->z[ck], m->z[ck + 1]};
  double thread_abs = 0.0, thread_track = 0.0;
  uint64_t segments = 0;
  int active = 1;
  while (active) {
    ++segments;
    const uint32_t seg_cell = cell;
    (void)seg_cell;
    const double sigma_s = c->op_s[cell];
    const double sigma_a = c->op_a[cell];
    const double f = c->f[cell];
    const double total_sigma_s = (1.0 - f) * sigma_a + sigma_s;
    const double dist_to_scatter =
        (total_sigma_s > 0.0) ? neg_log_u(rng_next(&r)) / total_sigma_s : 1.0e100;
    const double dist_to_boundary = distance_to_boundary(nodes, p->pos, p->dir, &surface_cross);
    double face_q[3] = {0.0, 0.0, 0.0};
    if (trace)
      for (uint32_t i = 0; i < 3; ++i)
        face_q[i] = (nodes[2 * i + (uint32_t)(0.0 < p->dir[i])] - p->pos[i]) / p->dir[i];
    const double dist_to_census = p->life_dx;
    /* std::min(a, b) is (b < a) ? b : a */
    const double db_dc = (dist_to_census < dist_to_boundary) ? dist_to_census : dist_to_boundary;
    const double dist_to_event = (db_dc < dist_to_scatter) ? db_dc : dist_to_scatter;
    const double absorbed_E = p->E * (1.0 - exp_of(-sigma_a * f * dist_to_event));
    thread_abs += absorbed_E;
    thread_track += absorbed_E / (sigma_a * f);
    p->E = p->E - absorbed_E;
    p->pos[0] += p->dir[0] * dist_to_event; /* Photon::move (photon.h:109-114) */
    p->pos[1] += p->dir[1] * dist_to_event;
    p->pos[2] += p->dir[2] * dist_to_event;
    p->life_dx -= dist_to_event;
    if (p->E / p->E0 < BO_CUTOFF) { /* below_cutoff (photon.h:47-49) */
      thread_abs += p->E;
      abs_t[cell] += thread_abs;
      track_t[cell] += thread_track;
      active = 0;
      p->descriptor = BO_KILLED;
    } else if (dist_to_event == dist_to_scatter) {
      uniform_angle(&r, p->dir);
      if (rng_next(&r) > (sigma_s / ((1.0 - f) * sigma_a + sigma_s)))
        p->group = sample_emission_group(&r, sigma_a, m->n_groups);
      p->descriptor = BO_SCATTER;
    } else if (dist_to_event == dist_to_boundary) {
      /* interior faces are ELEMENT, domain faces carry the deck's boundary
       * (proto_mesh.h:156-202) */
      int interior;
      switch (surface_cross) {
      case 0: interior = ci > 0; break;
      case 1: interior = ci + 1 < m->ngx; break;
      case 2: interior = cj > 0; break;
      case 3: interior = cj + 1 < m->ngy; break;
      case 4: interior = ck > 0; break;
      default: interior = ck + 1 < m->ngz; break;
      }
      const int bc = interior ? BO_ELEMENT : m->bc[surface_cross];
      if (bc == BO_ELEMENT) {
        abs_t[cell] += thread_abs;
        track_t[cell] += thread_track;
        switch (surface_cross) {
        case 0: --ci; cell -= 1; break;
        case 1: ++ci; cell += 1; break;
        case 2: --cj; cell -= m->ngx; break;
        case 3: ++cj; cell += m->ngx; break;
        case 4: --ck; cell -= sxy; break;
        default: ++ck; cell += sxy; break;
        }
        p->cell = cell;
        nodes[0] = m->x[ci]; nodes[1] = m->x[ci + 1];
        nodes[2] = m->y[cj]; nodes[3] = m->y[cj + 1];
        nodes[4] = m->z[ck]; nodes[5] = m->z[ck + 1];
        p->descriptor = BO_BOUND;
        thread_abs = 0.0;
        thread_track = 0.0;
      } else if (bc == BO_VACUUM || bc == BO_SOURCE) {
        active = 0;
        p->descriptor = BO_EXIT;
        abs_t[cell] += thread_abs;
        track_t[cell] += thread_track;
      } else { /* REFLECT: Photon::reflect (photon.h:151-155) */
        p->dir[surface_cross / 2] = -p->dir[surface_cross / 2];
        p->descriptor = BO_BOUND;
      }
    } else if (dist_to_event == dist_to_census) {
      active = 0;
      p->descriptor = BO_CENSUS;
      abs_t[cell] += thread_abs;
      track_t[cell] += thread_track;
    }
    if (trace && segments <= trace_cap) {
      bo_trace_rec *t = &trace[segments - 1];
      t->d_scatter = dist_to_scatter;
      t->d_boundary = dist_to_boundary;
      t->d_census = dist_to_census;
      t->face_q[0] = face_q[0];
      t->face_q[1] = face_q[1];
      t->face_q[2] = face_q[2];
      t->E = p->E;
      t->E0 = p->E0;
      t->cell = seg_cell;
      t->descriptor = p->descriptor;
      t->surface = surface_cross;
      t->counter = (uint32_t)r.counter;
    }
  }
  p->counter = r.counter;
  return segments;
}

static uint64_t transport_photon(const bo_mesh *m, const bo_cells *c, uint32_t seed, bo_photon *p,
                                 double *abs_t, double *track_t) {
  return transport_photon_traced(m, c, seed, p, abs_t, track_t, NULL, 0);
}

size_t bo_trace_photon(const bo_mesh *m, const bo_cells *c, uint32_t seed, const bo_photon *start,
                       bo_trace_rec *out, size_t max_segments, bo_photon *end) {
  const size_t n_cells = (size_t)m->ngx * m->ngy * m->ngz;
  double *t = (double *)calloc(2 * n_cells, sizeof(double));
  bo_photon p = *start;
  const uint64_t segs = transport_photon_traced(m, c, seed, &p, t, t + n_cells, out, max_segments);
  free(t);
  if (end)
    *end = p;
  return (size_t)segs;
}

/* history_cpu_transport_photons (history_based_transport.h:279-308):
 * OpenMP guided loop, one tally array per thread, merged cell by cell in
 * thread order. */
uint64_t bo_transport(const bo_mesh *m, const bo_cells *c, uint32_t seed, bo_photon *photons,
                      size_t n, double *abs_E, double *track_E, int n_threads) {
  const size_t n_cells = (size_t)m->ngx * m->ngy * m->ngz;
  int nt = 1;
#ifdef _OPENMP
  nt = n_threads > 0 ? n_threads : omp_get_max_threads();
#else
  (void)n_threads;
#endif
  double *tallies = (double *)calloc((size_t)nt * n_cells * 2, sizeof(double));
  uint64_t segments = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt) reduction(+ : segments)
#endif
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    double *ta = tallies + (size_t)t * n_cells * 2;
    double *tt = ta + n_cells;
#ifdef _OPENMP
#pragma omp for schedule(guided)
#endif
    for (long i = 0; i < (long)n; ++i)
      segments += transport_photon(m, c, seed, &photons[i], ta, tt);
  }
  for (size_t g = 0; g < n_cells; ++g) {
    double a = 0.0, tr = 0.0; /* Cell_Tally starts at zero (cell_tally.h:32-34) */
    for (int t = 0; t < nt; ++t) {
      a += tallies[(size_t)t * n_cells * 2 + g];
      tr += tallies[(size_t)t * n_cells * 2 + n_cells + g];
    }
    abs_E[g] = a;
    track_E[g] = tr;
  }
  free(tallies);
  return segments;
}

/* post_process_photons, AoS (post_process_functions.h:33-59) */
size_t bo_post_process(double next_dt, bo_photon *photons, size_t n, bo_photon *census_out,
                       double *census_E, double *exit_E) {
  size_t nc = 0;
  for (size_t i = 0; i < n; ++i) {
    bo_photon *p = &photons[i];
    if (p->descriptor == BO_EXIT) {
      *exit_E += p->E;
    } else if (p->descriptor == BO_CENSUS) {
      p->life_dx = BO_C * next_dt;
      if (census_out)
        census_out[nc] = *p;
      ++nc;
      *census_E += p->E;
    }
  }
  return nc;
}

/* comb_photons (census_functions.h:48-93) */
size_t bo_comb_census(const bo_photon *photons, size_t n, uint32_t n_cells, int64_t max_census, uint32_t seed,
                      uint64_t stream, uint64_t *counter, bo_photon *out) {
  /* get_photon_list_E (census_functions.h:40-46); the allreduce is one rank */
  double census_E = 0.0;
  for (size_t k = 0; k < n; ++k) census_E += photons[k].E;
  const double comb_E = census_E / (double)max_census;
  uint32_t *count = calloc(n_cells ? n_cells : 1, sizeof(uint32_t));
  double *cell_E = calloc(n_cells ? n_cells : 1, sizeof(double));
  double *corrected = calloc(n_cells ? n_cells : 1, sizeof(double));
  for (size_t k = 0; k < n; ++k) {
    count[photons[k].cell]++;
    cell_E[photons[k].cell] += photons[k].E;
  }
  bo_rng r;
  rng_init(&r, seed, stream, *counter);
  size_t m = 0;
  for (size_t k = 0; k < n; ++k) {
    const bo_photon p = photons[k];
    const uint32_t cell = p.cell;
    const double p_kill = 1.0 - p.E / comb_E;
    const double u = rng_next(&r);
    if (u > p_kill || count[cell] == 1) {
      out[m] = p;
      out[m].E = comb_E;
      corrected[cell] += comb_E;
      ++m;
    } else {
      count[cell]--;
    }
  }
  for (size_t j = 0; j < m; ++j) {
    const uint32_t cell = out[j].cell;
    out[j].E = out[j].E + (cell_E[cell] - corrected[cell]) / (double)count[cell];
  }
  *counter = r.counter;
  free(count);
  free(cell_E);
  free(corrected);
  return m;
}

/* Mesh::update_temperature (mesh.h:349-362, :419-422) */
void bo_update_temperature(const bo_mesh *m, bo_cells *c, double dt, double *abs_E,
                           double *track_E, double *total_abs_E, double *post_mat_E) {
  const uint32_t n = m->ngx * m->ngy * m->ngz;
  double tot_abs = 0.0, tot_mat = 0.0;
  for (uint32_t g = 0; g < n; ++g) {
    const bo_region *r = &m->regions[m->region[g]];
    const double cV = r->cv, rho = r->rho;
    double nodes[6];
    bo_cell_nodes(m, g, nodes);
    const double vol = cell_volume(nodes);
    const double T = c->T_e[g];
    const double T_new = T + (abs_E[g] - c->emission_E[g]) / (cV * vol * rho);
    c->T_r_diag[g] = pow(track_E[g] / (vol * dt * BO_A * BO_C), 0.25);
    c->T_e[g] = T_new;
    tot_abs += abs_E[g];
    tot_mat += T_new * cV * vol * rho;
    abs_E[g] = 0.0;
    track_E[g] = 0.0;
  }
  *total_abs_E = tot_abs;
  *post_mat_E = tot_mat;
}

/* ------------------------------------------------------------------ adjoint
 * CPU replay of the GPU adjoint estimator (no upstream counterpart; the
 * estimator is documented in branson_gb300/csrc/bgs_adjoint.cu).  Each
 * history is walked with the statements of transport_photon above, so the
 * path is the forward one; per segment in cell j with length d:
 *   s = 1/sigma_eff - d (ended at the collision distance) or -d,
 *   A += (1-f^2) s - f^2 d,
 *   B += (1-f^2) s prefix_before - f^2 d (prefix_after + w_j W_after),
 * per cell visit G*A - B is added to the cell, and an emission photon adds
 * G f/sigma_a to its birth cell; G is the history's weighted deposit.  Sums
 * are 128-bit two's-complement fixed point with the truncating conversion
 * of the device code, so both give the same bits for the same histories. */
typedef struct {
  double f2, g2, inv_se, src;
} bo_adj_coef;

typedef struct {
  uint32_t cell;
  double a, b;
} bo_visit;

typedef struct {
  bo_visit *v;
  size_t n, cap;
} bo_visit_log;

static void visit_push(bo_visit_log *L, uint32_t cell, double a, double b) {
  if (L->n == L->cap) {
    L->cap = L->cap ? 2 * L->cap : 64;
    L->v = (bo_visit *)realloc(L->v, L->cap * sizeof(bo_visit));
  }
  L->v[L->n].cell = cell;
  L->v[L->n].a = a;
  L->v[L->n].b = b;
  ++L->n;
}

/* floor(|x| * 2^scale) as a 128-bit integer, negated for x < 0; 0 if out of
 * range (the caller checks the range first) */
static unsigned __int128 fixed128_signed(double x, int scale) {
  const double ax = fabs(x);
  uint64_t bits;
  memcpy(&bits, &ax, sizeof(bits));
  const int e = (int)((bits >> 52) & 0x7FF);
  unsigned __int128 v = 0;
  if (e != 0 && e != 0x7FF) {
    const uint64_t mant = (bits & 0x000FFFFFFFFFFFFFULL) | 0x0010000000000000ULL;
    const int sh = e - 1075 + scale;
    if (sh >= 0) {
      if (sh <= 74) v = (unsigned __int128)mant << sh;
    } else if (sh > -64) {
      v = (unsigned __int128)(mant >> (-sh));
    }
  }
  return x < 0.0 ? (unsigned __int128)0 - v : v;
}

static double fixed128_to_double(unsigned __int128 v, int scale) {
  const int neg = (int)(v >> 127);
  if (neg) v = (unsigned __int128)0 - v;
  const uint64_t hi = (uint64_t)(v >> 64), lo = (uint64_t)v;
  const double d = (double)hi * 18446744073709551616.0 + (double)lo;
  const double r = scalbn(d, -scale);
  return neg ? -r : r;
}

/* One history replayed from its start state.  Fills `log` with its cell
 * visits (A, B) and returns G.  With op_a_p/f_p (perturbed opacities and
 * Fleck factors) it also returns, in *L_rw, the history's contribution to
 * L at the perturbed opacities estimated on this same path: weights decay
 * with the perturbed sigma_a f, an emission weight scales with f sigma_a,
 * and each deposit is multiplied by the likelihood ratio of the path's
 * segment lengths up to it (sigma_eff' exp(-sigma_eff' d) over sigma_eff
 * exp(-sigma_eff d) for collisions, exp(-(sigma_eff' - sigma_eff) d)
 * otherwise).  Its derivative at the unperturbed values is this history's
 * estimator term. */
static double adjoint_replay_photon(const bo_mesh *m, const bo_cells *c, const bo_adj_coef *k,
                                    uint32_t seed, const bo_photon *start, const double *w,
                                    bo_visit_log *visits, const double *op_a_p, const double *f_p,
                                    double *L_rw) {
  bo_photon ph = *start;
  bo_photon *p = &ph;
  bo_rng r;
  rng_init(&r, seed, p->stream, p->counter);
  uint32_t surface_cross = 0;
  uint32_t cell = p->cell;
  const uint32_t sxy = m->ngx * m->ngy;
  uint32_t ci = cell % m->ngx, cj = (cell / m->ngx) % m->ngy, ck = cell / sxy;
  double nodes[6] = {m->x[ci], m->x[ci + 1], m->y[cj], m->y[cj + 1], m->z[ck], m->z[ck + 1]};
  double prefix = 0.0, vis_a = 0.0, vis_b = 0.0;
  double W_rw = p->E, lr = 1.0, acc_rw = 0.0;
  visits->n = 0;
  if (p->source_type == 2) { /* emission: weight proportional to f sigma_a of the birth cell */
    visit_push(visits, cell, k[cell].src, 0.0);
    if (op_a_p) W_rw = p->E * ((f_p[cell] * op_a_p[cell]) / (c->f[cell] * c->op_a[cell]));
  }
  int active = 1;
  while (active) {
    const double sigma_s = c->op_s[cell];
    const double sigma_a = c->op_a[cell];
    const double f = c->f[cell];
    const double total_sigma_s = (1.0 - f) * sigma_a + sigma_s;
    const double dist_to_scatter =
        (total_sigma_s > 0.0) ? neg_log_u(rng_next(&r)) / total_sigma_s : 1.0e100;
    const double dist_to_boundary = distance_to_boundary(nodes, p->pos, p->dir, &surface_cross);
    const double dist_to_census = p->life_dx;
    const double db_dc = (dist_to_census < dist_to_boundary) ? dist_to_census : dist_to_boundary;
    const double dist_to_event = (db_dc < dist_to_scatter) ? db_dc : dist_to_scatter;
    const double absorbed_E = p->E * (1.0 - exp_of(-sigma_a * f * dist_to_event));
    p->E = p->E - absorbed_E;
    p->pos[0] += p->dir[0] * dist_to_event;
    p->pos[1] += p->dir[1] * dist_to_event;
    p->pos[2] += p->dir[2] * dist_to_event;
    p->life_dx -= dist_to_event;
    const int collided = !(db_dc < dist_to_scatter);
    const int killed = p->E / p->E0 < BO_CUTOFF;
    { /* estimator terms of this segment */
      const bo_adj_coef a = k[cell];
      const double wj = w[cell];
      const double d = dist_to_event;
      const double s = collided ? a.inv_se - d : -d;
      const double gs = a.g2 * s;
      const double pa = a.f2 * d;
      const double prev = prefix;
      prefix = fma(wj, absorbed_E, prefix);
      const double tail = fma(wj, p->E, prefix);
      vis_a = vis_a + (gs - pa);
      vis_b = fma(gs, prev, fma(-pa, tail, vis_b));
      if (killed) prefix = tail;
      if (op_a_p) {
        const double sp = op_a_p[cell], fp = f_p[cell];
        const double se_p = (1.0 - fp) * sp + sigma_s;
        lr *= exp(-(se_p - total_sigma_s) * d);
        if (collided) lr *= se_p / total_sigma_s;
        const double dep = W_rw * (1.0 - exp(-sp * fp * d));
        W_rw -= dep;
        acc_rw += wj * dep * lr;
        if (killed) acc_rw += wj * W_rw * lr;
      }
    }
    if (killed) {
      visit_push(visits, cell, vis_a, vis_b);
      active = 0;
    } else if (collided) {
      uniform_angle(&r, p->dir);
      if (rng_next(&r) > (sigma_s / ((1.0 - f) * sigma_a + sigma_s)))
        p->group = sample_emission_group(&r, sigma_a, m->n_groups);
    } else if (dist_to_event == dist_to_boundary) {
      int interior;
      switch (surface_cross) {
      case 0: interior = ci > 0; break;
      case 1: interior = ci + 1 < m->ngx; break;
      case 2: interior = cj > 0; break;
      case 3: interior = cj + 1 < m->ngy; break;
      case 4: interior = ck > 0; break;
      default: interior = ck + 1 < m->ngz; break;
      }
      const int bc = interior ? BO_ELEMENT : m->bc[surface_cross];
      if (bc == BO_ELEMENT) {
        visit_push(visits, cell, vis_a, vis_b);
        vis_a = 0.0;
        vis_b = 0.0;
        switch (surface_cross) {
        case 0: --ci; cell -= 1; break;
        case 1: ++ci; cell += 1; break;
        case 2: --cj; cell -= m->ngx; break;
        case 3: ++cj; cell += m->ngx; break;
        case 4: --ck; cell -= sxy; break;
        default: ++ck; cell += sxy; break;
        }
        nodes[0] = m->x[ci]; nodes[1] = m->x[ci + 1];
        nodes[2] = m->y[cj]; nodes[3] = m->y[cj + 1];
        nodes[4] = m->z[ck]; nodes[5] = m->z[ck + 1];
      } else if (bc == BO_VACUUM || bc == BO_SOURCE || bc == BO_PROCESSOR) {
        visit_push(visits, cell, vis_a, vis_b);
        active = 0;
      } else {
        p->dir[surface_cross / 2] = -p->dir[surface_cross / 2];
      }
    } else { /* census */
      visit_push(visits, cell, vis_a, vis_b);
      active = 0;
    }
  }
  if (L_rw) *L_rw = acc_rw;
  return prefix;
}

static bo_adj_coef *adjoint_coefs(const bo_cells *c, size_t n_cells) {
  bo_adj_coef *k = (bo_adj_coef *)malloc(n_cells * sizeof(bo_adj_coef));
  for (size_t g = 0; g < n_cells; ++g) {
    const double op_a = c->op_a[g], op_s = c->op_s[g], f = c->f[g];
    const double sig_eff = (1.0 - f) * op_a + op_s;
    k[g].f2 = f * f;
    k[g].g2 = 1.0 - f * f;
    k[g].inv_se = sig_eff > 0.0 ? 1.0 / sig_eff : 0.0;
    k[g].src = op_a > 0.0 ? f / op_a : 0.0;
  }
  return k;
}

uint64_t bo_adjoint_replay(const bo_mesh *m, const bo_cells *c, uint32_t seed, const bo_photon *start,
                           size_t n, const double *w, int scale, double visit_bound, double *grad,
                           int n_threads) {
  const size_t n_cells = (size_t)m->ngx * m->ngy * m->ngz;
  bo_adj_coef *k = adjoint_coefs(c, n_cells);
  int nt = 1;
#ifdef _OPENMP
  nt = n_threads > 0 ? n_threads : omp_get_max_threads();
#else
  (void)n_threads;
#endif
  unsigned __int128 *sums = (unsigned __int128 *)calloc((size_t)nt * n_cells, sizeof(unsigned __int128));
  uint64_t range_errors = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt) reduction(+ : range_errors)
#endif
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    unsigned __int128 *mine = sums + (size_t)t * n_cells;
    bo_visit_log log = {NULL, 0, 0};
#ifdef _OPENMP
#pragma omp for schedule(guided)
#endif
    for (long i = 0; i < (long)n; ++i) {
      const double G = adjoint_replay_photon(m, c, k, seed, &start[i], w, &log, NULL, NULL, NULL);
      for (size_t v = 0; v < log.n; ++v) {
        const double val = G * log.v[v].a - log.v[v].b;
        if (val == 0.0) continue;
        if (!(fabs(val) <= visit_bound)) {
          ++range_errors;
          continue;
        }
        mine[log.v[v].cell] += fixed128_signed(val, scale);
      }
    }
    free(log.v);
  }
  for (size_t g = 0; g < n_cells; ++g) {
    unsigned __int128 acc = 0;
    for (int t = 0; t < nt; ++t) acc += sums[(size_t)t * n_cells + g];
    grad[g] = fixed128_to_double(acc, scale);
  }
  free(sums);
  free(k);
  return range_errors;
}

double bo_adjoint_reweighted(const bo_mesh *m, const bo_cells *c, const double *op_a_p, const double *f_p,
                             uint32_t seed, const bo_photon *start, size_t n, const double *w) {
  const size_t n_cells = (size_t)m->ngx * m->ngy * m->ngz;
  bo_adj_coef *k = adjoint_coefs(c, n_cells);
  bo_visit_log log = {NULL, 0, 0};
  double L = 0.0;
  for (size_t i = 0; i < n; ++i) {
    double l = 0.0;
    adjoint_replay_photon(m, c, k, seed, &start[i], w, &log, op_a_p, f_p, &l);
    L += l;
  }
  free(log.v);
  free(k);
  return L;
}
