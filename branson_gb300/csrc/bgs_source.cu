// Photon sourcing on the device: initial census (step 1), emission and
// boundary-source photons (source.h:27-131, :134-366), written straight into
// the photon bank after the census already there.  One thread per photon;
// each photon finds its cell by binary search in the prefix-summed counts,
// so the photon order, stream numbers and energies are those of the
// upstream cell-order loops.
#include "bgs_fixmath.cuh"
#include "bgs_kernels.cuh"

namespace bgs {

// Bank bookkeeping of one step, all on the device: sizes from the prefix
// sums, capacity check, and the transport work queue reset.  The bank holds
// [census carried in | photons made this step]; at step 1 the carried census
// is the initial census (make_initial_census_photons, source.h:183-204).
__device__ __forceinline__ void plan_bank_body(const MeshDev &m, const CellsDev &c, DeviceDiag *d, uint32_t step,
                                               unsigned long long capacity) {
  const unsigned long long n_new = c.off_new[m.n_cells];
  const unsigned long long n_ic = step == 1 ? c.off_ce[m.n_cells] : 0ULL;
  if (step == 1) {
    d->n_census_in = n_ic;
    d->census_E_in = 0.0;
  }
  d->n_init_census = n_ic;
  unsigned long long made = n_new;
  if (d->n_census_in + n_new > capacity) {
    d->flags |= FLAG_CAPACITY;
    made = 0;
    if (step == 1) { d->n_census_in = 0; d->n_init_census = 0; }
  }
  d->n_new = made;
  d->n_bank = d->n_census_in + made;
  d->work_counter = 0;
  d->n_segments = 0;
}

__global__ void k_plan_bank(MeshDev m, CellsDev c, DeviceDiag *d, uint32_t step,
                            unsigned long long capacity) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  plan_bank_body(m, c, d, step, capacity);
}

// get_uniform_position_in_cell (sampling_functions.h:22-29)
__device__ __forceinline__ void position_in_cell(const double n[6], Rng &r, double p[3]) {
  p[0] = n[0] + r.next() * (n[1] - n[0]);
  p[1] = n[2] + r.next() * (n[3] - n[2]);
  p[2] = n[4] + r.next() * (n[5] - n[4]);
}

// get_uniform_angle (sampling_functions.h:57-70)
__device__ __forceinline__ void uniform_angle(Rng &r, double d[3]) {
  const double mu = mu_from_m53(r.next_m53());
  const double phi = r.next_twice() * kPi;  // RN(RN(u * 2.0) * pi), u * 2.0 exact
  const double sin_theta = sqrt(1.0 - mu * mu);
  double s, c;
  fix::sincos_phi(phi, &s, &c);
  d[0] = sin_theta * c;
  d[1] = sin_theta * s;
  d[2] = mu;
}

// get_uniform_position_on_face (sampling_functions.h:32-52)
__device__ __forceinline__ void position_on_face(const double n[6], Rng &r, int face, double p[3]) {
  if (face == 0 || face == 1) {
    p[0] = (face == 0) ? n[0] : n[1];
    p[1] = n[2] + r.next() * (n[3] - n[2]);
    p[2] = n[4] + r.next() * (n[5] - n[4]);
  } else if (face == 2 || face == 3) {
    p[0] = n[0] + r.next() * (n[1] - n[0]);
    p[1] = (face == 2) ? n[2] : n[3];
    p[2] = n[4] + r.next() * (n[5] - n[4]);
  } else {
    p[0] = n[0] + r.next() * (n[1] - n[0]);
    p[1] = n[2] + r.next() * (n[3] - n[2]);
    p[2] = (face == 4) ? n[4] : n[5];
  }
}

// get_source_angle_on_face (sampling_functions.h:94-121): the inward sign is
// applied on the x faces only, as upstream.
__device__ __forceinline__ void source_angle(Rng &r, int face, double d[3]) {
  // theta = acos(sqrt(u)): cos(theta) = sqrt(u) and sin(theta) = sqrt(1-u)
  // exactly, so both come from square roots instead of acos, sin and cos
  const double u = r.next();
  const double ct = sqrt(u);
  const double st = sqrt(1.0 - u);
  const double phi = r.next_twice() * kPi;  // RN(RN(u * 2.0) * pi), u * 2.0 exact
  const double sign = (face % 2) ? -1.0 : 1.0;
  double sp, cp;
  fix::sincos_phi(phi, &sp, &cp);
  if (face == 0 || face == 1) {
    d[0] = ct * sign;
    d[1] = st * sp;
    d[2] = st * cp;
  } else if (face == 2 || face == 3) {
    d[0] = st * sp;
    d[1] = ct;
    d[2] = st * cp;
  } else {
    d[0] = st * cp;
    d[1] = st * sp;
    d[2] = ct;
  }
}

// the photon's group, floor(u * n_groups) (source.h:94, :111, :128); with one
// group it is 0 whatever u is, so that draw only advances the counter
__device__ __forceinline__ uint32_t sample_uniform_group(Rng &r, uint32_t n_groups) {
  if (n_groups == 1) {
    r.skip();
    return 0u;
  }
  return (uint32_t)floor(r.next() * (double)n_groups);
}

// index of the cell whose [off[c], off[c+1]) range holds p
__device__ __forceinline__ uint32_t find_cell(const unsigned long long *off, uint32_t n_cells,
                                              unsigned long long p) {
  uint32_t lo = 0, hi = n_cells;  // off[lo] <= p < off[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (off[mid] <= p) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void store_photon(const Bank &b, unsigned long long i, const double p[3],
                                             const double d[3], double E, double life, uint32_t cell,
                                             uint32_t group, uint8_t stype, unsigned long long stream,
                                             unsigned long long ctr) {
  b.px[i] = p[0]; b.py[i] = p[1]; b.pz[i] = p[2];
  b.dx[i] = d[0]; b.dy[i] = d[1]; b.dz[i] = d[2];
  b.E[i] = E; b.E0[i] = E; b.life[i] = life;
  b.cell[i] = cell; b.group[i] = group;
  b.desc[i] = PASS; b.stype[i] = stype;
  b.stream[i] = stream; b.ctr[i] = ctr;
}

// Initial census photons (get_initial_census_photon, source.h:117-131):
// stream = ith census photon (rank 0), 6 draws, life = c*dt.
__device__ __forceinline__ void source_census_body(const MeshDev &m, const CellsDev &c, const Bank &b,
                                                   const DeviceDiag *d, unsigned long long seed_hi, double dt,
                                                   uint32_t bx, uint32_t nbx) {
  const unsigned long long n = d->n_init_census;
  for (unsigned long long p = bx * (unsigned long long)blockDim.x + threadIdx.x; p < n;
       p += (unsigned long long)nbx * blockDim.x) {
    const uint32_t g = find_cell(c.off_ce, m.n_cells, p);
    double nodes[6], pos[3], dir[3];
    cell_nodes(m, g, nodes);
    Rng r{p, 0ULL, seed_hi};
    position_in_cell(nodes, r, pos);
    uniform_angle(r, dir);
    const double E = c.ce_E[g] / (double)c.n_ce[g];
    const uint32_t group = sample_uniform_group(r, m.n_groups);
    store_photon(b, p, pos, dir, E, kC * dt, g, group, 0, p, r.ctr);
  }
}

__global__ void k_source_census(MeshDev m, CellsDev c, Bank b, const DeviceDiag *d,
                                unsigned long long seed_hi, double dt) {
  source_census_body(m, c, b, d, seed_hi, dt, blockIdx.x, gridDim.x);
}

// Emission (source.h:84-97, 7 draws) and boundary-source (source.h:100-114,
// 6 draws) photons, stream = 1e13*cycle + ith photon, stored after the census.
__device__ __forceinline__ void source_new_body(const MeshDev &m, const CellsDev &c, const Bank &b,
                                                const DeviceDiag *d, unsigned long long seed_hi, uint32_t cycle,
                                                double dt, uint32_t bx, uint32_t nbx) {
  const unsigned long long n = d->n_new, base = d->n_census_in;
  const unsigned long long cycle_offset = 10000000000000ULL * (unsigned long long)cycle;
  for (unsigned long long p = bx * (unsigned long long)blockDim.x + threadIdx.x; p < n;
       p += (unsigned long long)nbx * blockDim.x) {
    const uint32_t g = find_cell(c.off_new, m.n_cells, p);
    const unsigned long long local = p - c.off_new[g];
    double nodes[6], pos[3], dir[3];
    cell_nodes(m, g, nodes);
    const unsigned long long stream = cycle_offset + p;
    Rng r{stream, 0ULL, seed_hi};
    double E;
    uint8_t stype;
    const uint32_t n_em = c.n_em[g];
    if (local < n_em) {
      position_in_cell(nodes, r, pos);
      uniform_angle(r, dir);
      E = c.em_E[g] / (double)n_em;
      stype = 2;
    } else {
      const int face = c.source_face[g];
      position_on_face(nodes, r, face, pos);
      source_angle(r, face, dir);
      E = c.so_E[g] / (double)c.n_so[g];
      stype = 1;
    }
    const double life = r.next() * kC * dt;
    const uint32_t group = sample_uniform_group(r, m.n_groups);
    store_photon(b, base + p, pos, dir, E, life, g, group, stype, stream, r.ctr);
  }
}

__global__ void k_source_new(MeshDev m, CellsDev c, Bank b, const DeviceDiag *d,
                             unsigned long long seed_hi, uint32_t cycle, double dt) {
  source_new_body(m, c, b, d, seed_hi, cycle, dt, blockIdx.x, gridDim.x);
}

void launch_plan_bank(const MeshDev &m, const CellsDev &c, DeviceDiag *d, uint32_t step,
                      unsigned long long capacity, cudaStream_t s) {
  k_plan_bank<<<1, 1, 0, s>>>(m, c, d, step, capacity);
}

void launch_source(const MeshDev &m, const CellsDev &c, const Bank &b, DeviceDiag *d, uint32_t seed,
                   uint32_t step, double dt, int n_sm, cudaStream_t s) {
  const unsigned long long seed_hi = (unsigned long long)seed << 32;
  if (step == 1) k_source_census<<<n_sm * 8, 256, 0, s>>>(m, c, b, d, seed_hi, dt);
  k_source_new<<<n_sm * 8, 256, 0, s>>>(m, c, b, d, seed_hi, step, dt);
}

// batched: problem blockIdx.y of the view table (plan, initial census at
// step 1, then this step's photons)
__global__ void k_b_plan_bank(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  if (threadIdx.x == 0) plan_bank_body(P.m, P.c, P.d, P.step, P.capacity);
}
__global__ void __launch_bounds__(256) k_b_source_census(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  if (P.step == 1) source_census_body(P.m, P.c, P.from, P.d, P.seed_hi, P.dt, blockIdx.x, gridDim.x);
}
__global__ void __launch_bounds__(256) k_b_source_new(const ProblemView *v) {
  const ProblemView &P = v[blockIdx.y];
  source_new_body(P.m, P.c, P.from, P.d, P.seed_hi, P.step, P.dt, blockIdx.x, gridDim.x);
}

void launch_batch_source(const ProblemView *v, const BatchGrid &g, cudaStream_t s) {
  k_b_plan_bank<<<dim3(1, g.n), 32, 0, s>>>(v);
  k_b_source_census<<<dim3(g.photons, g.n), 256, 0, s>>>(v);
  k_b_source_new<<<dim3(g.photons, g.n), 256, 0, s>>>(v);
}

}  // namespace bgs
