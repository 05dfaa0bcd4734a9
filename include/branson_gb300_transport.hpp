// Drop-in replacement for Branson's replicated_transport<Census_T>
// (src/replicated_transport.h:33-158), running the transport on a GB300
// through the C ABI in branson_gb300.h.
//
// Use: in the Branson tree, include this header instead of
// "replicated_transport.h" (the include at src/replicated_driver.h:28), or
// define BRANSON_GB300_TRANSPORT and include it after the upstream headers;
// link against libbranson_gb300.so.  imc_replicated_driver is unchanged: it
// calls (src/replicated_driver.h:87-88)
//
//   census = replicated_transport<Census_T>(mesh, gpu_setup, imc_state,
//                abs_E, track_E, all_photons, n_omp_threads, batch_size,
//                transport_algorithm);
//
// exactly as before, with the upstream semantics:
//   * all_photons is updated in place with the end states (descriptor,
//     position, direction, energy, cell, group, RNG counter);
//   * the returned census holds the CENSUS photons in input order with
//     life_dx = c * next_dt (post_process_photons,
//     post_process_functions.h:33-109);
//   * rank_abs_E / rank_track_E are overwritten with this step's tallies
//     (replicated_transport.h:135-140);
//   * IMC_State receives exit_E, post_census_E, census_size and the
//     transport time (replicated_transport.h:151-155).
// Errors abort through Insist (config.h.in:86-91), as upstream.
//
// One device context per process (the replicated mesh is uploaded on the
// first call; opacities and Fleck factors are uploaded every call).  The
// photon banks are sized for twice the first call's list; a later, longer
// list (census growth over steps) replaces the context with one twice its
// length.  Only group 0's absorption and scattering opacities are uploaded:
// the upstream cells set every group to the same value (Cell::set_op_a /
// set_op_s, cell.h:260-275), and the device tables keep one opacity per cell
// with the group drawn uniformly.  The header needs the upstream types (Mesh,
// Cell, Photon, PhotonArray, RNG, IMC_State, GPU_Setup, Timer) to be
// declared before it is included.
#ifndef BRANSON_GB300_TRANSPORT_HPP
#define BRANSON_GB300_TRANSPORT_HPP

#include <cstdint>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "branson_gb300.h"

namespace branson_gb300 {

struct HostSoA {
  std::vector<double> px, py, pz, dx, dy, dz, E, E0, life;
  std::vector<uint32_t> cell, group;
  std::vector<uint8_t> desc, stype;
  std::vector<uint64_t> stream, ctr;
  void resize(size_t n) {
    for (auto *v : {&px, &py, &pz, &dx, &dy, &dz, &E, &E0, &life}) v->resize(n);
    cell.resize(n); group.resize(n); desc.resize(n); stype.resize(n);
    stream.resize(n); ctr.resize(n);
  }
  bgs_photons_host view() {
    return bgs_photons_host{px.data(), py.data(), pz.data(), dx.data(), dy.data(), dz.data(),
                            E.data(), E0.data(), life.data(), cell.data(), group.data(),
                            desc.data(), stype.data(), stream.data(), ctr.data()};
  }
};

// RNG is four 64-bit words {counter lo, seed << 32, stream, 0} (RNG.h:318-330)
inline void rng_words(const RNG &r, uint64_t w[4]) { std::memcpy(w, &r, 4 * sizeof(uint64_t)); }
inline RNG rng_from(uint64_t seed_hi, uint64_t stream, uint64_t counter) {
  RNG r;
  const uint64_t w[4] = {counter, seed_hi, stream, 0};
  std::memcpy(&r, w, sizeof w);
  return r;
}

struct Context {
  bgs_context *ctx = nullptr;
  uint64_t seed_hi = 0;
  uint64_t capacity = 0;  // photons per device bank
  uint32_t n_cells = 0;
  std::vector<double> x, y, z;
  std::vector<double> op_a, op_s, f;
  HostSoA in, census;
  ~Context() { bgs_destroy(ctx); }
};

inline void check(bgs_context *ctx, int rc, const char *what) {
  if (rc != BGS_OK)
    Insist(false, std::string(what) + ": " + bgs_status_string(rc) + " (" +
                      (ctx ? bgs_last_error(ctx) : "") + ")");
}

// Planes and boundary codes of the structured replicated mesh, read back
// from the upstream cells (cell g = i + ngx*j + ngx*ngy*k, proto_mesh.h).
inline void upload_mesh(Context &C, const Mesh &mesh) {
  const uint32_t ngx = mesh.get_global_n_x_faces() - 1, ngy = mesh.get_global_n_y_faces() - 1,
                 ngz = mesh.get_global_n_z_faces() - 1;
  const auto &cells = mesh.get_cells();
  C.x.resize(ngx + 1); C.y.resize(ngy + 1); C.z.resize(ngz + 1);
  for (uint32_t i = 0; i < ngx; ++i) C.x[i] = cells[i].get_node_array()[0];
  C.x[ngx] = cells[ngx - 1].get_node_array()[1];
  for (uint32_t j = 0; j < ngy; ++j) C.y[j] = cells[j * ngx].get_node_array()[2];
  C.y[ngy] = cells[(ngy - 1) * ngx].get_node_array()[3];
  for (uint32_t k = 0; k < ngz; ++k) C.z[k] = cells[k * ngx * ngy].get_node_array()[4];
  C.z[ngz] = cells[(ngz - 1) * ngx * ngy].get_node_array()[5];
  bgs_mesh_desc d{};
  d.ngx = ngx; d.ngy = ngy; d.ngz = ngz; d.n_groups = BRANSON_N_GROUPS;
  d.x_planes = C.x.data(); d.y_planes = C.y.data(); d.z_planes = C.z.data();
  std::vector<uint32_t> region(cells.size(), 0);
  const double row[8] = {1, 1, 0, 0, 0, 0, 0, 0};  // transport reads no region data
  d.cell_region = region.data(); d.n_regions = 1; d.regions = row;
  const uint32_t last = (uint32_t)cells.size() - 1;
  const uint32_t face_cell[6] = {0, ngx - 1, 0, (ngy - 1) * ngx, 0, last};
  for (int face = 0; face < 6; ++face) d.bc[face] = (int32_t)cells[face_cell[face]].get_bc(face);
  d.T_source = 0.0;
  check(C.ctx, bgs_set_mesh(C.ctx, &d), "bgs_set_mesh");
  C.n_cells = (uint32_t)cells.size();
}

inline Context &context(const Mesh &mesh, size_t n_photons, uint64_t seed_hi) {
  static Context C;
  if (C.ctx && (uint64_t)n_photons > C.capacity) {  // a longer list than the banks hold: a new context
    check(C.ctx, bgs_destroy(C.ctx), "bgs_destroy");
    C.ctx = nullptr;
  }
  if (!C.ctx) {
    const uint64_t cap = 2 * (uint64_t)n_photons + 4096;
    check(nullptr, bgs_create(&C.ctx, 0, cap, nullptr, (uint32_t)(seed_hi >> 32), 0), "bgs_create");
    upload_mesh(C, mesh);
    C.seed_hi = seed_hi;
    C.capacity = cap;
  }
  return C;
}

template <typename Census_T> struct Access;

template <> struct Access<std::vector<Photon>> {
  static size_t size(const std::vector<Photon> &p) { return p.size(); }
  static uint64_t seed_hi(const std::vector<Photon> &p) {
    uint64_t w[4] = {0, 0, 0, 0};
    if (!p.empty()) rng_words(p[0].get_rng(), w);
    return w[1];
  }
  static void to_soa(const std::vector<Photon> &p, HostSoA &s) {
    s.resize(p.size());
    for (size_t i = 0; i < p.size(); ++i) {
      const Photon &q = p[i];
      const auto pos = q.get_position(), dir = q.get_angle();
      s.px[i] = pos[0]; s.py[i] = pos[1]; s.pz[i] = pos[2];
      s.dx[i] = dir[0]; s.dy[i] = dir[1]; s.dz[i] = dir[2];
      s.E[i] = q.get_E(); s.E0[i] = q.get_E0(); s.life[i] = q.get_distance_remaining();
      s.cell[i] = q.get_cell(); s.group[i] = q.get_group();
      s.desc[i] = (uint8_t)Constants::PASS; s.stype[i] = (uint8_t)const_cast<Photon &>(q).get_source_type();
      uint64_t w[4];
      rng_words(q.get_rng(), w);
      s.stream[i] = w[2]; s.ctr[i] = w[0];
    }
  }
  static void from_soa(const HostSoA &s, size_t n, uint64_t seed_hi, std::vector<Photon> &p) {
    p.resize(n);
    for (size_t i = 0; i < n; ++i) {
      Photon &q = p[i];
      q.set_position({s.px[i], s.py[i], s.pz[i]});
      q.set_angle({s.dx[i], s.dy[i], s.dz[i]});
      q.set_E0(s.E0[i]);
      q.set_E(s.E[i]);
      q.set_distance_to_census(s.life[i]);
      q.set_cell(s.cell[i]); q.set_group(s.group[i]);
      q.set_source_type(s.stype[i]);
      q.set_descriptor(static_cast<Constants::event_type>(s.desc[i]));
      q.set_rng(rng_from(seed_hi, s.stream[i], s.ctr[i]));
    }
  }
};

template <> struct Access<PhotonArray> {
  static size_t size(const PhotonArray &p) { return p.size(); }
  static uint64_t seed_hi(const PhotonArray &p) {
    uint64_t w[4] = {0, 0, 0, 0};
    if (p.size()) rng_words(p.rng[0], w);
    return w[1];
  }
  static void to_soa(const PhotonArray &p, HostSoA &s) {
    const size_t n = p.size();
    s.resize(n);
    for (size_t i = 0; i < n; ++i) {
      s.px[i] = p.pos[i][0]; s.py[i] = p.pos[i][1]; s.pz[i] = p.pos[i][2];
      s.dx[i] = p.angle[i][0]; s.dy[i] = p.angle[i][1]; s.dz[i] = p.angle[i][2];
      s.E[i] = p.E[i]; s.E0[i] = p.E0[i]; s.life[i] = p.life_dx[i];
      s.cell[i] = p.cell_ID[i]; s.group[i] = p.group[i];
      s.desc[i] = p.descriptors[i]; s.stype[i] = (uint8_t)p.source_type[i];
      uint64_t w[4];
      rng_words(p.rng[i], w);
      s.stream[i] = w[2]; s.ctr[i] = w[0];
    }
  }
  static void from_soa(const HostSoA &s, size_t n, uint64_t seed_hi, PhotonArray &p) {
    p.resize(n);
    for (size_t i = 0; i < n; ++i) {
      p.pos[i] = {s.px[i], s.py[i], s.pz[i]};
      p.angle[i] = {s.dx[i], s.dy[i], s.dz[i]};
      p.E[i] = s.E[i]; p.E0[i] = s.E0[i]; p.life_dx[i] = s.life[i];
      p.cell_ID[i] = s.cell[i]; p.group[i] = s.group[i];
      p.descriptors[i] = s.desc[i]; p.source_type[i] = s.stype[i];
      p.rng[i] = rng_from(seed_hi, s.stream[i], s.ctr[i]);
    }
  }
};

}  // namespace branson_gb300

template <typename Census_T>
Census_T replicated_transport(const Mesh &mesh, const GPU_Setup &gpu_setup, IMC_State &imc_state,
                              std::vector<double> &rank_abs_E, std::vector<double> &rank_track_E,
                              Census_T &all_photons, const int n_omp_threads, const uint32_t batch_size,
                              const int transport_algorithm) {
  using namespace branson_gb300;
  (void)gpu_setup;
  (void)n_omp_threads;
  (void)batch_size;  // the whole list is one device batch
  Timer t_transport;
  t_transport.start_timer("timestep transport");
  const size_t n = Access<Census_T>::size(all_photons);
  const uint64_t seed_hi = Access<Census_T>::seed_hi(all_photons);
  Context &C = context(mesh, n, seed_hi);
  // this step's opacities and Fleck factors (Mesh::calculate_photon_energy)
  const auto &cells = mesh.get_cells();
  C.op_a.resize(cells.size()); C.op_s.resize(cells.size()); C.f.resize(cells.size());
  for (size_t i = 0; i < cells.size(); ++i) {
    C.op_a[i] = cells[i].get_op_a(0u);
    C.op_s[i] = cells[i].get_op_s(0u);
    C.f[i] = cells[i].get_f();
  }
  check(C.ctx, bgs_set_cell_field(C.ctx, BGS_FIELD_OP_A, C.op_a.data()), "op_a");
  check(C.ctx, bgs_set_cell_field(C.ctx, BGS_FIELD_OP_S, C.op_s.data()), "op_s");
  check(C.ctx, bgs_set_cell_field(C.ctx, BGS_FIELD_F, C.f.data()), "f");
  Access<Census_T>::to_soa(all_photons, C.in);
  C.census.resize(n);
  bgs_photons_host in = C.in.view(), cen = C.census.view();
  uint64_t n_census = 0;
  double census_E = 0.0, exit_E = 0.0;
  const uint32_t algo = transport_algorithm == Constants::EVENT ? BGS_EVENT : BGS_HISTORY;
  check(C.ctx, bgs_replicated_transport(C.ctx, n, &in, imc_state.get_next_dt(), algo, rank_abs_E.data(),
                                        rank_track_E.data(), &cen, n, &n_census, &census_E, &exit_E),
        "bgs_replicated_transport");
  Access<Census_T>::from_soa(C.in, n, seed_hi, all_photons);
  Census_T census_list;
  Access<Census_T>::from_soa(C.census, (size_t)n_census, seed_hi, census_list);
  t_transport.stop_timer("timestep transport");
  MPI_Barrier(MPI_COMM_WORLD);
  imc_state.set_exit_E(exit_E);
  imc_state.set_post_census_E(census_E);
  imc_state.set_census_size(census_list.size());
  imc_state.set_rank_transport_runtime(t_transport.get_time("timestep transport"));
  return census_list;
}

#endif  // BRANSON_GB300_TRANSPORT_HPP
