// CPU reference harness: drives the UNMODIFIED upstream Branson headers
// (compiled from their original location, never copied) through the
// replicated-mode time step and dumps every quantity the GPU path must
// reproduce.  Test infrastructure only: it generates golden vectors, pins
// the C restatement in oracle/branson_oracle.c, and serves as the CPU
// baseline where it can be built.  Nothing in the product links it.
//
// The step loop mirrors imc_replicated_driver (src/replicated_driver.h:33-122)
// with dumps inserted between its phases:
//   calculate_photon_energy (mesh.h:237)            -> cells_pre
//   make_initial_census_photons / make_photons       -> source list
//   replicated_transport (replicated_transport.h:33) -> end states, census
//   update_temperature (mesh.h:327)                  -> cells_post
//
// Usage: ref_harness <deck.xml> <out_dir> <n_steps> <n_threads> [--no-dump]
//                    [--comb <max_census_photons> <stream>]
// Output (little endian):
//   cells.bin                 per cell: nodes[6] (f64), region_ID (u32), pad
//   stepNNN_source.bin        photon records before transport
//   stepNNN_end.bin           photon records after transport (same order)
//   stepNNN_census.bin        census list returned by replicated_transport
//   stepNNN_cells.bin         per cell: op_a f emission_E census_E source_E
//                             abs_E track_E T_e_new T_r  (9 x f64)
//   stepNNN_scalars.txt       key value lines (conservation, counts, timing)
//   stepNNN_comb.bin          (--comb) the census after comb_photons
//                             (census_functions.h:48-93) with a fresh
//                             RNG(seed, stream); the step itself goes on
//                             with the uncombed census
// Photon record (104 B): stream u64, counter u64, cell u32, group u32,
//   source_type u32, descriptor u32, pos[3] dir[3] E E0 life_dx (9 x f64).

#include <chrono>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "config.h"

// upstream headers are not self-contained: keep the order main.cc uses
#include "constants.h"
#include "imc_parameters.h"
#include "imc_state.h"
#include "info.h"
#include "input.h"
#include "mesh.h"
#include "mpi_types.h"
#include "photon.h"
#include "census_functions.h"
#include "source.h"
#include "replicated_transport.h"

namespace {

struct PhotonRecord {
  uint64_t stream, counter;
  uint32_t cell, group, source_type, descriptor;
  double pos[3], dir[3], E, E0, life_dx;
};
static_assert(sizeof(PhotonRecord) == 104, "record layout");
static_assert(sizeof(RNG) == 32, "RNG is four 64-bit words");

PhotonRecord record_of(const Photon &p) {
  PhotonRecord r;
  uint64_t words[4];
  RNG rng = p.get_rng();
  std::memcpy(words, &rng, sizeof(words));
  r.stream = words[2];
  r.counter = words[0];
  r.cell = p.get_cell();
  r.group = p.get_group();
  r.source_type = const_cast<Photon &>(p).get_source_type();
  r.descriptor = static_cast<uint32_t>(p.get_descriptor());
  auto pos = p.get_position();
  auto dir = p.get_angle();
  for (int i = 0; i < 3; ++i) {
    r.pos[i] = pos[i];
    r.dir[i] = dir[i];
  }
  r.E = p.get_E();
  r.E0 = p.get_E0();
  r.life_dx = p.get_distance_remaining();
  return r;
}

void dump_photons(const std::string &path, const std::vector<Photon> &ps) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::perror(path.c_str());
    std::exit(2);
  }
  std::vector<PhotonRecord> recs;
  recs.reserve(ps.size());
  for (const auto &p : ps)
    recs.push_back(record_of(p));
  if (!recs.empty())
    std::fwrite(recs.data(), sizeof(PhotonRecord), recs.size(), f);
  std::fclose(f);
}

void dump_doubles(const std::string &path, const std::vector<double> &v) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::perror(path.c_str());
    std::exit(2);
  }
  if (!v.empty())
    std::fwrite(v.data(), sizeof(double), v.size(), f);
  std::fclose(f);
}

std::string step_name(const std::string &dir, uint32_t step, const char *what) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "/step%03u_%s", step, what);
  return dir + buf;
}

} // namespace

int main(int argc, char **argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s deck.xml out_dir n_steps n_threads [--no-dump]\n", argv[0]);
    return 1;
  }
  const std::string deck = argv[1];
  const std::string out = argv[2];
  const int n_steps = std::atoi(argv[3]);
  const int n_threads = std::atoi(argv[4]);
  bool dump = true;
  int64_t comb_max = 0;
  uint64_t comb_stream = 0;
  for (int a = 5; a < argc; ++a) {
    const std::string opt = argv[a];
    if (opt == "--no-dump") {
      dump = false;
    } else if (opt == "--comb" && a + 2 < argc) {
      comb_max = std::atoll(argv[a + 1]);
      comb_stream = std::strtoull(argv[a + 2], nullptr, 10);
      a += 2;
    }
  }

  MPI_Init(&argc, &argv);
  const Info mpi_info;
  MPI_Types mpi_types;
  Input input(deck, mpi_types);
  IMC_Parameters imc_p(input);
  IMC_State imc_state(input, mpi_info.get_rank());
  Mesh mesh(input, mpi_types, mpi_info, imc_p);
  mesh.initialize_physical_properties(input);
#ifdef USE_OPENMP
  omp_set_num_threads(n_threads);
#endif

  const uint32_t n_cells = mesh.get_n_local_cells();
  if (dump) {
    FILE *f = std::fopen((out + "/cells.bin").c_str(), "wb");
    if (!f) {
      std::perror("cells.bin");
      return 2;
    }
    for (const auto &cell : mesh.get_cells()) {
      std::fwrite(cell.get_node_array(), sizeof(double), 6, f);
      uint32_t rid[2] = {cell.get_region_ID(), 0};
      std::fwrite(rid, sizeof(uint32_t), 2, f);
    }
    std::fclose(f);
  }

  std::vector<double> abs_E(mesh.get_n_global_cells(), 0.0);
  std::vector<double> track_E(mesh.get_n_global_cells(), 0.0);
  std::vector<Photon> census_photons;
  const uint64_t n_user = imc_p.get_n_user_photons();
  const uint32_t seed = imc_p.get_rng_seed();
  double total_transport_s = 0.0;
  uint64_t total_histories = 0;

  for (int s = 0; s < n_steps && !imc_state.finished(); ++s) {
    const uint32_t step = imc_state.get_step();
    mesh.calculate_photon_energy(imc_state, n_user);
    double global_source_energy = mesh.get_total_photon_E();
    imc_state.set_pre_census_E(get_photon_list_E(census_photons));
    GPU_Setup gpu_setup(0, 1, false, mesh.get_cells());
    if (step == 1)
      census_photons = make_initial_census_photons<std::vector<Photon>>(
          imc_state.get_dt(), mesh, 0, seed, n_user, global_source_energy);
    imc_state.set_pre_census_E(get_photon_list_E(census_photons));
    auto all_photons = make_photons<std::vector<Photon>>(imc_state.get_dt(), mesh, 0, step, seed,
                                                         n_user, global_source_energy);
    join_photon_arrays(all_photons, census_photons);
    imc_state.set_transported_particles(all_photons.size());
    if (dump)
      dump_photons(step_name(out, step, "source.bin"), all_photons);

    std::vector<double> pre(5 * (size_t)n_cells);
    {
      auto em = mesh.get_emission_E();
      auto ce = mesh.get_census_E();
      auto so = mesh.get_source_E();
      for (uint32_t i = 0; i < n_cells; ++i) {
        const Cell &c = mesh.get_cells()[i];
        pre[5 * i + 0] = c.get_op_a(0u);
        pre[5 * i + 1] = c.get_f();
        pre[5 * i + 2] = em[i];
        pre[5 * i + 3] = ce[i];
        pre[5 * i + 4] = so[i];
      }
    }

    auto t0 = std::chrono::high_resolution_clock::now();
    census_photons = replicated_transport<std::vector<Photon>>(
        mesh, gpu_setup, imc_state, abs_E, track_E, all_photons, n_threads,
        imc_p.get_batch_size(), imc_p.get_transport_algorithm());
    auto t1 = std::chrono::high_resolution_clock::now();
    const double transport_s = std::chrono::duration<double>(t1 - t0).count();
    total_transport_s += transport_s;
    total_histories += all_photons.size();

    if (dump) {
      dump_photons(step_name(out, step, "end.bin"), all_photons);
      dump_photons(step_name(out, step, "census.bin"), census_photons);
    }
    uint64_t comb_draws = 0;
    if (dump && comb_max > 0) {
      std::vector<Photon> combed = census_photons;
      RNG comb_rng(seed, comb_stream);
      comb_photons(combed, comb_max, &comb_rng);
      uint64_t words[4];
      std::memcpy(words, &comb_rng, sizeof(words));
      comb_draws = words[0];
      dump_photons(step_name(out, step, "comb.bin"), combed);
    }
    std::vector<double> tallies_abs(abs_E.begin(), abs_E.begin() + n_cells);
    std::vector<double> tallies_track(track_E.begin(), track_E.begin() + n_cells);

    mesh.update_temperature(abs_E, track_E, imc_state);

    if (dump) {
      std::vector<double> cells(9 * (size_t)n_cells);
      for (uint32_t i = 0; i < n_cells; ++i) {
        cells[9 * i + 0] = pre[5 * i + 0];
        cells[9 * i + 1] = pre[5 * i + 1];
        cells[9 * i + 2] = pre[5 * i + 2];
        cells[9 * i + 3] = pre[5 * i + 3];
        cells[9 * i + 4] = pre[5 * i + 4];
        cells[9 * i + 5] = tallies_abs[i];
        cells[9 * i + 6] = tallies_track[i];
        cells[9 * i + 7] = mesh.get_cells()[i].get_T_e();
        cells[9 * i + 8] = mesh.get_T_r(i);
      }
      dump_doubles(step_name(out, step, "cells.bin"), cells);
    }

    // conservation scalars exactly as print_conservation forms them
    // (imc_state.h:254-258); one rank so every reduction is the identity
    FILE *f = dump ? std::fopen(step_name(out, step, "scalars.txt").c_str(), "w") : stdout;
    std::fprintf(f, "step %u\n", step);
    std::fprintf(f, "dt %.17g\n", imc_state.get_dt());
    std::fprintf(f, "next_dt %.17g\n", imc_state.get_next_dt());
    std::fprintf(f, "total_photon_E %.17g\n", global_source_energy);
    std::fprintf(f, "emission_E %.17g\n", imc_state.get_emission_E());
    std::fprintf(f, "pre_census_E %.17g\n", imc_state.get_pre_census_E());
    std::fprintf(f, "n_transported %llu\n", (unsigned long long)all_photons.size());
    std::fprintf(f, "census_size %llu\n", (unsigned long long)census_photons.size());
    std::fprintf(f, "post_census_E %.17g\n", get_photon_list_E(census_photons));
    std::fprintf(f, "transport_s %.9g\n", transport_s);
    if (comb_max > 0) {
      std::fprintf(f, "comb_max %lld\n", (long long)comb_max);
      std::fprintf(f, "comb_stream %llu\n", (unsigned long long)comb_stream);
      std::fprintf(f, "comb_draws %llu\n", (unsigned long long)comb_draws);
    }
    if (dump)
      std::fclose(f);
    imc_state.print_conservation(imc_p.get_dd_mode());
    imc_state.next_time_step();
  }
  std::printf("HARNESS histories %llu transport_s %.6f histories_per_s %.6g threads %d\n",
              (unsigned long long)total_histories, total_transport_s,
              total_transport_s > 0 ? total_histories / total_transport_s : 0.0, n_threads);
  MPI_Finalize();
  return 0;
}
