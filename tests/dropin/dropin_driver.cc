// Compile/link check of include/branson_gb300_transport.hpp inside the
// upstream code base: the upstream headers (unmodified, from the reference
// checkout) with the drop-in replicated_transport in place of
// src/replicated_transport.h, driven by the replicated step loop.
#include <iostream>
#include <string>
#include <vector>

#include "config.h"
#include "constants.h"
#include "imc_parameters.h"
#include "imc_state.h"
#include "info.h"
#include "input.h"
#include "mesh.h"
#include "mpi_types.h"
#include "photon.h"
#include "photon_array.h"
#include "census_functions.h"
#include "source.h"
#include "gpu_setup.h"
#include "timer.h"

#include "branson_gb300_transport.hpp"

template <typename Census_T>
void step_loop(Mesh &mesh, IMC_State &imc_state, const IMC_Parameters &p) {
  std::vector<double> abs_E(mesh.get_n_global_cells(), 0.0), track_E(mesh.get_n_global_cells(), 0.0);
  Census_T census;
  while (!imc_state.finished()) {
    mesh.calculate_photon_energy(imc_state, p.get_n_user_photons());
    const double total = mesh.get_total_photon_E();
    GPU_Setup gpu_setup(0, 1, false, mesh.get_cells());
    if (imc_state.get_step() == 1)
      census = make_initial_census_photons<Census_T>(imc_state.get_dt(), mesh, 0, p.get_rng_seed(),
                                                     p.get_n_user_photons(), total);
    auto all = make_photons<Census_T>(imc_state.get_dt(), mesh, 0, imc_state.get_step(), p.get_rng_seed(),
                                      p.get_n_user_photons(), total);
    join_photon_arrays(all, census);
    census = replicated_transport<Census_T>(mesh, gpu_setup, imc_state, abs_E, track_E, all,
                                            p.get_n_omp_threads(), p.get_batch_size(),
                                            p.get_transport_algorithm());
    mesh.update_temperature(abs_E, track_E, imc_state);
    imc_state.print_conservation(p.get_dd_mode());
    imc_state.next_time_step();
  }
}

int main(int argc, char **argv) {
  MPI_Init(&argc, &argv);
  if (argc < 2) return 1;
  const Info info;
  MPI_Types types;
  Input input(argv[1], types);
  IMC_Parameters p(input);
  IMC_State state(input, 0);
  Mesh mesh(input, types, info, p);
  mesh.initialize_physical_properties(input);
  if (input.get_particle_storage() == Constants::SOA)
    step_loop<PhotonArray>(mesh, state, p);
  else
    step_loop<std::vector<Photon>>(mesh, state, p);
  MPI_Finalize();
  return 0;
}
