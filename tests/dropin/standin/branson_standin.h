// Stand-ins for the upstream Branson types that the C++ drop-in
// (include/branson_gb300_transport.hpp) reads and writes, so that the
// drop-in's conversions and side effects run on a host without the upstream
// checkout (the GPU host).  TEST INFRASTRUCTURE ONLY.
//
// Each type keeps only the members the drop-in calls, with the upstream
// member names, argument types and meaning (the file:line of each upstream
// member is given); the bodies are plain storage written here.  The drop-in
// itself is compiled against the real upstream headers by
// tests/test_dropin_shim.py; this header lets the same template code run.
#ifndef BRANSON_STANDIN_H
#define BRANSON_STANDIN_H

#include <array>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <vector>

#ifndef BRANSON_N_GROUPS
#define BRANSON_N_GROUPS 1  // config.h.in
#endif

// Insist (config.h.in:86-91): abort with a message
inline void Insist(bool cond, const std::string &msg) {
  if (!cond) {
    std::fprintf(stderr, "Insist failed: %s\n", msg.c_str());
    std::exit(3);
  }
}

// the single-rank barrier of the drop-in's transport timer
typedef int MPI_Comm;
constexpr MPI_Comm MPI_COMM_WORLD = 0;
inline int MPI_Barrier(MPI_Comm) { return 0; }

namespace Constants {
enum bc_type { REFLECT, VACUUM, ELEMENT, SOURCE, PROCESSOR };                   // constants.h:26
enum event_type : unsigned char { EXIT, PASS, CENSUS, SCATTER, KILLED, BOUND };  // constants.h:28
enum { HISTORY, EVENT };                                                         // constants.h:34
}  // namespace Constants

// RNG (RNG.h:306-340): four 64-bit words, counter {lo, seed << 32} and key
// {stream, 0}; the drop-in reads and writes them as raw words
class RNG {
 public:
  RNG() {}

 private:
  uint64_t words_[4] = {0, 0, 0, 0};
};

// Photon (photon.h:33-183)
class Photon {
 public:
  std::array<double, 3> get_position() const { return pos_; }       // photon.h:64
  std::array<double, 3> get_angle() const { return angle_; }        // photon.h:68
  double get_E() const { return E_; }                               // photon.h:72
  double get_E0() const { return E0_; }                             // photon.h:76
  double get_distance_remaining() const { return life_; }           // photon.h:80
  uint32_t get_cell() const { return cell_; }                       // photon.h:56
  uint32_t get_group() const { return group_; }                     // photon.h:60
  uint32_t get_source_type() const { return source_type_; }         // photon.h:116
  Constants::event_type get_descriptor() const { return desc_; }    // photon.h:101
  RNG get_rng() const { return rng_; }                              // photon.h:161
  void set_position(const std::array<double, 3> &p) { pos_ = p; }   // photon.h:147
  void set_angle(const std::array<double, 3> &a) { angle_ = a; }    // photon.h:143
  void set_E0(const double E) { E0_ = E; E_ = E; }                  // photon.h:128-131 (sets both)
  void set_E(const double E) { E_ = E; }                            // photon.h:135
  void set_distance_to_census(const double d) { life_ = d; }        // photon.h:139
  void set_cell(const uint32_t c) { cell_ = c; }                    // photon.h:121
  void set_group(const uint32_t g) { group_ = g; }                  // photon.h:125
  void set_source_type(uint32_t t) { source_type_ = t; }            // photon.h:117
  void set_descriptor(const Constants::event_type d) { desc_ = d; } // photon.h:158
  void set_rng(const RNG &r) { rng_ = r; }                          // photon.h:166

 private:
  std::array<double, 3> pos_{}, angle_{};
  double E_ = 0, E0_ = 0, life_ = 0;
  uint32_t cell_ = 0, group_ = 0, source_type_ = 0;
  Constants::event_type desc_ = Constants::PASS;
  RNG rng_;
};

// PhotonArray (photon_array.h:25-135): structure of arrays
struct PhotonArray {
  std::vector<uint32_t> cell_ID, group, source_type;
  std::vector<unsigned char> descriptors;
  std::vector<std::array<double, 3>> pos, angle;
  std::vector<double> E, E0, life_dx;
  std::vector<RNG> rng;
  size_t size() const { return E.size(); }
  void resize(size_t n) {
    cell_ID.resize(n); group.resize(n); source_type.resize(n); descriptors.resize(n);
    pos.resize(n); angle.resize(n); E.resize(n); E0.resize(n); life_dx.resize(n); rng.resize(n);
  }
};

// Cell (cell.h): nodes {x_lo, x_hi, y_lo, y_hi, z_lo, z_hi}, per-face boundary
// codes, opacities and the Fleck factor
class Cell {
 public:
  Cell(const std::array<double, 6> &nodes, const std::array<Constants::bc_type, 6> &bc)
      : nodes_(nodes), bc_(bc) {}
  const double *get_node_array() const { return nodes_.data(); }                 // cell.h:154
  Constants::bc_type get_bc(const uint32_t &dir) const { return bc_[dir]; }      // cell.h:104
  double get_op_a(uint32_t) const { return op_a_; }                              // cell.h:168
  double get_op_s(uint32_t) const { return op_s_; }                              // cell.h:176
  double get_f() const { return f_; }
  void set_coefficients(double op_a, double op_s, double f) { op_a_ = op_a; op_s_ = op_s; f_ = f; }

 private:
  std::array<double, 6> nodes_;
  std::array<Constants::bc_type, 6> bc_;
  double op_a_ = 0, op_s_ = 0, f_ = 0;
};

// Mesh (mesh.h): the replicated structured mesh, cell g = i + ngx*(j + ngy*k)
class Mesh {
 public:
  Mesh(const std::vector<double> &x, const std::vector<double> &y, const std::vector<double> &z,
       const std::array<Constants::bc_type, 6> &bc)
      : nx_((uint32_t)x.size() - 1), ny_((uint32_t)y.size() - 1), nz_((uint32_t)z.size() - 1) {
    for (uint32_t k = 0; k < nz_; ++k)
      for (uint32_t j = 0; j < ny_; ++j)
        for (uint32_t i = 0; i < nx_; ++i) {
          std::array<Constants::bc_type, 6> b;
          const bool inside[6] = {i > 0, i + 1 < nx_, j > 0, j + 1 < ny_, k > 0, k + 1 < nz_};
          for (int f = 0; f < 6; ++f) b[f] = inside[f] ? Constants::ELEMENT : bc[f];
          cells_.emplace_back(std::array<double, 6>{x[i], x[i + 1], y[j], y[j + 1], z[k], z[k + 1]}, b);
        }
  }
  uint32_t get_global_n_x_faces() const { return nx_ + 1; }  // mesh.h:223
  uint32_t get_global_n_y_faces() const { return ny_ + 1; }
  uint32_t get_global_n_z_faces() const { return nz_ + 1; }
  const std::vector<Cell> &get_cells() const { return cells_; }  // mesh.h:212
  std::vector<Cell> &cells() { return cells_; }

 private:
  uint32_t nx_, ny_, nz_;
  std::vector<Cell> cells_;
};

// IMC_State (imc_state.h): the next time step in, the step's results out
class IMC_State {
 public:
  explicit IMC_State(double next_dt) : next_dt_(next_dt) {}
  double get_next_dt() const { return next_dt_; }                                       // imc_state.h:112
  void set_exit_E(double e) { exit_E = e; }                                             // imc_state.h:322
  void set_post_census_E(double e) { post_census_E = e; }                               // imc_state.h:302
  void set_census_size(uint64_t n) { census_size = n; }                                 // imc_state.h:330
  void set_rank_transport_runtime(double t) { rank_transport_runtime = t; }             // imc_state.h:350
  double exit_E = -1, post_census_E = -1, rank_transport_runtime = -1;
  uint64_t census_size = ~0ULL;

 private:
  double next_dt_;
};

struct GPU_Setup {};

// Timer (timer.h:26-51): named wall-clock intervals
class Timer {
 public:
  void start_timer(std::string name) { start_[name] = std::chrono::steady_clock::now(); }
  void stop_timer(std::string name) {
    times_[name] += std::chrono::duration<double>(std::chrono::steady_clock::now() - start_[name]).count();
  }
  double get_time(std::string name) { return times_[name]; }

 private:
  std::map<std::string, std::chrono::steady_clock::time_point> start_;
  std::map<std::string, double> times_;
};

#endif
