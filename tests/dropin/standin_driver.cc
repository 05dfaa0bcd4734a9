// Runs the C++ drop-in replicated_transport<Census_T>
// (include/branson_gb300_transport.hpp) on the GPU over a sequence of calls
// prepared by tests/test_dropin_run_gpu.py, with the stand-in upstream types
// of tests/dropin/standin/branson_standin.h.  TEST INFRASTRUCTURE ONLY.
//
// Usage: standin_driver <dir> <aos|soa>
// <dir>/mesh.bin      u32 ngx ngy ngz, i32 bc[6], u32 seed, then the x, y, z
//                     planes (f64)
// <dir>/calls.txt     one line per call: n_photons next_dt
// <dir>/callK_cells.bin  op_a, op_s, f (n_cells f64 each)
// <dir>/callK_in.bin  photon records (104 B: stream u64, counter u64, cell,
//                     group, source_type, descriptor u32, pos[3] dir[3] E E0
//                     life_dx f64)
// Writes per call, with the suffix _aos or _soa:
//   callK_end.bin (the list after the call, records), callK_census.bin (the
//   returned census, records), callK_tally.bin (abs_E then track_E), and
//   callK_state.txt (exit_E post_census_E census_size transport_runtime).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "branson_standin.h"
#include "branson_gb300_transport.hpp"

namespace {

struct Record {
  uint64_t stream, counter;
  uint32_t cell, group, source_type, descriptor;
  double pos[3], dir[3], E, E0, life_dx;
};
static_assert(sizeof(Record) == 104, "record layout");

std::vector<char> slurp(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  Insist(bool(f), "cannot read " + path);
  return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

void spill(const std::string &path, const void *p, size_t bytes) {
  std::FILE *f = std::fopen(path.c_str(), "wb");
  Insist(f != nullptr, "cannot write " + path);
  if (bytes) std::fwrite(p, 1, bytes, f);
  std::fclose(f);
}

RNG make_rng(uint64_t seed_hi, uint64_t stream, uint64_t counter) {
  return branson_gb300::rng_from(seed_hi, stream, counter);
}

void rng_parts(const RNG &r, uint64_t &stream, uint64_t &counter) {
  uint64_t w[4];
  branson_gb300::rng_words(r, w);
  stream = w[2];
  counter = w[0];
}

void load(const std::vector<Record> &in, uint64_t seed_hi, std::vector<Photon> &out) {
  out.resize(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    const Record &r = in[i];
    Photon &p = out[i];
    p.set_position({r.pos[0], r.pos[1], r.pos[2]});
    p.set_angle({r.dir[0], r.dir[1], r.dir[2]});
    p.set_E0(r.E0);
    p.set_E(r.E);
    p.set_distance_to_census(r.life_dx);
    p.set_cell(r.cell);
    p.set_group(r.group);
    p.set_source_type(r.source_type);
    p.set_descriptor(static_cast<Constants::event_type>(r.descriptor));
    p.set_rng(make_rng(seed_hi, r.stream, r.counter));
  }
}

void load(const std::vector<Record> &in, uint64_t seed_hi, PhotonArray &out) {
  out.resize(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    const Record &r = in[i];
    out.pos[i] = {r.pos[0], r.pos[1], r.pos[2]};
    out.angle[i] = {r.dir[0], r.dir[1], r.dir[2]};
    out.E[i] = r.E;
    out.E0[i] = r.E0;
    out.life_dx[i] = r.life_dx;
    out.cell_ID[i] = r.cell;
    out.group[i] = r.group;
    out.source_type[i] = r.source_type;
    out.descriptors[i] = (unsigned char)r.descriptor;
    out.rng[i] = make_rng(seed_hi, r.stream, r.counter);
  }
}

std::vector<Record> store(const std::vector<Photon> &in) {
  std::vector<Record> out(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    const Photon &p = in[i];
    Record &r = out[i];
    const auto pos = p.get_position(), dir = p.get_angle();
    for (int a = 0; a < 3; ++a) { r.pos[a] = pos[a]; r.dir[a] = dir[a]; }
    r.E = p.get_E(); r.E0 = p.get_E0(); r.life_dx = p.get_distance_remaining();
    r.cell = p.get_cell(); r.group = p.get_group(); r.source_type = p.get_source_type();
    r.descriptor = p.get_descriptor();
    rng_parts(p.get_rng(), r.stream, r.counter);
  }
  return out;
}

std::vector<Record> store(const PhotonArray &in) {
  std::vector<Record> out(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    Record &r = out[i];
    for (int a = 0; a < 3; ++a) { r.pos[a] = in.pos[i][a]; r.dir[a] = in.angle[i][a]; }
    r.E = in.E[i]; r.E0 = in.E0[i]; r.life_dx = in.life_dx[i];
    r.cell = in.cell_ID[i]; r.group = in.group[i]; r.source_type = in.source_type[i];
    r.descriptor = in.descriptors[i];
    rng_parts(in.rng[i], r.stream, r.counter);
  }
  return out;
}

template <typename Census_T>
void run(const std::string &dir, const std::string &tag, Mesh &mesh, uint64_t seed_hi) {
  std::ifstream calls(dir + "/calls.txt");
  Insist(bool(calls), "no calls.txt");
  size_t n;
  double next_dt;
  const size_t n_cells = mesh.get_cells().size();
  for (int k = 0; calls >> n >> next_dt; ++k) {
    const std::string base = dir + "/call" + std::to_string(k);
    const auto cells = slurp(base + "_cells.bin");
    Insist(cells.size() == 3 * n_cells * sizeof(double), "cell coefficients");
    const double *c = reinterpret_cast<const double *>(cells.data());
    for (size_t g = 0; g < n_cells; ++g) mesh.cells()[g].set_coefficients(c[g], c[n_cells + g], c[2 * n_cells + g]);
    const auto raw = slurp(base + "_in.bin");
    Insist(raw.size() == n * sizeof(Record), "photon list");
    std::vector<Record> in(n);
    if (n) std::memcpy(in.data(), raw.data(), raw.size());
    Census_T all;
    load(in, seed_hi, all);
    IMC_State state(next_dt);
    GPU_Setup gpu_setup;
    std::vector<double> abs_E(n_cells, -1.0), track_E(n_cells, -1.0);  // overwritten by the call
    Census_T census = replicated_transport<Census_T>(mesh, gpu_setup, state, abs_E, track_E, all, 1, 0,
                                                     Constants::HISTORY);
    const auto end = store(all), cen = store(census);
    spill(base + "_end_" + tag + ".bin", end.data(), end.size() * sizeof(Record));
    spill(base + "_census_" + tag + ".bin", cen.data(), cen.size() * sizeof(Record));
    std::vector<double> t(abs_E);
    t.insert(t.end(), track_E.begin(), track_E.end());
    spill(base + "_tally_" + tag + ".bin", t.data(), t.size() * sizeof(double));
    std::FILE *f = std::fopen((base + "_state_" + tag + ".txt").c_str(), "w");
    std::fprintf(f, "%.17g %.17g %llu %.9g\n", state.exit_E, state.post_census_E,
                 (unsigned long long)state.census_size, state.rank_transport_runtime);
    std::fclose(f);
  }
}

}  // namespace

int main(int argc, char **argv) {
  Insist(argc == 3, "usage: standin_driver <dir> <aos|soa>");
  const std::string dir = argv[1], tag = argv[2];
  const auto m = slurp(dir + "/mesh.bin");
  uint32_t hdr[3];
  int32_t bc[6];
  uint32_t seed;
  std::memcpy(hdr, m.data(), sizeof hdr);
  std::memcpy(bc, m.data() + 12, sizeof bc);
  std::memcpy(&seed, m.data() + 36, sizeof seed);
  const double *planes = reinterpret_cast<const double *>(m.data() + 40);
  std::vector<double> x(planes, planes + hdr[0] + 1);
  std::vector<double> y(planes + hdr[0] + 1, planes + hdr[0] + hdr[1] + 2);
  std::vector<double> z(planes + hdr[0] + hdr[1] + 2, planes + hdr[0] + hdr[1] + hdr[2] + 3);
  std::array<Constants::bc_type, 6> b;
  for (int f = 0; f < 6; ++f) b[f] = static_cast<Constants::bc_type>(bc[f]);
  Mesh mesh(x, y, z, b);
  const uint64_t seed_hi = (uint64_t)seed << 32;
  if (tag == "aos")
    run<std::vector<Photon>>(dir, tag, mesh, seed_hi);
  else
    run<PhotonArray>(dir, tag, mesh, seed_hi);
  return 0;
}
