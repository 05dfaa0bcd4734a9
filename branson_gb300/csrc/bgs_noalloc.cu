// bgs_transport_device_noalloc: the history transport on caller-owned device
// buffers, with every byte of scratch in one file-scope static device array,
// so the call allocates nothing.
//
// Who needs it: host codes that own all device memory through their own
// pool allocator (the LANL physics codes Branson proxies allocate through
// memory pools and do not let libraries call cudaMalloc/cudaFree), and code
// running where a device allocation is not allowed or would serialise the
// device (inside a pool-managed time step, or between launches that must not
// be separated by an implicit device synchronisation).  bgs_create and the
// other entry points allocate their banks and tables with cudaMalloc; this
// one uses the static array below instead.
//
// The scratch: 128-bit fixed-point tallies, the per-cell transport table,
// the work-queue/diagnostic block and the fixed-point scale bounds, sized for
// at most kNoAllocMaxCells cells (about 11 MB, held by every GPU that loads
// the library until the process exits).  The photon arrays, geometry,
// opacities and output tallies are the caller's device buffers.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (once per device, with that device current), so
// the first call on each device must come before any stream capture.
// Every call is synchronous: it enqueues its work on the caller's stream,
// copies the device checks' flags back into host memory and waits for the
// stream before it returns.
// Every call shares the one array: the tallies and counters are cleared at
// the start of each call, and two calls whose work overlaps on the GPU (on
// different streams, or from different host threads) race on it.
#include <cstdint>
#include <mutex>

#include "../../include/branson_gb300.h"
#include "bgs_kernels.cuh"

namespace bgs {
namespace {

constexpr uint32_t kNoAllocMaxCells = 131072;  // 2^17: the 50^3 hot zone fits

struct NoAllocLayout {
  static constexpr size_t tally = 0;
  static constexpr size_t xs = tally + sizeof(TallyCell) * kNoAllocMaxCells;
  static constexpr size_t group_v = xs + sizeof(CellXS) * kNoAllocMaxCells;
  static constexpr size_t inv_saf = group_v + sizeof(double) * kNoAllocMaxCells;
  static constexpr size_t diag = (inv_saf + sizeof(double) * kNoAllocMaxCells + 255) & ~size_t(255);
  static constexpr size_t maxbits = (diag + sizeof(DeviceDiag) + 255) & ~size_t(255);
  static constexpr size_t bytes = maxbits + 2 * sizeof(unsigned long long);
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[NoAllocLayout::bytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_ptr[kMaxDevices] = {};  // device address per device

__global__ void k_noalloc_begin(DeviceDiag *d, unsigned long long n) {
  d->n_bank = n;
  d->work_counter = 0;
  d->n_segments = 0;
  d->flags = 0;
}

// post_process_photons' census reset (post_process_functions.h:80): life_dx
// of CENSUS photons becomes c*next_dt in place (no compaction here)
__global__ void k_noalloc_census_life(Bank b, unsigned long long n, double life) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x)
    if (b.desc[i] == CENSUS) b.life[i] = life;
}

}  // namespace
}  // namespace bgs

using namespace bgs;

extern "C" BGS_API int bgs_transport_device_noalloc(
    uint32_t ngx, uint32_t ngy, uint32_t ngz, uint32_t n_groups, const double *x_planes,
    const double *y_planes, const double *z_planes, const int32_t bc[6], const double *op_a,
    const double *op_s, const double *f, uint32_t seed, uint64_t n, const bgs_photons_host *photons,
    double next_dt, double *abs_E, double *track_E, void *stream) {
  if (!x_planes || !y_planes || !z_planes || !bc || !op_a || !op_s || !f || !photons || !abs_E ||
      !track_E || n_groups == 0)
    return BGS_ERR_INVALID;
  const uint64_t n_cells64 = (uint64_t)ngx * ngy * ngz;
  if (ngx == 0 || ngy == 0 || ngz == 0) return BGS_ERR_INVALID;
  if (n_cells64 > kNoAllocMaxCells) return BGS_ERR_CAPACITY;  // beyond the static scratch
  for (int k = 0; k < 6; ++k)
    if (bc[k] != BGS_REFLECT && bc[k] != BGS_VACUUM && bc[k] != BGS_SOURCE) return BGS_ERR_INVALID;
  const bgs_photons_host &p = *photons;
  if (!p.pos_x || !p.pos_y || !p.pos_z || !p.dir_x || !p.dir_y || !p.dir_z || !p.E || !p.E0 ||
      !p.life_dx || !p.cell || !p.group || !p.descriptor || !p.rng_stream || !p.rng_counter)
    return BGS_ERR_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return BGS_ERR_NO_DEVICE;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void *ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return BGS_ERR_CUDA;
      g_scratch_ptr[dev] = static_cast<unsigned char *>(ptr);
    }
  }
  unsigned char *base = g_scratch_ptr[dev];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int n_sm = 0;
  if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return BGS_ERR_CUDA;

  MeshDev m{};
  m.ngx = ngx; m.ngy = ngy; m.ngz = ngz; m.n_groups = n_groups;
  m.n_cells = (uint32_t)n_cells64; m.n_regions = 0;
  m.x = x_planes; m.y = y_planes; m.z = z_planes;
  m.region = nullptr; m.regions = nullptr;
  for (int k = 0; k < 6; ++k) m.bc[k] = bc[k];
  m.T_source = 0.0;
  m.inv_ngx = div_multiplier(m.ngx);
  m.inv_ngxy = div_multiplier((uint64_t)m.ngx * m.ngy);
  CellsDev c{};
  c.op_a = const_cast<double *>(op_a);
  c.op_s = const_cast<double *>(op_s);
  c.f = const_cast<double *>(f);
  c.tally = reinterpret_cast<TallyCell *>(base + NoAllocLayout::tally);
  c.xs = reinterpret_cast<CellXS *>(base + NoAllocLayout::xs);
  c.group_v = reinterpret_cast<double *>(base + NoAllocLayout::group_v);
  c.inv_saf = reinterpret_cast<double *>(base + NoAllocLayout::inv_saf);
  DeviceDiag *d = reinterpret_cast<DeviceDiag *>(base + NoAllocLayout::diag);
  unsigned long long *maxbits = reinterpret_cast<unsigned long long *>(base + NoAllocLayout::maxbits);
  Bank b{p.pos_x, p.pos_y, p.pos_z, p.dir_x, p.dir_y, p.dir_z, p.E, p.E0, p.life_dx, p.cell, p.group,
         p.descriptor, p.source_type, reinterpret_cast<unsigned long long *>(p.rng_stream),
         reinterpret_cast<unsigned long long *>(p.rng_counter)};

  // clear what must start at zero: this call's tallies and the diagnostics
  if (cudaMemsetAsync(c.tally, 0, sizeof(TallyCell) * m.n_cells, s) != cudaSuccess) return BGS_ERR_CUDA;
  if (cudaMemsetAsync(d, 0, sizeof(DeviceDiag), s) != cudaSuccess) return BGS_ERR_CUDA;
  k_noalloc_begin<<<1, 1, 0, s>>>(d, n);
  launch_cell_xs(m, c, s);
  launch_bank_bounds(b, maxbits, d, n_sm, s);
  launch_transport_history(m, c, b, d, seed, transport_launch_shape(n_sm), s);
  k_noalloc_census_life<<<n_sm * 4, 256, 0, s>>>(b, n, kC * next_dt);
  launch_tally_to_double(m, c, d, abs_E, track_E, s);
  if (cudaGetLastError() != cudaSuccess) return BGS_ERR_CUDA;
  uint32_t flags = 0;
  if (cudaMemcpyAsync(&flags, &d->flags, sizeof(flags), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return BGS_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return BGS_ERR_CUDA;
  return flags ? BGS_ERR_DEVICE : BGS_OK;
}
