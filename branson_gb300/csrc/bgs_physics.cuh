// Per-segment physics of transport_photon (history_based_transport.h:55-139),
// shared by the history kernel (bgs_transport.cu), the batched kernel
// (bgs_batch.cu), the event-mode stage kernels (bgs_event.cu) and the adjoint
// replay (bgs_adjoint.cu), so all of them run the identical arithmetic.
#pragma once

#include "bgs_fixmath.cuh"
#include "bgs_kernels.cuh"

namespace bgs {

constexpr int kTransportThreads = 128;
// Minimum resident 128-thread blocks per SM of the history kernel (its
// register budget: 7 blocks is 72 registers)
#ifndef BGS_MIN_BLOCKS
#define BGS_MIN_BLOCKS 7
#endif


// a/b correctly rounded from y = RN(1/b): q0 = RN(a*y) is within one ulp of
// a/b, the remainder a - b*q0 is exact in one fma, and RN(q0 + r*y) is the
// correctly rounded quotient (Markstein's theorem for round-to-nearest, no
// overflow or underflow in the steps: |b| in [2^-900, 2^900] and |a| far
// below 2^100 here).  Three FP64 operations instead of a division; y == 0
// marks a divisor outside that range, which is divided directly.  The
// result equals the IEEE quotient a/b bit for bit (also checked against it
// on 1e9 random and adversarial operand pairs).
__device__ __forceinline__ double div_recip(double a, double b, double y) {
  if (__double_as_longlong(y) == 0) return a / b;
  const double q0 = __dmul_rn(a, y);
  const double r = __fma_rn(-q0, b, a);
  return __fma_rn(r, y, q0);
}

// One history's state in registers.  The birth weight E0 is not kept: the
// cutoff runs against RN(0.01 E0), and the rare exact test reads E0 from the
// bank.  The face planes ahead are kept only by kernels that ask for them
// (kFaces); the others read them from the mesh planes per segment.
struct Lane {
  double px, py, pz, dx, dy, dz, E, life;
  long long kill_key;  // f64_key(RN(0.01 * E0)): the cutoff test runs against it in integer ulps
  double fx, fy, fz;  // the current cell's face planes ahead along x, y, z (kFaces)
  double thr_abs;   // absorbed energy of the current cell visit
  double thr_dep;   // the remaining energy a cutoff kill deposits (visit_deposit)
  uint32_t idx;  // bank index (bgs_create keeps banks below 2^32 photons)
  Rng rng;
  uint32_t cell, group, ci, cj, ck, segs;
};

// the node planes the photon moves toward along each axis: the upper one
// for a positive direction cosine, else the lower one (the faces
// get_distance_to_boundary measures to, cell.h:117-132)
template <bool kFaces = false>
__device__ __forceinline__ void load_faces(const MeshDev &m, Lane &L) {
  if constexpr (kFaces) {
    L.fx = m.x[L.ci + ((__double_as_longlong(L.dx) > 0) ? 1u : 0u)];
    L.fy = m.y[L.cj + ((__double_as_longlong(L.dy) > 0) ? 1u : 0u)];
    L.fz = m.z[L.ck + ((__double_as_longlong(L.dz) > 0) ? 1u : 0u)];
  }
}


// Warp-aggregated tally flush of cell visits (a: the visit's absorbed
// energy, t: the part of it a cutoff kill deposited; TallyCell): every lane
// of the warp calls it (flush false for lanes with nothing to add); lanes
// flushing into the same cell
// (__match_any_sync on the cell, or on problem<<32|cell for the batched
// kernel) add their 128-bit fixed-point contributions by shuffles and one
// lane per cell issues the atomics.  Fixed-point sums are exact, so the
// tallies are the same bits as with one atomic per lane; few-cell meshes
// (where many lanes hit one cell) need far fewer atomics.
__device__ __forceinline__ void add128(unsigned long long &lo, unsigned long long &hi, unsigned long long vlo,
                                       unsigned long long vhi) {
  lo += vlo;
  hi += vhi + (lo < vlo ? 1ULL : 0ULL);
}

template <typename Key>
__device__ __forceinline__ void flush_tally_warp(TallyCell *tally, bool flush, Key key, uint32_t cell, double a,
                                                 double t, uint32_t &flags, int sa) {
  if (!__any_sync(0xffffffffu, flush)) return;
  unsigned long long alo = 0, ahi = 0, tlo = 0, thi = 0;
  if (flush) {
    if ((__double_as_longlong(a) << 1) != 0 && !to_fixed128(a, sa, alo, ahi)) {
      flags |= (a == a) ? FLAG_TALLY_RANGE : FLAG_NAN;
      alo = ahi = 0;
    }
    if ((__double_as_longlong(t) << 1) != 0 && !to_fixed128(t, sa, tlo, thi)) {
      flags |= (t == t) ? FLAG_TALLY_RANGE : FLAG_NAN;
      tlo = thi = 0;
    }
  }
  const unsigned grp = __match_any_sync(0xffffffffu, flush ? key : (Key)~(Key)0);
  if (!flush) return;
  if (grp & (grp - 1)) {  // several lanes on this cell: sum into the first
    unsigned long long s_alo = 0, s_ahi = 0, s_tlo = 0, s_thi = 0;
    unsigned mm = grp;
    while (mm) {
      const int m = __ffs(mm) - 1;
      mm &= mm - 1;
      add128(s_alo, s_ahi, __shfl_sync(grp, alo, m), __shfl_sync(grp, ahi, m));
      add128(s_tlo, s_thi, __shfl_sync(grp, tlo, m), __shfl_sync(grp, thi, m));
    }
    alo = s_alo; ahi = s_ahi; tlo = s_tlo; thi = s_thi;
  }
  if ((int)(threadIdx.x & 31u) == __ffs(grp) - 1) {
    TallyCell *tc = &tally[cell];
    if (alo | ahi) atomic_add128(&tc->abs_lo, &tc->abs_hi, alo, ahi);
    if (tlo | thi) atomic_add128(&tc->dep_lo, &tc->dep_hi, tlo, thi);
  }
}


// Per-warp ring of cell visits waiting for their tally flush, in shared
// memory.  A loop trip ends a visit in only a few lanes, so flushing every
// trip runs the conversions, the cell match and the atomics (whose L2
// round trip the warp waits for) with most lanes idle; instead each trip
// appends its ended visits, and once 32 are waiting the whole warp flushes
// them, one visit per lane.  Integer tally sums do not depend on the order
// of the adds, so the tallies are the same bits.  key is the cell, or
// problem << 32 | cell in the batched kernel.
constexpr uint32_t kFlushRing = 64;  // < 32 waiting before a trip's (at most 32) appends
struct FlushRing {
  unsigned long long key[kFlushRing];
  double a[kFlushRing], t[kFlushRing];
};

// append this trip's ended visits; head/tail are the warp's (uniform) counters
__device__ __forceinline__ void ring_push(FlushRing &r, uint32_t tail_in, uint32_t &tail, bool flush,
                                          unsigned long long key, double a, double t) {
  const unsigned fb = __ballot_sync(0xffffffffu, flush);
  if (flush) {
    const uint32_t s = (tail_in + __popc(fb & ((1u << (threadIdx.x & 31u)) - 1u))) & (kFlushRing - 1u);
    r.key[s] = key;
    r.a[s] = a;
    r.t[s] = t;
  }
  tail = tail_in + __popc(fb);
}

// take the next n (<= 32) waiting visits, one per lane (flush false past n)
__device__ __forceinline__ bool ring_take(const FlushRing &r, uint32_t head, uint32_t n, unsigned long long &key,
                                          double &a, double &t) {
  __syncwarp();
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t s = (head + lane) & (kFlushRing - 1u);
  const bool take = lane < n;
  key = take ? r.key[s] : 0ULL;
  a = take ? r.a[s] : 0.0;
  t = take ? r.t[s] : 0.0;
  __syncwarp();  // every lane has read its slot before the slots are reused
  return take;
}

__device__ __forceinline__ void store_end(const Bank &b, const Lane &L, uint8_t desc) {
  const unsigned long long i = L.idx;
  b.px[i] = L.px; b.py[i] = L.py; b.pz[i] = L.pz;
  b.dx[i] = L.dx; b.dy[i] = L.dy; b.dz[i] = L.dz;
  b.E[i] = L.E; b.life[i] = L.life;
  b.cell[i] = L.cell; b.group[i] = L.group;
  b.desc[i] = desc; b.ctr[i] = L.rng.ctr;
}

// sample_emission_group, Cell version (sampling_functions.h:126-138) with
// all groups at the same opacity: walk the CDF in steps of v; a walk that
// would run past the last group stays in the last group.
__device__ __forceinline__ uint32_t sample_group(Rng &r, double v, uint32_t n_groups) {
  double cdf = r.next();
  int g = -1;
  while (cdf > 0) {
    ++g;
    cdf -= v;
    if ((uint32_t)g == n_groups - 1) break;
  }
  return g < 0 ? 0u : (uint32_t)g;
}


// Comparisons on the integer pipe.  FP64 issue is the transport kernels'
// bound on this part (two FP64 lanes per clock per SM), so the segment's
// ordering tests use the doubles' bit patterns: for any non-NaN a and b,
// a < b exactly when f64_key(a) < f64_key(b) (the key is monotone over the
// signed 64-bit integers and gives -0 and +0 the same value), and
// f64_positive(x) is 0.0 < x.
__device__ __forceinline__ long long f64_key(double x) {
  long long b = __double_as_longlong(x);
  if (b == (long long)0x8000000000000000ULL) b = 0;  // -0 orders as +0
  return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ bool f64_positive(double x) { return __double_as_longlong(x) > 0; }

// a history's birth weight: the key of the cutoff threshold RN(0.01 E0)
__device__ __forceinline__ void set_birth(Lane &L, double E0) { L.kill_key = f64_key(kCutoff * E0); }

// what one segment ends in (the event branches of transport_photon)
enum SegEvent : int { SEG_KILLED = 0, SEG_SCATTER = 1, SEG_BOUNDARY = 2, SEG_CENSUS = 3 };

// Cutoff-kill part of the absorbed energy of the visit being flushed (the
// remaining weight a killed history deposits, history_based_transport.h:
// 81-82); the track-length tally of a cell is (abs - dep) / (sigma_a f)
// (TallyCell).  Upstream adds absorbed/(sigma_a f) per segment
// (history_based_transport.h:75-77); with sigma_a f constant in the cell
// over the step, the per-cell form is equal up to rounding.
__device__ __forceinline__ double visit_deposit(const Lane &L, int ev) {
  return ev == SEG_KILLED ? L.thr_dep : 0.0;
}

// Single-precision image of a double, truncated (relative error below
// 2^-23); false when |x| is nonzero and outside float's normal range.
__device__ __forceinline__ bool f32_image(double x, float &f) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const bool zero = (u << 1) == 0;
  const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
  const unsigned mag = hi & 0x7FFFFFFFu;
  // exponent field e in [897, 1150] is float's normal range: the float's
  // exponent field is e - 896 and its 23 mantissa bits the double's top 23
  const unsigned bits = __funnelshift_l(lo, mag - (896u << 20), 3) | (hi & 0x80000000u);
  f = zero ? 0.0f : __uint_as_float(bits);
  return zero || (mag - (897u << 20)) < ((1151u - 897u) << 20);
}

// approximate single-precision reciprocal (PTX rcp.approx: within one ulp)
// of a normal float
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// The face that get_distance_to_boundary picks (cell.h:117-132), decided
// from single-precision quotients, with one double division for the
// winner.  Each approximate quotient (two truncated images, the reciprocal
// within one ulp, the product) is within 2^-21 (relative) of the correctly
// rounded one, so when the winner is separated from every other candidate
// by more than 2^-18 of their magnitudes, and every quotient from the 1e16
// limit by more than 1e-4 of it, the exact comparisons order them the same
// way and the division returns the distance the three-division form would.
// A lane whose winner exceeds its collision distance by more than 2^-18
// skips the division (the boundary is then not the event); FP64 work costs
// the pipe per active lane, so the division runs on the pipe only for the
// lanes whose boundary can come first.
// Anything else (near ties, a zero or subnormal-range direction cosine, a
// cosine image whose reciprocal flushes to zero, a quotient near 1e16 or
// beyond float's range) returns false and the caller runs the three exact
// divisions.
__device__ __forceinline__ bool approx_faces(double ax, double ay, double az, const Lane &L, bool posx,
                                             bool posy, bool posz, double dist_to_scatter, double &dist_to_boundary,
                                             long long &k_boundary, uint32_t &surface_cross) {
  float fax, fay, faz, fdx, fdy, fdz;
  bool ok = f32_image(ax, fax) & f32_image(ay, fay) & f32_image(az, faz);
  ok &= f32_image(L.dx, fdx) & f32_image(L.dy, fdy) & f32_image(L.dz, fdz);
  ok &= (fdx != 0.0f) & (fdy != 0.0f) & (fdz != 0.0f);
  const float rx = rcp_approx(fdx), ry = rcp_approx(fdy), rz = rcp_approx(fdz);
  // reciprocals that flushed to zero (cosine images above 2^126) fall back
  ok &= ((__float_as_uint(rx) & 0x7F800000u) != 0) & ((__float_as_uint(ry) & 0x7F800000u) != 0) &
        ((__float_as_uint(rz) & 0x7F800000u) != 0);
  const float qx = fax * rx, qy = fay * ry, qz = faz * rz;
  constexpr float kLo = 9.9999e15f, kHi = 1.0001e16f, kTol = 3.814697265625e-06f;  // 1e16 -+ 1e-4, 2^-18
  const float kInf = __int_as_float(0x7f800000);
  ok &= !(qx >= kLo && qx <= kHi) & !(qy >= kLo && qy <= kHi) & !(qz >= kLo && qz <= kHi);
  const float cx = qx < kLo ? qx : kInf, cy = qy < kLo ? qy : kInf, cz = qz < kLo ? qz : kInf;
  // the first smallest (x, then y, then z) and the smallest of the others,
  // by selects: which face wins differs from lane to lane
  const bool y_first = cy < cx;
  int j = y_first ? 1 : 0;
  float m = y_first ? cy : cx;
  float second = y_first ? fminf(cx, cz) : fminf(cy, cz);
  const bool z_first = cz < m;
  j = z_first ? 2 : j;
  second = z_first ? fminf(cx, cy) : second;
  m = z_first ? cz : m;
  if (m != kInf) ok &= (second == kInf) || (second - m > kTol * (fabsf(second) + fabsf(m)));
  if (!ok) return false;
  if (m == kInf) {  // no face closer than 1e16
    dist_to_boundary = 1.0e16;
    k_boundary = f64_key(1.0e16);
    surface_cross = 0;
    return true;
  }
  const bool pos = j == 0 ? posx : (j == 1 ? posy : posz);
  surface_cross = 2u * (uint32_t)j + (pos ? 1u : 0u);
  // the collision comes first by more than the quotients' error: the
  // boundary is not the event and no comparison needs its exact distance
  // (census first or collision first is then decided by those two alone),
  // so that lane leaves the division out
  float fs;
  if (f32_image(dist_to_scatter, fs) && fs > 0.0f && m > fs * (1.0f + kTol)) {
    dist_to_boundary = __longlong_as_double(0x7FF0000000000000LL);
    k_boundary = 0x7FF0000000000000LL;
    return true;
  }
  const double a = j == 0 ? ax : (j == 1 ? ay : az);
  const double b = j == 0 ? L.dx : (j == 1 ? L.dy : L.dz);
  dist_to_boundary = a / b;
  k_boundary = f64_key(dist_to_boundary);
  return true;
}

// details of a segment the adjoint replay needs (unused elsewhere, so the
// compiler drops them from the other kernels)
struct SegInfo {
  double d;          // distance moved
  double absorbed;   // energy absorbed on the way
  bool collided;     // the segment ended at the sampled collision distance
};

// One segment up to the event decision: distance to collision, to the cell
// faces and to census, implicit-capture decay and track tally, the move, and
// the cutoff test (history_based_transport.h:56-91).  On SEG_KILLED the
// remaining energy has been added to the cell's absorbed energy, as upstream.
template <bool kFaces = false>
__device__ __forceinline__ int segment_advance(const MeshDev &m, const double *E0s, const CellXS &xs, Lane &L,
                                               uint32_t &surface_cross, uint32_t &flags,
                                               SegInfo *info = nullptr) {
  ++L.segs;
  const bool scatters = f64_positive(xs.sig_eff);
  // -log(u) / sigma_eff with the integer, correctly rounded -log
  // (bgs_fixmath.cuh) and the division by the cell's stored reciprocal
  const double dist_to_scatter =
      scatters ? div_recip(fix::neg_log_u53(L.rng.next_m53()), xs.sig_eff, xs.inv_se) : 1.0e100;
  // Cell::get_distance_to_boundary (cell.h:117-132): the first face with
  // the smallest (face - pos)/dir below 1e16, else 1e16 and face 0.  The
  // comparisons are the upstream ones, evaluated on the integer keys.
  double dist_to_boundary = 1.0e16;
  long long k_boundary = f64_key(1.0e16);
  surface_cross = 0;
  const bool posx = f64_positive(L.dx), posy = f64_positive(L.dy), posz = f64_positive(L.dz);
  double ax, ay, az;
  if constexpr (kFaces) {
    ax = L.fx - L.px;
    ay = L.fy - L.py;
    az = L.fz - L.pz;
  } else {
    ax = m.x[L.ci + (posx ? 1u : 0u)] - L.px;
    ay = m.y[L.cj + (posy ? 1u : 0u)] - L.py;
    az = m.z[L.ck + (posz ? 1u : 0u)] - L.pz;
  }
  if (!approx_faces(ax, ay, az, L, posx, posy, posz, dist_to_scatter, dist_to_boundary, k_boundary, surface_cross)) {
    double dist = ax / L.dx;
    long long k = f64_key(dist);
    if (k < k_boundary) { dist_to_boundary = dist; k_boundary = k; surface_cross = posx ? 1u : 0u; }
    dist = ay / L.dy;
    k = f64_key(dist);
    if (k < k_boundary) { dist_to_boundary = dist; k_boundary = k; surface_cross = posy ? 3u : 2u; }
    dist = az / L.dz;
    k = f64_key(dist);
    if (k < k_boundary) { dist_to_boundary = dist; k_boundary = k; surface_cross = posz ? 5u : 4u; }
  }
  const double dist_to_census = L.life;
  // std::min(a, b) == (b < a) ? b : a; the event tests that follow
  // (dist_to_event == dist_to_scatter, then == dist_to_boundary) are the
  // same comparisons read back
  const long long k_census = f64_key(dist_to_census);
  const bool census_first = k_census < k_boundary;
  const double inner = census_first ? dist_to_census : dist_to_boundary;
  const bool inner_first = (census_first ? k_census : k_boundary) < f64_key(dist_to_scatter);
  const double dist_to_event = inner_first ? inner : dist_to_scatter;

  const double absorbed_E = L.E * (1.0 - fix::exp_neg(-(xs.neg_saf * dist_to_event)));
  L.thr_abs += absorbed_E;
  L.E = L.E - absorbed_E;
  L.px += L.dx * dist_to_event;  // Photon::move (photon.h:109-114)
  L.py += L.dy * dist_to_event;
  L.pz += L.dz * dist_to_event;
  L.life -= dist_to_event;
  if (info) {
    info->d = dist_to_event;
    info->absorbed = absorbed_E;
    info->collided = !inner_first;
  }

  // below_cutoff: E/E0 < 0.01 (photon.h:47-49).  More than four ulps from
  // RN(0.01*E0), E < RN(0.01*E0) decides it the same way as RN(E/E0) < 0.01;
  // closer than that the exact quotient settles it
  const long long k_e = f64_key(L.E), k_thr = L.kill_key;
  bool killed = k_e < k_thr;
  if (k_e - k_thr <= 4 && k_thr - k_e <= 4) killed = L.E / E0s[L.idx] < kCutoff;
  if (killed || L.segs >= kMaxSegmentsPerHistory) {
    if (!killed) flags |= FLAG_SEGMENT_LIMIT;
    L.thr_dep = L.E;  // the kill deposit, outside the track tally
    L.thr_abs += L.E;
    return SEG_KILLED;
  }
  if (!inner_first) return SEG_SCATTER;
  if (!census_first) return SEG_BOUNDARY;
  return SEG_CENSUS;
}

// Effective scatter (history_based_transport.h:96-99): isotropic new
// direction (get_uniform_angle, sampling_functions.h:57-70) and, unless
// physical scattering wins, a resampled group.  kGray: one group and no
// physical scattering anywhere (MeshDev::gray), where both of those draws
// only advance the counter (below), so they are left out of the build.
template <bool kFaces = false, bool kGray = false>
__device__ __forceinline__ void scatter_update(const MeshDev &m, const CellsDev &c, const CellXS &xs,
                                               Lane &L) {
  const double mu = mu_from_m53(L.rng.next_m53());
  const double phi = L.rng.next_twice() * kPi;  // RN(RN(u * 2.0) * pi), u * 2.0 exact
  const double sin_theta = fix::sqrt_rn(1.0 - mu * mu);
  double sp, cp;
  fix::sincos_phi(phi, &sp, &cp);
  L.dx = sin_theta * cp;
  L.dy = sin_theta * sp;
  L.dz = mu;
  load_faces<kFaces>(m, L);
  if constexpr (kGray) {  // the two draws below, both skipped, and group 0
    L.rng.ctr += 2;
    L.group = 0;
    return;
  }
  // effective-scatter test and group resample (history_based_transport.h:97-98):
  // with sigma_s = 0 the test u > 0 always passes, and with one group the
  // walk always ends in group 0, so those draws only advance the counter
  bool resample;
  if (f64_positive(xs.p_scat)) resample = L.rng.next() > xs.p_scat;
  else { L.rng.skip(); resample = true; }
  if (resample) {
    if (m.n_groups > 1) L.group = sample_group(L.rng, c.group_v[L.cell], m.n_groups);
    else { L.rng.skip(); L.group = 0; }
  }
}

// boundary condition of the crossed face: interior faces are ELEMENT
// (proto_mesh.h:156-202).  Selects rather than a switch: the few lanes of a
// warp that cross a face in one loop trip cross different faces, and the
// cases of a switch would run one after another.
__device__ __forceinline__ int face_bc(const MeshDev &m, const Lane &L, uint32_t surface_cross) {
  const uint32_t axis = surface_cross >> 1;
  const bool up = (surface_cross & 1u) != 0u;
  const uint32_t idx = axis == 0 ? L.ci : (axis == 1 ? L.cj : L.ck);
  const uint32_t n = axis == 0 ? m.ngx : (axis == 1 ? m.ngy : m.ngz);
  if (up ? idx + 1 < n : idx > 0) return ELEMENT;
  // constant indices: a variable index into the kernel parameter's array
  // would make the compiler copy the whole MeshDev to local memory
  int bc = m.bc[5];
  bc = surface_cross == 4 ? m.bc[4] : bc;
  bc = surface_cross == 3 ? m.bc[3] : bc;
  bc = surface_cross == 2 ? m.bc[2] : bc;
  bc = surface_cross == 1 ? m.bc[1] : bc;
  bc = surface_cross == 0 ? m.bc[0] : bc;
  return bc;
}

// ELEMENT crossing: the photon enters the neighbour (cell.h:110-112); only
// the crossed axis gets a new face ahead.  Selects, as in face_bc.
template <bool kFaces = false>
__device__ __forceinline__ void enter_neighbour(const MeshDev &m, Lane &L, uint32_t surface_cross) {
  const uint32_t axis = surface_cross >> 1;
  const bool up = (surface_cross & 1u) != 0u;
  const uint32_t step = up ? 1u : 0xFFFFFFFFu;  // +1 or -1
  const uint32_t stride = axis == 0 ? 1u : (axis == 1 ? m.ngx : m.ngx * m.ngy);
  L.cell = up ? L.cell + stride : L.cell - stride;
  L.ci += axis == 0 ? step : 0u;
  L.cj += axis == 1 ? step : 0u;
  L.ck += axis == 2 ? step : 0u;
  if constexpr (kFaces) {
    const double *planes = axis == 0 ? m.x : (axis == 1 ? m.y : m.z);
    const uint32_t idx = (axis == 0 ? L.ci : (axis == 1 ? L.cj : L.ck)) + (up ? 1u : 0u);
    const double f = planes[idx];
    L.fx = axis == 0 ? f : L.fx;
    L.fy = axis == 1 ? f : L.fy;
    L.fz = axis == 2 ? f : L.fz;
  }
}

// REFLECT: Photon::reflect (photon.h:151-155): the direction cosine flips
// and the face ahead on that axis becomes the opposite plane of the cell.
// Selects, as in face_bc.
template <bool kFaces = false>
__device__ __forceinline__ void reflect(const MeshDev &m, Lane &L, uint32_t surface_cross) {
  const uint32_t axis = surface_cross >> 1;
  constexpr long long kSign = (long long)0x8000000000000000ULL;  // negation as a sign-bit flip
  L.dx = __longlong_as_double(__double_as_longlong(L.dx) ^ (axis == 0 ? kSign : 0LL));
  L.dy = __longlong_as_double(__double_as_longlong(L.dy) ^ (axis == 1 ? kSign : 0LL));
  L.dz = __longlong_as_double(__double_as_longlong(L.dz) ^ (axis == 2 ? kSign : 0LL));
  if constexpr (kFaces) {
    const double dir = axis == 0 ? L.dx : (axis == 1 ? L.dy : L.dz);
    const double *planes = axis == 0 ? m.x : (axis == 1 ? m.y : m.z);
    const uint32_t idx = (axis == 0 ? L.ci : (axis == 1 ? L.cj : L.ck)) + ((__double_as_longlong(dir) > 0) ? 1u : 0u);
    const double f = planes[idx];
    L.fx = axis == 0 ? f : L.fx;
    L.fy = axis == 1 ? f : L.fy;
    L.fz = axis == 2 ? f : L.fz;
  }
}

// cell coordinates and the faces ahead from the global cell index
template <bool kFaces = false>
__device__ __forceinline__ void locate(const MeshDev &m, Lane &L) {
  cell_coords(m, L.cell, L.ci, L.cj, L.ck);
  load_faces<kFaces>(m, L);
}

}  // namespace bgs
