"""ctypes binding to the C restatement in oracle/branson_oracle.c.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by the CPU-baseline leg of bench.py as the checker.  The product package
(branson_gb300) never imports this module.

``Oracle(deck)`` holds the mesh, the per-cell state and the census, and
``step()`` runs one replicated IMC time step the way imc_replicated_driver
does (src/replicated_driver.h:47-120): energies, sourcing, transport,
post-processing and the temperature update, returning everything a parity
test compares.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import time
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbranson_oracle.so")
# the diagnostic twin: the same C with the GPU path's integer -log/exp/sin/cos
# in place of libm (branson_oracle.c, BO_GPU_MATH); math="gpu" selects it
GPU_MATH_LIB_PATH = os.path.join(HERE, "_build", "libbranson_oracle_gpumath.so")
REF_DIR = os.path.join(HERE, "_ref")
FIXMATH_DIR = os.path.join(os.path.dirname(HERE), "branson_gb300", "csrc")

# bo_photon / harness record (104 bytes)
PHOTON_DTYPE = np.dtype([
    ("stream", "<u8"), ("counter", "<u8"), ("cell", "<u4"), ("group", "<u4"),
    ("source_type", "<u4"), ("descriptor", "<u4"), ("pos", "<f8", (3,)), ("dir", "<f8", (3,)),
    ("E", "<f8"), ("E0", "<f8"), ("life_dx", "<f8")])
assert PHOTON_DTYPE.itemsize == 104

C_LIGHT = 299.792458
EXIT, PASS, CENSUS, SCATTER, KILLED, BOUND = range(6)


def _stale(target: str, sources) -> bool:
    return not os.path.exists(target) or any(os.path.getmtime(target) < os.path.getmtime(s) for s in sources)


def build(force: bool = False, math: str = "libm") -> str:
    """Compile the C restatement with gcc (make -C oracle port), or its
    GPU-math twin (make -C oracle gpumath)."""
    srcs = [os.path.join(HERE, "branson_oracle.c"), os.path.join(HERE, "branson_oracle.h")]
    if math == "gpu":
        srcs += [os.path.join(HERE, "gpu_math.cc"), os.path.join(FIXMATH_DIR, "bgs_fixmath.cuh"),
                 os.path.join(FIXMATH_DIR, "bgs_fixmath_tables.h")]
        if force or _stale(GPU_MATH_LIB_PATH, srcs):
            subprocess.run(["make", "-s", "-C", HERE, "gpumath"], check=True)
        return GPU_MATH_LIB_PATH
    if math != "libm":
        raise ValueError("math is 'libm' (the oracle) or 'gpu' (its GPU-math twin)")
    if force or _stale(LIB_PATH, srcs):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


class _Region(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("cv", "rho", "opacA", "opacB", "opacC", "opacS", "T_e", "T_r")]


class _Mesh(C.Structure):
    _fields_ = [("ngx", C.c_uint32), ("ngy", C.c_uint32), ("ngz", C.c_uint32), ("n_groups", C.c_uint32),
                ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)), ("z", C.POINTER(C.c_double)),
                ("region", C.POINTER(C.c_uint32)), ("regions", C.POINTER(_Region)),
                ("bc", C.c_int * 6), ("T_source", C.c_double)]


class _Cells(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in
                ("T_e", "T_r", "T_s", "op_a", "op_s", "f", "emission_E", "census_E", "source_E", "T_r_diag")]


class _Energy(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("total_photon_E", "emission_E", "census_E", "source_E", "pre_mat_E")]


class TraceRec(C.Structure):
    _fields_ = [("d_scatter", C.c_double), ("d_boundary", C.c_double), ("d_census", C.c_double),
                ("face_q", C.c_double * 3), ("E", C.c_double), ("E0", C.c_double), ("cell", C.c_uint32),
                ("descriptor", C.c_uint32), ("surface", C.c_uint32), ("counter", C.c_uint32)]


TRACE_DTYPE = np.dtype([("d_scatter", "<f8"), ("d_boundary", "<f8"), ("d_census", "<f8"),
                        ("face_q", "<f8", (3,)), ("E", "<f8"), ("E0", "<f8"), ("cell", "<u4"),
                        ("descriptor", "<u4"), ("surface", "<u4"), ("counter", "<u4")])
assert TRACE_DTYPE.itemsize == C.sizeof(TraceRec)

_libs = {}


def lib(math: str = "libm"):
    if math not in _libs:
        path = build(math=math)
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        pp = C.c_void_p
        L.bo_rng_draw.restype = C.c_double
        L.bo_rng_draw.argtypes = [C.c_uint32, C.c_uint64, C.POINTER(C.c_uint64)]
        L.bo_threefry2x64_20.argtypes = [C.POINTER(C.c_uint64)] * 3
        L.bo_distance_to_boundary.restype = C.c_double
        L.bo_distance_to_boundary.argtypes = [dp, dp, dp, C.POINTER(C.c_uint32)]
        L.bo_initialize_cells.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells)]
        L.bo_calculate_photon_energy.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells), C.c_uint32,
                                                 C.c_double, C.POINTER(_Energy)]
        L.bo_count_photons.restype = C.c_uint64
        L.bo_count_photons.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells), C.c_uint64, C.c_double]
        L.bo_count_initial_census.restype = C.c_uint64
        L.bo_count_initial_census.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells), C.c_uint64, C.c_double]
        L.bo_make_photons.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells), C.c_double, C.c_uint32,
                                      C.c_uint32, C.c_uint64, C.c_double, pp]
        L.bo_make_initial_census.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells), C.c_double,
                                             C.c_uint32, C.c_uint64, C.c_double, pp]
        L.bo_transport.restype = C.c_uint64
        L.bo_transport.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells), C.c_uint32, pp, C.c_size_t,
                                   dp, dp, C.c_int]
        L.bo_post_process.restype = C.c_size_t
        L.bo_post_process.argtypes = [C.c_double, pp, C.c_size_t, pp, dp, dp]
        L.bo_update_temperature.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells), C.c_double, dp, dp,
                                            dp, dp]
        L.bo_adjoint_replay.restype = C.c_uint64
        L.bo_adjoint_replay.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells), C.c_uint32, pp, C.c_size_t, dp,
                                        C.c_int, C.c_double, dp, C.c_int]
        L.bo_comb_census.restype = C.c_size_t
        L.bo_comb_census.argtypes = [pp, C.c_size_t, C.c_uint32, C.c_int64, C.c_uint32, C.c_uint64,
                                     C.POINTER(C.c_uint64), pp]
        L.bo_adjoint_reweighted.restype = C.c_double
        L.bo_adjoint_reweighted.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells), dp, dp, C.c_uint32, pp,
                                            C.c_size_t, dp]
        L.bo_trace_photon.restype = C.c_size_t
        L.bo_trace_photon.argtypes = [C.POINTER(_Mesh), C.POINTER(_Cells), C.c_uint32, pp, pp, C.c_size_t, pp]
        _libs[math] = L
    return _libs[math]


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def rng_draws(seed: int, stream: int, n: int, counter: int = 0) -> np.ndarray:
    """n consecutive RNG(seed, stream) draws starting at ``counter``."""
    L = lib()
    c = C.c_uint64(counter)
    return np.array([L.bo_rng_draw(seed, stream, C.byref(c)) for _ in range(n)])


def threefry(ctr, key):
    L = lib()
    a = (C.c_uint64 * 2)(*ctr)
    k = (C.c_uint64 * 2)(*key)
    o = (C.c_uint64 * 2)()
    L.bo_threefry2x64_20(a, k, o)
    return int(o[0]), int(o[1])


@dataclass
class StepResult:
    step: int
    dt: float
    next_dt: float
    total_photon_E: float
    emission_E: float
    source_E: float
    pre_census_E: float
    op_a: np.ndarray
    f: np.ndarray
    emission_cell_E: np.ndarray
    census_cell_E: np.ndarray
    source_cell_E: np.ndarray
    source: np.ndarray          # photon records before transport
    end: np.ndarray             # after transport + post-process
    census: np.ndarray
    abs_E: np.ndarray
    track_E: np.ndarray
    T_e: np.ndarray             # after the temperature update
    T_r: np.ndarray
    census_E: float
    exit_E: float
    absorbed_E: float
    pre_mat_E: float
    post_mat_E: float
    segments: int
    transport_s: float


class Oracle:
    """CPU replicated IMC problem driven through the C restatement."""

    def __init__(self, deck, n_threads: int = 1, math: str = "libm"):
        self.deck = deck
        self.n_threads = n_threads
        self.math = math
        self.L = lib(math)
        x, y, z = deck.planes()
        self._keep = [np.ascontiguousarray(x), np.ascontiguousarray(y), np.ascontiguousarray(z),
                      deck.cell_regions()]
        regs = deck.region_table()
        self._regions = (_Region * len(regs))(*[_Region(*row) for row in regs])
        nx, ny, nz = deck.shape
        self.n_cells = nx * ny * nz
        self.mesh = _Mesh(nx, ny, nz, deck.n_groups, _dptr(self._keep[0]), _dptr(self._keep[1]),
                          _dptr(self._keep[2]), self._keep[3].ctypes.data_as(C.POINTER(C.c_uint32)),
                          self._regions, (C.c_int * 6)(*deck.bc), deck.T_source)
        self.arr = {k: np.zeros(self.n_cells) for k in
                    ("T_e", "T_r", "T_s", "op_a", "op_s", "f", "emission_E", "census_E", "source_E", "T_r_diag")}
        self.cells = _Cells(*[_dptr(self.arr[n]) for n, _ in _Cells._fields_])
        self.L.bo_initialize_cells(C.byref(self.mesh), C.byref(self.cells))
        self.census = np.zeros(0, PHOTON_DTYPE)
        # IMC_State time stepping (src/imc_state.h:42-45, :112-134, :292-296)
        self.time = deck.t_start
        self.dt = deck.dt_start
        self.step_no = 1

    def next_dt(self) -> float:
        d = self.deck
        nd = self.dt * d.t_mult if self.dt * d.t_mult < d.dt_max else d.dt_max
        if self.time + nd > d.t_stop:
            nd = d.t_stop - self.time
        return nd

    def finished(self) -> bool:
        return abs(self.time - self.deck.t_stop) < 1.0e-8

    def set_T_e(self, T_e: np.ndarray) -> None:
        self.arr["T_e"][:] = T_e

    def source(self, step: int):
        """Energies and the photon list of one step (driver :54-75)."""
        L = self.L
        d = self.deck
        en = _Energy()
        L.bo_calculate_photon_energy(C.byref(self.mesh), C.byref(self.cells), step, self.dt, C.byref(en))
        total = en.total_photon_E
        if step == 1:
            n_ce = L.bo_count_initial_census(C.byref(self.mesh), C.byref(self.cells), d.photons, total)
            self.census = np.zeros(n_ce, PHOTON_DTYPE)
            L.bo_make_initial_census(C.byref(self.mesh), C.byref(self.cells), self.dt, d.seed, d.photons,
                                     total, self.census.ctypes.data)
        n_new = L.bo_count_photons(C.byref(self.mesh), C.byref(self.cells), d.photons, total)
        new = np.zeros(n_new, PHOTON_DTYPE)
        L.bo_make_photons(C.byref(self.mesh), C.byref(self.cells), self.dt, step, d.seed, d.photons, total,
                          new.ctypes.data)
        return en, np.concatenate([new, self.census])

    def transport(self, photons: np.ndarray, next_dt: float, n_threads: Optional[int] = None):
        """replicated_transport's CPU history branch (replicated_transport.h:88-92)."""
        L = self.L
        abs_E = np.zeros(self.n_cells)
        track_E = np.zeros(self.n_cells)
        t0 = time.perf_counter()
        segs = L.bo_transport(C.byref(self.mesh), C.byref(self.cells), self.deck.seed, photons.ctypes.data,
                              len(photons), _dptr(abs_E), _dptr(track_E),
                              self.n_threads if n_threads is None else n_threads)
        census = np.zeros(len(photons), PHOTON_DTYPE)
        ce, ex = C.c_double(0.0), C.c_double(0.0)
        nc = L.bo_post_process(next_dt, photons.ctypes.data, len(photons), census.ctypes.data,
                               C.byref(ce), C.byref(ex))
        elapsed = time.perf_counter() - t0
        return abs_E, track_E, census[:nc].copy(), ce.value, ex.value, int(segs), elapsed

    def adjoint(self, start: np.ndarray, w: np.ndarray, scale: int, visit_bound: float,
                n_threads: Optional[int] = None):
        """dL/dsigma_a of L = sum w*abs_E by the CPU replay of the adjoint
        estimator over the step's start photons, at the op_a/op_s/f of the
        step's energies (still in the cell arrays after the step); returns
        (gradient, visits dropped as out of range)."""
        w = np.ascontiguousarray(w, dtype=np.float64)
        grad = np.zeros(self.n_cells)
        start = np.ascontiguousarray(start)
        bad = self.L.bo_adjoint_replay(C.byref(self.mesh), C.byref(self.cells), self.deck.seed, start.ctypes.data,
                                      len(start), _dptr(w), int(scale), float(visit_bound), _dptr(grad),
                                      self.n_threads if n_threads is None else n_threads)
        return grad, int(bad)

    def reweighted_L(self, start: np.ndarray, w: np.ndarray, op_a_p: np.ndarray, f_p: np.ndarray) -> float:
        """L at perturbed opacities estimated on the unperturbed paths with
        likelihood ratios (its finite difference is the adjoint estimator)."""
        w = np.ascontiguousarray(w, dtype=np.float64)
        op_a_p = np.ascontiguousarray(op_a_p, dtype=np.float64)
        f_p = np.ascontiguousarray(f_p, dtype=np.float64)
        start = np.ascontiguousarray(start)
        return float(self.L.bo_adjoint_reweighted(C.byref(self.mesh), C.byref(self.cells), _dptr(op_a_p),
                                                 _dptr(f_p), self.deck.seed, start.ctypes.data, len(start),
                                                 _dptr(w)))

    def trace(self, start_record: np.ndarray, max_segments: int = 1 << 16):
        """transport_photon on one photon (a PHOTON_DTYPE record) with the
        cell state of the current step: (per-segment TRACE_DTYPE records,
        end record)."""
        rec = np.ascontiguousarray(np.asarray(start_record, dtype=PHOTON_DTYPE).reshape(1))
        out = np.zeros(max_segments, TRACE_DTYPE)
        end = np.zeros(1, PHOTON_DTYPE)
        n = self.L.bo_trace_photon(C.byref(self.mesh), C.byref(self.cells), self.deck.seed, rec.ctypes.data,
                                   out.ctypes.data, max_segments, end.ctypes.data)
        return out[:min(n, max_segments)].copy(), end[0]

    def fleck(self, op_a: np.ndarray, dt: float) -> np.ndarray:
        """Fleck factor per cell for the given opacities at the current
        temperatures (mesh.h:267)."""
        regs = self.deck.region_table()
        reg = self.deck.cell_regions()
        cv, rho = regs[reg, 0], regs[reg, 1]
        T = self.arr["T_e"]
        return 1.0 / (1.0 + dt * op_a * C_LIGHT * (4.0 * 0.01372 * T ** 3.0 / (cv * rho)))

    def step(self) -> StepResult:
        L = self.L
        step = self.step_no
        en, photons = self.source(step)
        pre_census_E = float(np.sum(self.census["E"]))
        source_copy = photons.copy()
        op_a, f = self.arr["op_a"].copy(), self.arr["f"].copy()
        em, ce_cell, so = self.arr["emission_E"].copy(), self.arr["census_E"].copy(), self.arr["source_E"].copy()
        nd = self.next_dt()
        abs_E, track_E, census, census_E, exit_E, segs, el = self.transport(photons, nd)
        abs_keep, track_keep = abs_E.copy(), track_E.copy()
        tot_abs, post_mat = C.c_double(), C.c_double()
        L.bo_update_temperature(C.byref(self.mesh), C.byref(self.cells), self.dt, _dptr(abs_E), _dptr(track_E),
                                C.byref(tot_abs), C.byref(post_mat))
        res = StepResult(step=step, dt=self.dt, next_dt=nd, total_photon_E=en.total_photon_E,
                         emission_E=en.emission_E, source_E=en.source_E, pre_census_E=pre_census_E,
                         op_a=op_a, f=f, emission_cell_E=em, census_cell_E=ce_cell, source_cell_E=so,
                         source=source_copy, end=photons, census=census, abs_E=abs_keep, track_E=track_keep,
                         T_e=self.arr["T_e"].copy(), T_r=self.arr["T_r_diag"].copy(), census_E=census_E,
                         exit_E=exit_E, absorbed_E=tot_abs.value, pre_mat_E=en.pre_mat_E,
                         post_mat_E=post_mat.value, segments=segs, transport_s=el)
        self.census = census
        self.time += self.dt
        self.dt = nd
        self.step_no += 1
        return res


def adjoint_scale(w, start, op_a, op_s, f, n_segments):
    """Fixed-point exponent and per-visit bound of the gradient sums, by the
    rule the GPU backward applies (bgs_adjoint_api.cu)."""
    import math
    w = np.asarray(w, np.float64)
    wmax = float(np.max(np.abs(w))) if w.size else 0.0
    max_E = float(np.max(np.abs(start["E"]))) if len(start) else 0.0
    max_L = float(np.max(np.abs(start["life_dx"]))) if len(start) else 0.0
    sig_eff = (1.0 - f) * op_a + op_s
    inv_se = np.where(sig_eff > 0.0, 1.0 / np.where(sig_eff > 0.0, sig_eff, 1.0), 0.0)
    src = np.where(op_a > 0.0, f / np.where(op_a > 0.0, op_a, 1.0), 0.0)
    coef = float(max(np.max(np.abs(src)), np.max(np.abs((1.0 - f * f) * inv_se))))
    bound = wmax * max_E * (3.0 * max_L + 8.0 * coef) * 4096.0
    if not bound > 0.0:
        return 0, bound
    _, e = math.frexp(bound * float(n_segments + len(start) + 1))
    return 118 - e, bound


def comb(census: np.ndarray, n_cells: int, max_census: int, seed: int, stream: int, counter: int = 0):
    """comb_photons (census_functions.h:48-93) on a census list (PHOTON_DTYPE
    records, list order) with RNG(seed, stream) from ``counter``: returns the
    combed list and the RNG counter after its draws (bo_comb_census)."""
    src = np.ascontiguousarray(census, dtype=PHOTON_DTYPE)
    out = np.empty_like(src)
    ctr = C.c_uint64(counter)
    m = lib().bo_comb_census(src.ctypes.data, len(src), n_cells, int(max_census), seed, stream, C.byref(ctr),
                             out.ctypes.data)
    return out[:m].copy(), int(ctr.value)


def read_harness_step(out_dir: str, step: int, n_cells: int) -> dict:
    """Load one step of oracle/ref_harness.cc output."""
    def rec(name):
        return np.fromfile(os.path.join(out_dir, f"step{step:03d}_{name}.bin"), dtype=PHOTON_DTYPE)
    cells = np.fromfile(os.path.join(out_dir, f"step{step:03d}_cells.bin"), dtype="<f8").reshape(n_cells, 9)
    scalars = {}
    with open(os.path.join(out_dir, f"step{step:03d}_scalars.txt")) as fh:
        for line in fh:
            k, v = line.split()
            scalars[k] = float(v)
    out = {"source": rec("source"), "end": rec("end"), "census": rec("census"), "cells": cells,
           "scalars": scalars}
    if os.path.exists(os.path.join(out_dir, f"step{step:03d}_comb.bin")):
        out["comb"] = rec("comb")
    return out


def run_reference_harness(deck, out_dir: str, n_steps: int, n_threads: int = 1, dump: bool = True,
                          timeout: Optional[float] = None, comb: Optional[tuple] = None) -> str:
    """Run the upstream-header harness (oracle/_ref) on ``deck``; returns stdout."""
    exe = os.path.join(REF_DIR, "ref_harness_g30" if deck.n_groups == 30 else "ref_harness_g1")
    if deck.n_groups not in (1, 30):
        raise ValueError("the reference harness is built for 1 and 30 groups")
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, "deck.xml")
    with open(path, "w") as fh:
        fh.write(deck.to_xml())
    args = [exe, path, out_dir, str(n_steps), str(n_threads)] + ([] if dump else ["--no-dump"])
    if comb is not None:  # (max_census_photons, stream): comb each step's census
        args += ["--comb", str(int(comb[0])), str(int(comb[1]))]
    r = subprocess.run(args, capture_output=True, text=True, timeout=timeout, check=True)
    return r.stdout
