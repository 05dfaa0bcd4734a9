"""Host-side mirror of Branson's replicated driver over the C ABI.

``ReplicatedIMC`` owns one device context and runs the replicated time step
(imc_replicated_driver, src/replicated_driver.h:33-122) on the GPU: per-cell
energies, sourcing, transport with census post-processing, and the tally
reduce fused with the temperature update.  Time stepping mirrors IMC_State
(src/imc_state.h:42-45, :112-134, :292-296).

``replicated_transport`` is the drop-in for the upstream call of the same
name (src/replicated_transport.h:33-158) on host photon buffers.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, Optional, Tuple

import numpy as np

from . import _lib
from ._lib import BransonError, PhotonArrays
from .deck import Deck


@dataclass
class StepReport:
    step: int
    dt: float
    next_dt: float
    n_transported: int
    n_census: int
    n_segments: int
    census_E: float
    exit_E: float
    absorbed_E: float
    post_mat_E: float
    device_flags: int


def default_capacity(deck: Deck) -> int:
    """Bank capacity: new photons are at most n_user + 2 per cell (the
    at-least-one rule, source.h:232-242), plus the census carried in."""
    return int(2 * (deck.photons + 3 * deck.n_cells) + 4096)


class ReplicatedIMC:
    def __init__(self, deck: Deck, device: int = 0, capacity: Optional[int] = None,
                 stream: Optional[int] = None):
        self.lib = _lib.load()
        self.deck = deck
        self.device = device
        self.algorithm = deck.algorithm  # HISTORY or EVENT for step(); the tuner may change it
        deck.validate()
        self.capacity = int(capacity or default_capacity(deck))
        ctx = C.c_void_p()
        rc = self.lib.bgs_create(C.byref(ctx), device, self.capacity, stream, deck.seed & 0xFFFFFFFF,
                                 int(deck.photons))
        if rc != 0:
            raise BransonError(rc, f"bgs_create: {self.lib.bgs_status_string(rc).decode()}")
        self.ctx = ctx
        self._set_mesh()
        self.time = deck.t_start
        self.dt = deck.dt_start
        self.step_no = 1

    # -------------------------------------------------------------- plumbing
    def _check(self, rc: int, what: str) -> None:
        if rc != 0:
            msg = self.lib.bgs_last_error(self.ctx).decode()
            raise BransonError(rc, f"{what}: {msg}")

    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.lib.bgs_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _set_mesh(self) -> None:
        d = self.deck
        x, y, z = d.planes()
        self._mesh_keep = [np.ascontiguousarray(x), np.ascontiguousarray(y), np.ascontiguousarray(z),
                           d.cell_regions(), np.ascontiguousarray(d.region_table())]
        nx, ny, nz = d.shape
        desc = _lib.MeshDesc(nx, ny, nz, d.n_groups, _lib.ptr(self._mesh_keep[0]), _lib.ptr(self._mesh_keep[1]),
                             _lib.ptr(self._mesh_keep[2]), _lib.ptr(self._mesh_keep[3]), len(d.regions),
                             _lib.ptr(self._mesh_keep[4]), (C.c_int32 * 6)(*d.bc), d.T_source)
        self._check(self.lib.bgs_set_mesh(self.ctx, C.byref(desc)), "bgs_set_mesh")
        self.n_cells = nx * ny * nz

    # ----------------------------------------------------------- time steps
    def next_dt(self) -> float:
        """IMC_State::get_next_dt (src/imc_state.h:112-125)."""
        d = self.deck
        nd = self.dt * d.t_mult if self.dt * d.t_mult < d.dt_max else d.dt_max
        if self.time + nd > d.t_stop:
            nd = d.t_stop - self.time
        return nd

    def finished(self) -> bool:
        return abs(self.time - self.deck.t_stop) < 1.0e-8

    def advance_time(self, nd: float) -> None:
        self.time += self.dt
        self.dt = nd
        self.step_no += 1

    def step(self, algorithm: Optional[int] = None, sync: bool = True) -> Optional[StepReport]:
        """One replicated IMC time step on the device (bgs_step), in the given
        algorithm or the context's (the deck's, or the tuner's choice)."""
        if algorithm is None:
            algorithm = self.algorithm
        nd = self.next_dt()
        if nd <= 0.0:  # past t_stop: keep stepping with the current dt
            nd = self.dt
        p = _lib.StepParams(self.step_no, algorithm, self.dt, nd)
        diag = _lib.TransportDiag()
        self._check(self.lib.bgs_step(self.ctx, C.byref(p), C.byref(diag) if sync else None), "bgs_step")
        rep = None
        if sync:
            rep = StepReport(self.step_no, self.dt, nd, diag.n_transported, diag.n_census, diag.n_segments,
                             diag.census_E, diag.exit_E, diag.absorbed_E, diag.post_mat_E, diag.device_flags)
        self.advance_time(nd)
        return rep

    def synchronize(self) -> None:
        self._check(self.lib.bgs_synchronize(self.ctx), "bgs_synchronize")

    # -------------------------------------------------------- staged calls
    def calculate_photon_energy(self, step: int, dt: float) -> Dict[str, float]:
        e = _lib.EnergyDiag()
        self._check(self.lib.bgs_calculate_photon_energy(self.ctx, step, dt, C.byref(e)),
                    "bgs_calculate_photon_energy")
        return {k: getattr(e, k) for k, _ in _lib.EnergyDiag._fields_}

    def source(self, step: int, dt: float) -> None:
        self._check(self.lib.bgs_source(self.ctx, step, dt), "bgs_source")

    def transport(self, next_dt: float, algorithm: Optional[int] = None) -> Dict[str, float]:
        algorithm = self.algorithm if algorithm is None else algorithm
        t = _lib.TransportDiag()
        self._check(self.lib.bgs_transport(self.ctx, next_dt, algorithm, C.byref(t)), "bgs_transport")
        return {k: getattr(t, k) for k, _ in _lib.TransportDiag._fields_}

    def update_temperature(self, dt: float) -> Dict[str, float]:
        t = _lib.TransportDiag()
        self._check(self.lib.bgs_update_temperature(self.ctx, dt, C.byref(t)), "bgs_update_temperature")
        return {k: getattr(t, k) for k, _ in _lib.TransportDiag._fields_}

    # ----------------------------------------------------------------- data
    def get_field(self, name: str) -> np.ndarray:
        out = np.empty(self.n_cells, np.float64)
        self._check(self.lib.bgs_get_cell_field(self.ctx, _lib.FIELDS[name], _lib.ptr(out)), "bgs_get_cell_field")
        return out

    def set_field(self, name: str, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, dtype=np.float64)
        if v.shape != (self.n_cells,):
            raise ValueError("one value per cell")
        self._check(self.lib.bgs_set_cell_field(self.ctx, _lib.FIELDS[name], _lib.ptr(v)), "bgs_set_cell_field")

    def bank_size(self) -> int:
        n = C.c_uint64()
        self._check(self.lib.bgs_bank_size(self.ctx, C.byref(n)), "bgs_bank_size")
        return int(n.value)

    def photons(self, offset: int = 0, count: Optional[int] = None) -> PhotonArrays:
        n = self.bank_size()
        count = n - offset if count is None else count
        out = PhotonArrays(count)
        s = out.struct()
        self._check(self.lib.bgs_get_photons(self.ctx, offset, count, C.byref(s)), "bgs_get_photons")
        return out

    def comb_census(self, max_census_photons: int, stream: int, counter: int = 0,
                    seed: Optional[int] = None) -> Tuple[int, int]:
        """comb_photons (census_functions.h:48-93) on the census the last
        transport left in the bank, with RNG(seed, stream) from ``counter``
        (the deck's seed by default).  Returns (census photons kept, the RNG
        counter after the comb's draws); the next step starts from the kept
        census."""
        seed = self.deck.seed if seed is None else seed
        ctr = C.c_uint64(counter)
        n = C.c_uint64()
        self._check(self.lib.bgs_comb_census(self.ctx, int(max_census_photons), seed, stream, C.byref(ctr),
                                             C.byref(n)), "bgs_comb_census")
        return int(n.value), int(ctr.value)

    def set_photons(self, ph: PhotonArrays) -> None:
        s = ph.struct()
        self._check(self.lib.bgs_set_photons(self.ctx, ph.n, C.byref(s)), "bgs_set_photons")

    def replicated_transport(self, ph: PhotonArrays, next_dt: float, algorithm: Optional[int] = None,
                             census: Optional[PhotonArrays] = None):
        """Drop-in replicated_transport on host buffers: ``ph`` is updated in
        place with the end states; returns (abs_E, track_E, census, census_E,
        exit_E) with the census in input order."""
        algorithm = self.algorithm if algorithm is None else algorithm
        abs_E = np.empty(self.n_cells)
        track_E = np.empty(self.n_cells)
        if census is None:
            census = PhotonArrays(ph.n)
        n_c = C.c_uint64()
        ce, ex = C.c_double(), C.c_double()
        s_in = ph.struct()
        s_out = census.struct()
        self._check(self.lib.bgs_replicated_transport(self.ctx, ph.n, C.byref(s_in), next_dt, algorithm,
                                                      _lib.ptr(abs_E), _lib.ptr(track_E), C.byref(s_out),
                                                      census.n, C.byref(n_c), C.byref(ce), C.byref(ex)),
                    "bgs_replicated_transport")
        return abs_E, track_E, census.subset(int(n_c.value)), ce.value, ex.value

    def set_option(self, name: str, value: float) -> None:
        """Scheduling option (see BGS_OPT_* in the header); results do not change."""
        self._check(self.lib.bgs_set_option(self.ctx, _lib.OPTIONS[name], float(value)), "bgs_set_option")

    def last_transport_ms(self):
        ms = C.c_float()
        k = C.c_uint32()
        self._check(self.lib.bgs_last_transport_ms(self.ctx, C.byref(ms), C.byref(k)), "bgs_last_transport_ms")
        return float(ms.value), int(k.value)

    def kernel_launches(self) -> int:
        return int(self.lib.bgs_kernel_launch_count(self.ctx))


# --------------------------------------------------------------- conversions
def records_to_arrays(rec: np.ndarray, pinned: bool = False) -> PhotonArrays:
    """Oracle / harness photon records (104-byte layout) to SoA arrays."""
    ph = PhotonArrays(len(rec), pinned=pinned)
    for k, axis in (("pos", "pos"), ("dir", "dir")):
        for i, a in enumerate("xyz"):
            ph[f"{axis}_{a}"][:] = rec[k][:, i]
    ph["E"][:] = rec["E"]
    ph["E0"][:] = rec["E0"]
    ph["life_dx"][:] = rec["life_dx"]
    ph["cell"][:] = rec["cell"]
    ph["group"][:] = rec["group"]
    ph["descriptor"][:] = rec["descriptor"].astype(np.uint8)
    ph["source_type"][:] = rec["source_type"].astype(np.uint8)
    ph["rng_stream"][:] = rec["stream"]
    ph["rng_counter"][:] = rec["counter"]
    return ph


def arrays_to_records(ph: PhotonArrays, dtype) -> np.ndarray:
    rec = np.zeros(ph.n, dtype)
    rec["pos"] = np.stack([ph["pos_x"], ph["pos_y"], ph["pos_z"]], 1)
    rec["dir"] = np.stack([ph["dir_x"], ph["dir_y"], ph["dir_z"]], 1)
    rec["E"] = ph["E"]
    rec["E0"] = ph["E0"]
    rec["life_dx"] = ph["life_dx"]
    rec["cell"] = ph["cell"]
    rec["group"] = ph["group"]
    rec["descriptor"] = ph["descriptor"]
    rec["source_type"] = ph["source_type"]
    rec["stream"] = ph["rng_stream"]
    rec["counter"] = ph["rng_counter"]
    return rec


class BatchIMC:
    """Independent problems stepped together through bgs_batch_step: one
    persistent transport launch over every problem's bank, the whole step
    recorded as a CUDA graph.  ``problems[i]`` is an ordinary ReplicatedIMC;
    read its results with its own calls."""

    def __init__(self, decks, device: int = 0, capacities=None):
        self.problems = [ReplicatedIMC(dk, device=device, capacity=None if capacities is None else capacities[i])
                         for i, dk in enumerate(decks)]
        self.lib = self.problems[0].lib
        n = len(self.problems)
        handles = (C.c_void_p * n)(*[p.ctx.value for p in self.problems])
        h = C.c_void_p()
        rc = self.lib.bgs_batch_create(C.byref(h), n, handles)
        if rc != 0:
            raise BransonError(rc, "bgs_batch_create")
        self.handle = h

    def _check(self, rc: int, what: str) -> None:
        if rc != 0:
            raise BransonError(rc, f"{what}: {self.lib.bgs_batch_last_error(self.handle).decode()}")

    def step(self, sync: bool = True):
        n = len(self.problems)
        params = (_lib.StepParams * n)()
        nds = []
        for i, p in enumerate(self.problems):
            nd = p.next_dt()
            if nd <= 0.0:
                nd = p.dt
            nds.append(nd)
            params[i] = _lib.StepParams(p.step_no, _lib.HISTORY, p.dt, nd)
        out = (_lib.TransportDiag * n)() if sync else None
        self._check(self.lib.bgs_batch_step(self.handle, params, out), "bgs_batch_step")
        reps = None
        if sync:
            reps = [StepReport(p.step_no, p.dt, nds[i], o.n_transported, o.n_census, o.n_segments, o.census_E,
                               o.exit_E, o.absorbed_E, o.post_mat_E, o.device_flags)
                    for i, (p, o) in enumerate(zip(self.problems, out))]
        for p, nd in zip(self.problems, nds):
            p.advance_time(nd)
        return reps

    def synchronize(self) -> None:
        self._check(self.lib.bgs_batch_synchronize(self.handle), "bgs_batch_synchronize")

    def set_option(self, name: str, value: float) -> None:
        self._check(self.lib.bgs_batch_set_option(self.handle, _lib.BATCH_OPTIONS[name], float(value)),
                    "bgs_batch_set_option")

    def last_transport_ms(self):
        ms = C.c_float()
        k = C.c_uint64()
        self._check(self.lib.bgs_batch_last_transport_ms(self.handle, C.byref(ms), C.byref(k)),
                    "bgs_batch_last_transport_ms")
        return float(ms.value), int(k.value)

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.bgs_batch_destroy(self.handle)
            self.handle = None
        for p in getattr(self, "problems", []):
            p.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
