"""Branson XML input decks: parse, write, and turn into a structured mesh.

The deck format and its defaults follow the upstream parser ``Input``
(src/input.h:43-490); the mesh numbering, node placement and boundary codes
follow ``Proto_Mesh`` (src/proto_mesh.h:48-220), where cell
``g = i + ngx*j + ngx*ngy*k`` and the cell nodes of a division are
``start + i*dx`` with ``dx = (end - start)/n`` (src/input.h:788-798), except that
the last cell of a non-final division ends exactly at the next division's
start (src/proto_mesh.h:130-145).  Every node is therefore one entry of a
per-axis plane array, which is how the device stores the geometry.

This module also generates the synthetic decks the benchmarks and tests use
(the Marshak wave, the 50^3 hot zone, the 60^3 multigroup hohlraum box, the
32^3 differentiation deck and the uneven batch ensemble).
"""
from __future__ import annotations

import dataclasses
import math
import xml.etree.ElementTree as ET
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# Constants::bc_type (src/constants.h:26)
REFLECT, VACUUM, ELEMENT, SOURCE, PROCESSOR = range(5)
BC_NAMES = {"REFLECT": REFLECT, "VACUUM": VACUUM, "SOURCE": SOURCE}
# Constants::dir_type order X-, X+, Y-, Y+, Z-, Z+ and the deck keys for each
# face (src/input.h:345-415)
FACE_KEYS = ("bc_left", "bc_right", "bc_down", "bc_up", "bc_bottom", "bc_top")
HISTORY, EVENT = 0, 1


class DeckError(ValueError):
    """Raised where the upstream parser prints an error and exits."""


@dataclasses.dataclass
class Region:
    """One <region> block (src/input.h:429-449, src/region.h)."""

    ID: int
    CV: float
    density: float
    opacA: float
    opacB: float
    opacC: float
    opacS: float
    T_e: float
    T_r: float

    def absorption_opacity(self, T: float) -> float:
        """Region::get_absorption_opacity (src/region.h:44-46)."""
        return self.opacA + self.opacB * math.pow(T, self.opacC)


@dataclasses.dataclass
class Division:
    start: float
    end: float
    n_cells: int

    @property
    def d(self) -> float:
        # Input::get_dx (src/input.h:788-790)
        return (self.end - self.start) / self.n_cells


@dataclasses.dataclass
class Deck:
    """Parsed deck: the fields the replicated IMC step reads."""

    t_start: float = 0.0
    t_stop: float = 1.0
    dt_start: float = 0.01
    t_mult: float = 1.0
    dt_max: float = 1.0
    photons: int = 10000
    seed: int = 777
    algorithm: int = HISTORY
    n_omp_threads: int = 1
    batch_size: int = 100000000
    use_gpu_transporter: bool = False
    write_silo: bool = False     # field output every output_frequency steps (input.h:143, :169-173)
    output_frequency: int = 1
    x_divisions: List[Division] = dataclasses.field(default_factory=list)
    y_divisions: List[Division] = dataclasses.field(default_factory=list)
    z_divisions: List[Division] = dataclasses.field(default_factory=list)
    # (x_div, y_div, z_div) -> region ID (src/input.h:328-338)
    region_map: Dict[Tuple[int, int, int], int] = dataclasses.field(default_factory=dict)
    bc: Tuple[int, int, int, int, int, int] = (VACUUM,) * 6
    T_source: float = 0.0
    regions: List[Region] = dataclasses.field(default_factory=list)
    n_groups: int = 1  # compile-time BRANSON_N_GROUPS upstream

    # ------------------------------------------------------------------ mesh
    @property
    def shape(self) -> Tuple[int, int, int]:
        return (sum(d.n_cells for d in self.x_divisions),
                sum(d.n_cells for d in self.y_divisions),
                sum(d.n_cells for d in self.z_divisions))

    @property
    def n_cells(self) -> int:
        nx, ny, nz = self.shape
        return nx * ny * nz

    def validate(self) -> None:
        """The checks the upstream parser exits on (src/input.h:111-126, :417-470)."""
        if not (self.x_divisions and self.y_divisions and self.z_divisions):
            raise DeckError("'spatial' section needs x, y and z divisions")
        if not self.regions:
            raise DeckError("No regions were specified")
        n_div = len(self.x_divisions) * len(self.y_divisions) * len(self.z_divisions)
        if n_div != len(self.region_map):
            raise DeckError("Number of total divisions must match the number of unique region maps")
        ids = {r.ID for r in self.regions}
        for key, rid in self.region_map.items():
            if rid not in ids:
                raise DeckError(f"region_map {key} names unknown region {rid}")
        for d in self.x_divisions + self.y_divisions + self.z_divisions:
            if d.n_cells <= 0:
                raise DeckError("a division needs at least one cell")
        if self.n_groups < 1:
            raise DeckError("n_groups must be positive")

    def planes(self) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Node planes per axis exactly as Proto_Mesh places them."""
        return tuple(_axis_planes(divs) for divs in
                     (self.x_divisions, self.y_divisions, self.z_divisions))

    def cell_regions(self) -> np.ndarray:
        """Region index (position in ``regions``) of every cell, cell order."""
        index_of = {r.ID: i for i, r in enumerate(self.regions)}
        rx = np.concatenate([np.full(d.n_cells, i, np.int64) for i, d in enumerate(self.x_divisions)])
        ry = np.concatenate([np.full(d.n_cells, i, np.int64) for i, d in enumerate(self.y_divisions)])
        rz = np.concatenate([np.full(d.n_cells, i, np.int64) for i, d in enumerate(self.z_divisions)])
        nxd, nyd = len(self.x_divisions), len(self.y_divisions)
        lut = np.zeros(nxd * nyd * len(self.z_divisions), np.uint32)
        for (xd, yd, zd), rid in self.region_map.items():
            lut[xd + nxd * (yd + nyd * zd)] = index_of[rid]
        div_id = rx[None, None, :] + nxd * (ry[None, :, None] + nyd * rz[:, None, None])
        return np.ascontiguousarray(lut[div_id].reshape(-1), dtype=np.uint32)

    def region_table(self) -> np.ndarray:
        """Regions as rows (cV, rho, A, B, C, S, T_e, T_r) in deck order."""
        return np.array([[r.CV, r.density, r.opacA, r.opacB, r.opacC, r.opacS, r.T_e, r.T_r]
                         for r in self.regions], dtype=np.float64).reshape(-1, 8)

    # -------------------------------------------------------------- writing
    def to_xml(self) -> str:
        """Write the deck in the upstream format (readable by ``Input``)."""
        algo = "EVENT" if self.algorithm == EVENT else "HISTORY"
        lines = ["<prototype>", "  <common>"]
        for key, val in (("t_start", self.t_start), ("t_stop", self.t_stop),
                         ("dt_start", self.dt_start), ("t_mult", self.t_mult),
                         ("dt_max", self.dt_max)):
            lines.append(f"    <{key}>{val!r}</{key}>")
        lines += [f"    <photons>{int(self.photons)}</photons>",
                  f"    <seed>{int(self.seed)}</seed>",
                  f"    <use_gpu_transporter>{'TRUE' if self.use_gpu_transporter else 'FALSE'}</use_gpu_transporter>",
                  "    <use_combing>FALSE</use_combing>",
                  "    <dd_transport_type>REPLICATED</dd_transport_type>",
                  "    <particle_storage>AOS</particle_storage>",
                  f"    <particle_algorithm>{algo}</particle_algorithm>",
                  f"    <n_omp_threads>{int(self.n_omp_threads)}</n_omp_threads>",
                  f"    <batch_size>{int(self.batch_size)}</batch_size>",
                  f"    <output_frequency>{int(self.output_frequency)}</output_frequency>",
                  f"    <write_silo>{'TRUE' if self.write_silo else 'FALSE'}</write_silo>",
                  "  </common>",
                  "  <debug_options><print_verbose>FALSE</print_verbose>"
                  "<print_mesh_info>FALSE</print_mesh_info></debug_options>",
                  "  <spatial>"]
        for axis, divs in (("x", self.x_divisions), ("y", self.y_divisions), ("z", self.z_divisions)):
            for d in divs:
                lines.append(f"    <{axis}_division><{axis}_start>{d.start!r}</{axis}_start>"
                             f"<{axis}_end>{d.end!r}</{axis}_end>"
                             f"<n_{axis}_cells>{int(d.n_cells)}</n_{axis}_cells></{axis}_division>")
        for (xd, yd, zd), rid in sorted(self.region_map.items(), key=lambda kv: (kv[0][2], kv[0][1], kv[0][0])):
            lines.append(f"    <region_map><x_div_ID>{xd}</x_div_ID><y_div_ID>{yd}</y_div_ID>"
                         f"<z_div_ID>{zd}</z_div_ID><region_ID>{rid}</region_ID></region_map>")
        lines += ["  </spatial>", "  <boundary>"]
        inv = {v: k for k, v in BC_NAMES.items()}
        for key, code in zip(FACE_KEYS, self.bc):
            lines.append(f"    <{key}>{inv[code]}</{key}>")
        lines.append(f"    <T_source>{self.T_source!r}</T_source>")
        lines += ["  </boundary>", "  <regions>"]
        for r in self.regions:
            lines.append(f"    <region><ID>{r.ID}</ID><density>{r.density!r}</density><CV>{r.CV!r}</CV>"
                         f"<opacA>{r.opacA!r}</opacA><opacB>{r.opacB!r}</opacB><opacC>{r.opacC!r}</opacC>"
                         f"<opacS>{r.opacS!r}</opacS><initial_T_e>{r.T_e!r}</initial_T_e>"
                         f"<initial_T_r>{r.T_r!r}</initial_T_r></region>")
        lines += ["  </regions>", "</prototype>", ""]
        return "\n".join(lines)


def _axis_planes(divs: Sequence[Division]) -> np.ndarray:
    """Plane coordinates along one axis (src/proto_mesh.h:106-148)."""
    out: List[float] = []
    for di, d in enumerate(divs):
        dx = d.d
        for i in range(d.n_cells):
            out.append(d.start + i * dx)
        if di == len(divs) - 1:
            out.append(d.start + d.n_cells * dx)
    return np.array(out, dtype=np.float64)


# ---------------------------------------------------------------- parsing
def _text(node: Optional[ET.Element], key: str) -> str:
    if node is None:
        return ""
    child = node.find(key)
    return (child.text or "").strip() if child is not None else ""


def _num(node, key, cast=float, default=0):
    t = _text(node, key)
    if t == "":
        return cast(default)
    return cast(float(t)) if cast is int else cast(t)


def parse_xml(text: str, n_groups: int = 1) -> Deck:
    """Parse deck text the way Input does (src/input.h:89-490).

    Unknown keys are ignored; a malformed boundary block or missing section
    raises ``DeckError`` where the upstream parser exits.
    """
    try:
        root = ET.fromstring(text)
    except ET.ParseError as exc:
        raise DeckError(f"Improperly formatted xml file: {exc}") from exc
    common = root.find("common")
    spatial = root.find("spatial")
    boundary = root.find("boundary")
    regions = root.find("regions")
    for node, name in ((common, "common"), (spatial, "spatial"), (boundary, "boundary"), (regions, "regions")):
        if node is None:
            raise DeckError(f"'{name}' section not found!")
    deck = Deck(n_groups=n_groups)
    deck.t_stop = _num(common, "t_stop")
    deck.dt_start = _num(common, "dt_start")
    deck.t_start = _num(common, "t_start")
    deck.t_mult = _num(common, "t_mult")
    deck.dt_max = _num(common, "dt_max")
    deck.photons = int(_text(common, "photons") or 0)
    deck.seed = int(_text(common, "seed") or 0) & 0xFFFFFFFF
    deck.use_gpu_transporter = _text(common, "use_gpu_transporter") == "TRUE"
    deck.write_silo = _text(common, "write_silo") == "TRUE"
    t = _text(common, "output_frequency")
    deck.output_frequency = int(t) if t else 0
    deck.algorithm = EVENT if _text(common, "particle_algorithm") == "EVENT" else HISTORY
    t = _text(common, "n_omp_threads")
    deck.n_omp_threads = int(t) if t else 1
    t = _text(common, "batch_size")
    deck.batch_size = int(t) if t else 10000
    if deck.algorithm == HISTORY:  # replicated + history (src/input.h:488-490)
        deck.batch_size = 100000000
    for child in spatial:
        if child.tag in ("x_division", "y_division", "z_division"):
            a = child.tag[0]
            div = Division(_num(child, f"{a}_start"), _num(child, f"{a}_end"),
                           int(_text(child, f"n_{a}_cells") or 0))
            getattr(deck, f"{a}_divisions").append(div)
        elif child.tag == "region_map":
            key = (int(_text(child, "x_div_ID") or 0), int(_text(child, "y_div_ID") or 0),
                   int(_text(child, "z_div_ID") or 0))
            deck.region_map[key] = int(_text(child, "region_ID") or 0)
    bcs = []
    source_on = False
    for key in FACE_KEYS:
        v = _text(boundary, key)
        if v not in BC_NAMES:
            raise DeckError("Boundary type not reconginzed")
        source_on |= v == "SOURCE"
        bcs.append(BC_NAMES[v])
    deck.bc = tuple(bcs)
    deck.T_source = _num(boundary, "T_source") if source_on else 0.0
    for child in regions:
        if child.tag != "region":
            continue
        deck.regions.append(Region(
            ID=int(_text(child, "ID") or 0), CV=_num(child, "CV"), density=_num(child, "density"),
            opacA=_num(child, "opacA"), opacB=_num(child, "opacB"), opacC=_num(child, "opacC"),
            opacS=_num(child, "opacS"), T_e=_num(child, "initial_T_e"), T_r=_num(child, "initial_T_r")))
    deck.validate()
    return deck


def load(path: str, n_groups: int = 1) -> Deck:
    with open(path, "r", encoding="utf-8") as fh:
        return parse_xml(fh.read(), n_groups=n_groups)


# ------------------------------------------------------ synthetic decks
def _uniform_axis(lo: float, hi: float, n: int) -> List[Division]:
    return [Division(lo, hi, n)]


def marshak_wave(n_cells: int = 100, photons: int = 1_000_000, n_steps: int = 50,
                 seed: int = 777) -> Deck:
    """Gray Marshak wave: 100x1x1 cells over 1 cm, reflecting y/z, 1 keV
    source on x-, vacuum on x+, sigma_a = 100/cm, cV = 0.1, T0 = 0.01 keV,
    dt = 0.001 sh."""
    dt = 0.001
    return Deck(t_start=0.0, t_stop=dt * n_steps, dt_start=dt, t_mult=1.0, dt_max=1.0,
                photons=photons, seed=seed,
                x_divisions=_uniform_axis(0.0, 1.0, n_cells),
                y_divisions=_uniform_axis(0.0, 1.0, 1), z_divisions=_uniform_axis(0.0, 1.0, 1),
                region_map={(0, 0, 0): 1},
                bc=(SOURCE, VACUUM, REFLECT, REFLECT, REFLECT, REFLECT), T_source=1.0,
                regions=[Region(1, 0.1, 1.0, 100.0, 0.0, 0.0, 0.0, 0.01, 0.01)])


def hot_zone(n_per_axis: int = 50, photons: int = 10_000_000, n_steps: int = 10,
             seed: int = 777) -> Deck:
    """Gray 3D hot zone: [0,1]^3 cut at 0.4/0.6 on every axis (20/10/20 cells
    for the 50^3 deck), central block at 1 keV, surround at 0.05 keV,
    sigma_a = 10*T^-3, rho = 1, cV = 0.1, vacuum boundaries, dt = 0.01 sh."""
    if n_per_axis % 5:
        raise DeckError("hot zone side must be a multiple of 5")
    outer, inner = 2 * n_per_axis // 5, n_per_axis // 5
    divs = [Division(0.0, 0.4, outer), Division(0.4, 0.6, inner), Division(0.6, 1.0, outer)]
    rmap = {}
    for zd in range(3):
        for yd in range(3):
            for xd in range(3):
                rmap[(xd, yd, zd)] = 2 if (xd, yd, zd) == (1, 1, 1) else 1
    dt = 0.01
    return Deck(t_start=0.0, t_stop=dt * n_steps, dt_start=dt, t_mult=1.0, dt_max=1.0,
                photons=photons, seed=seed,
                x_divisions=list(divs), y_divisions=list(divs), z_divisions=list(divs),
                region_map=rmap, bc=(VACUUM,) * 6, T_source=0.0,
                regions=[Region(1, 0.1, 1.0, 0.0, 10.0, -3.0, 0.0, 0.05, 0.05),
                         Region(2, 0.1, 1.0, 0.0, 10.0, -3.0, 0.0, 1.0, 1.0)])


def hohlraum(n_per_axis: int = 60, photons: int = 50_000_000, n_steps: int = 5,
             n_groups: int = 30, seed: int = 777) -> Deck:
    """Multigroup hohlraum-like box: 0.01 cm cells, a 3-cell-thick wall shell
    (sigma_a = 1000/cm, rho = 10) around a low-density fill (sigma_a = 0.1/cm,
    rho = 0.01), 0.3 keV source on x-, vacuum elsewhere, dt = 0.005 sh,
    gray-equal opacity in every group."""
    h = 0.01
    wall = 3
    inner = n_per_axis - 2 * wall
    if inner <= 0:
        raise DeckError("hohlraum side must exceed the wall thickness")
    divs = [Division(0.0, wall * h, wall), Division(wall * h, (wall + inner) * h, inner),
            Division((wall + inner) * h, n_per_axis * h, wall)]
    rmap = {}
    for zd in range(3):
        for yd in range(3):
            for xd in range(3):
                rmap[(xd, yd, zd)] = 2 if (xd, yd, zd) == (1, 1, 1) else 1
    dt = 0.005
    return Deck(t_start=0.0, t_stop=dt * n_steps, dt_start=dt, t_mult=1.0, dt_max=1.0,
                photons=photons, seed=seed,
                x_divisions=list(divs), y_divisions=list(divs), z_divisions=list(divs),
                region_map=rmap, bc=(SOURCE, VACUUM, VACUUM, VACUUM, VACUUM, VACUUM), T_source=0.3,
                regions=[Region(1, 0.1, 10.0, 1000.0, 0.0, 0.0, 0.0, 0.001, 0.001),
                         Region(2, 0.1, 0.01, 0.1, 0.0, 0.0, 0.0, 0.001, 0.001)],
                n_groups=n_groups)


def random_opacity_cube(n_per_axis: int = 32, photons: int = 10_000_000, seed: int = 777,
                        sigma_median: float = 20.0, sigma_log_sd: float = 0.5) -> Deck:
    """Differentiation deck: every cell its own region with sigma_a drawn
    lognormal(ln 20, 0.5) from the seed, T0 = 0.1 keV, 1 keV source on x-,
    vacuum elsewhere, one step of dt = 0.01 sh."""
    rng = np.random.default_rng(seed)
    n = n_per_axis
    sig = np.exp(rng.normal(math.log(sigma_median), sigma_log_sd, size=n ** 3))
    divs = [Division(i / n, (i + 1) / n, 1) for i in range(n)]
    rmap = {}
    regions = []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                c = i + n * (j + n * k)
                rmap[(i, j, k)] = c + 1
                regions.append(Region(c + 1, 0.1, 1.0, float(sig[c]), 0.0, 0.0, 0.0, 0.1, 0.1))
    dt = 0.01
    return Deck(t_start=0.0, t_stop=dt, dt_start=dt, t_mult=1.0, dt_max=1.0,
                photons=photons, seed=seed, x_divisions=list(divs), y_divisions=list(divs),
                z_divisions=list(divs), region_map=rmap,
                bc=(SOURCE, VACUUM, VACUUM, VACUUM, VACUUM, VACUUM), T_source=1.0, regions=regions)


def batch_ensemble(n_problems: int = 256, master_seed: int = 777, side_range=(8, 64),
                   photon_median: float = 1e5, photon_range=(10_000, 1_000_000)) -> List[Deck]:
    """Uneven ensemble: cubic side ~ U{8..64} on [0,1]^3, photons ~ lognormal
    (median 1e5) clipped to [1e4, 1e6], sigma_a ~ U(1,200), source T ~
    U(0.2,1) on x-, T0 = 0.01 keV, cV = 0.1, rho = 1, one step of 0.005 sh;
    per-problem seeds derive from the master seed."""
    rng = np.random.default_rng(master_seed)
    decks = []
    dt = 0.005
    for p in range(n_problems):
        side = int(rng.integers(side_range[0], side_range[1] + 1))
        photons = int(np.clip(round(float(np.exp(rng.normal(math.log(photon_median), 1.0)))),
                              photon_range[0], photon_range[1]))
        sigma = float(rng.uniform(1.0, 200.0))
        t_src = float(rng.uniform(0.2, 1.0))
        seed = int(rng.integers(1, 2 ** 31 - 1))
        decks.append(Deck(t_start=0.0, t_stop=dt, dt_start=dt, t_mult=1.0, dt_max=1.0,
                          photons=photons, seed=seed,
                          x_divisions=_uniform_axis(0.0, 1.0, side),
                          y_divisions=_uniform_axis(0.0, 1.0, side),
                          z_divisions=_uniform_axis(0.0, 1.0, side),
                          region_map={(0, 0, 0): 1},
                          bc=(SOURCE, VACUUM, VACUUM, VACUUM, VACUUM, VACUUM), T_source=t_src,
                          regions=[Region(1, 0.1, 1.0, sigma, 0.0, 0.0, 0.0, 0.01, 0.01)]))
    return decks
