"""Per-step cell fields written to a headless binary file, in place of the
SILO output of the upstream driver (write_silo, write_silo.h:31-270, called
every output_frequency steps when the deck sets write_silo,
replicated_driver.h:109-116).

The upstream file holds, per cell on the structured mesh, the material and
radiation temperatures, the region and the rank/transport/MPI timing; here
one file per output step holds T_e, T_r, the absorbed-energy tally and the
region index, plus the time, the step and the transport time, in a simple
little-endian layout:

    magic   8 bytes  b"BGSFLD01"
    header  uint32 nx, ny, nz, n_fields; uint32 step; uint32 reserved;
            float64 time, transport_s
    names   n_fields x 16 bytes, NUL padded ASCII
    data    n_fields x (nx*ny*nz) float64, cell g = i + nx*(j + ny*k)

The file name is output_<step>.bgsf, as upstream's output_<step>.silo.
"""
from __future__ import annotations

import os
import struct
from typing import Dict

import numpy as np

MAGIC = b"BGSFLD01"
FIELDS = ("T_e", "T_r", "abs_E", "region")


def write_fields(path: str, shape, step: int, time: float, fields: Dict[str, np.ndarray],
                 transport_s: float = 0.0) -> str:
    nx, ny, nz = (int(v) for v in shape)
    n = nx * ny * nz
    names = list(fields)
    with open(path, "wb") as fh:
        fh.write(MAGIC)
        fh.write(struct.pack("<6I2d", nx, ny, nz, len(names), int(step), 0, float(time), float(transport_s)))
        for name in names:
            b = name.encode("ascii")
            if len(b) > 16:
                raise ValueError(f"field name {name!r} longer than 16 bytes")
            fh.write(b.ljust(16, b"\0"))
        for name in names:
            a = np.ascontiguousarray(fields[name], dtype="<f8")
            if a.shape != (n,):
                raise ValueError(f"field {name!r}: {a.shape} values for {n} cells")
            fh.write(a.tobytes())
    return path


def read_fields(path: str) -> dict:
    with open(path, "rb") as fh:
        if fh.read(8) != MAGIC:
            raise ValueError(f"{path}: not a field file")
        nx, ny, nz, nf, step, _, time, transport_s = struct.unpack("<6I2d", fh.read(40))
        names = [fh.read(16).rstrip(b"\0").decode("ascii") for _ in range(nf)]
        n = nx * ny * nz
        data = {name: np.frombuffer(fh.read(8 * n), dtype="<f8").copy() for name in names}
    return {"shape": (nx, ny, nz), "step": step, "time": time, "transport_s": transport_s, "fields": data}


def dump_step(imc, out_dir: str, step: int, time: float, transport_s: float = 0.0) -> str:
    """Write the context's current fields (after a step's temperature update)."""
    os.makedirs(out_dir, exist_ok=True)
    f = {"T_e": imc.get_field("T_e"), "T_r": imc.get_field("T_r"), "abs_E": imc.get_field("abs_E"),
         "region": imc.deck.cell_regions().astype(np.float64)}
    return write_fields(os.path.join(out_dir, f"output_{step}.bgsf"), imc.deck.shape, step, time, f, transport_s)


def run(imc, out_dir: str = None, max_steps: int = None):
    """The replicated driver loop (replicated_driver.h:47-121): step until the
    deck's end time, writing the fields every output_frequency steps when the
    deck sets write_silo (and an output directory is given).  Returns the
    step reports."""
    reps = []
    d = imc.deck
    while not imc.finished() and (max_steps is None or len(reps) < max_steps):
        step = imc.step_no
        r = imc.step()
        reps.append(r)
        if out_dir and d.write_silo and d.output_frequency > 0 and step % d.output_frequency == 0:
            ms, _ = imc.last_transport_ms()
            dump_step(imc, out_dir, step, imc.time, ms * 1e-3)
    return reps
